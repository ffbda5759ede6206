"""C-ABI checks that need no GPU: the library builds and loads, exports every
function include/yelmo_gpu.h declares, and its host-side parameter logic
agrees with the Python mirror and the oracle."""
import ctypes as C
import os
import re

import pytest

from yelmo_gb300 import abi, gpu
from yelmo_gb300.params import YdynParams, parse_lis_opt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "yelmo_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ygpu_\w+)\s*\(", txt)))


def test_library_exports_every_declared_function():
    L = gpu.lib()
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    for n in gpu.EXPORTS:
        assert n in names


def test_version_and_boundary_codes():
    L = gpu.lib()
    assert b"sm_103a" in L.ygpu_version()
    for name, code in abi.BOUNDARY_CODES.items():
        assert L.ygpu_boundary_code(name.encode()) == code
    assert L.ygpu_boundary_code(b"nonsense") == -1


@pytest.mark.parametrize("opt", [
    "-i cg -p jacobi -maxiter 200 -tol 1.0e-2 -initx_zeros false",
    "-i minres -p jacobi -maxiter 100 -tol 1.0e-2 -initx_zeros false",
    "-i bicgstab -p ilu -maxiter 1000 -tol 1.0e-8 -initx_zeros true",
    "-i cg -p none -maxiter 5 -tol 1e-12",
])
def test_lis_option_parsing_matches_python(opt):
    L = gpu.lib()
    p = abi.DynPar()
    L.ygpu_dyn_par_defaults(C.byref(p))
    assert L.ygpu_parse_lis_opt(opt.encode(), C.byref(p)) == 0
    for k, v in parse_lis_opt(opt).items():
        assert getattr(p, k) == v, k


def test_bad_lis_option_rejected():
    L = gpu.lib()
    p = abi.DynPar()
    assert L.ygpu_parse_lis_opt(b"-i gmres -p jacobi", C.byref(p)) == abi.ERR_BAD_ARG
    assert L.ygpu_parse_lis_opt(b"-i cg -p", C.byref(p)) == abi.ERR_BAD_ARG


def test_defaults_match_namelist():
    L = gpu.lib()
    p = abi.DynPar()
    L.ygpu_dyn_par_defaults(C.byref(p))
    q = YdynParams().to_c()
    for k, _ in abi.DynPar._fields_:
        if k in ("no_slip",):
            continue
        assert getattr(p, k) == getattr(q, k), k


def test_struct_builders_reject_misshaped_arrays():
    """abi.jvel / abi.uz3d / abi.dyn_diag check every array's shape against the
    grid before any pointer reaches the library."""
    import numpy as np
    nx, ny, nz = 6, 5, 4
    z = np.linspace(0.0, 1.0, nz)
    base = {"H_ice": np.zeros((nx, ny), order="F"), "f_ice": np.ones((nx, ny), order="F"),
            "zeta_aa": z, "zeta_ac": np.linspace(0.0, 1.0, nz + 1)}
    good = dict(base, ux=np.zeros((nx, ny, nz), order="F"))
    abi.jvel(good, 1e3, 1e3)
    abi.uz3d(good, 1e3, 1e3)
    with pytest.raises(ValueError):
        abi.jvel(dict(base, ux=np.zeros((nx, ny, nz + 1), order="F")), 1e3, 1e3)
    with pytest.raises(ValueError):
        abi.uz3d(dict(base, uz=np.zeros((nx, ny, nz), order="F")), 1e3, 1e3)
    with pytest.raises(ValueError):
        abi.dyn_diag({"ux_bar": np.zeros((nx, ny + 1), order="F")}, nx, ny, nz, 1e3, 1e3)


@pytest.mark.parametrize("solver,opt,want", [
    ("energy", "-i cg -p jacobi", (abi.LIN_CG, abi.PRE_JACOBI)),
    ("energy", "-i cg -p ilu", (abi.LIN_CG, abi.PRE_TILE_BLOCK)),
    ("energy", "-i minres -p jacobi", (abi.LIN_CG, abi.PRE_JACOBI)),
    ("energy", "-i bicgstab -p ilu", (abi.LIN_BICGSTAB, abi.PRE_JACOBI)),
    ("residual", "-i bicgstab -p ilu", (abi.LIN_BICGSTAB, abi.PRE_ILU0)),
    ("residual", "-i minres -p jacobi", (abi.LIN_BICGSTAB, abi.PRE_JACOBI)),
    ("residual", "-i cg -p none", (abi.LIN_BICGSTAB, abi.PRE_NONE)),
])
def test_method_run_is_reported(solver, opt, want):
    """ygpu_lin_method_run names the Krylov method and preconditioner the GPU runs
    for a request (the values the solve's stats carry), so a substitution is visible."""
    L = gpu.lib()
    p = YdynParams(ssa_solver=solver, ssa_lis_opt_energy=opt, ssa_lis_opt_residual=opt).to_c()
    s, pc = C.c_int(-1), C.c_int(-1)
    L.ygpu_lin_method_run(C.byref(p), C.byref(s), C.byref(pc))
    assert (s.value, pc.value) == want


def test_new_entries_refuse_bad_arguments_before_any_device_call():
    """Argument checks of the background-slope prologue, its device form, the
    device masks and the member step count run on the host and refuse without
    touching CUDA."""
    import numpy as np
    L = gpu.lib()
    n = 8
    arrs = [np.zeros((n, n), order="F") for _ in range(16)]
    arrs[9] = np.zeros((n, n), dtype=np.int32, order="F")          # mask_frnt
    ptrs = [a.ctypes.data_as(C.POINTER(C.c_int if a.dtype == np.int32 else C.c_double)) for a in arrs]
    # a non-finite slope
    assert L.ygpu_calc_dyn_inputs_bg(*ptrs, 1e3, 0.5, 2e5, 910.0, 1028.0, 9.81, float("nan"), 0.0,
                                     0, n, n) == abi.ERR_BAD_ARG
    # a grid below 3 x 3
    assert L.ygpu_calc_dyn_inputs_bg(*ptrs, 1e3, 0.5, 2e5, 910.0, 1028.0, 9.81, 0.0, 0.0, 0, 2, n) == abi.ERR_BAD_ARG
    vp = [C.c_void_p(a.ctypes.data) for a in arrs]
    # the device forms need a context
    assert L.ygpu_calc_dyn_inputs_bg_device(None, *vp, 1e3, 0.5, 2e5, 910.0, 1028.0, 9.81, 0.0, 0.0,
                                            0, n, n) == abi.ERR_BAD_ARG
    assert L.ygpu_set_ssa_masks_device(None, vp[0], vp[1], vp[9], vp[2], vp[3], 2, 0, n, n) == abi.ERR_BAD_ARG
    steps = C.c_ulonglong(0)
    assert L.ygpu_server_member_steps(None, 0, C.byref(steps)) == abi.ERR_BAD_ARG
    assert L.ygpu_server_set_member_steps(None, 0, 3) == abi.ERR_BAD_ARG
