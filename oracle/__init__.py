"""Python binding of the CPU oracle (oracle/yelmo_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the yelmo_gb300 package. The oracle is
an FP64 restatement of the reference solve; see yelmo_oracle.h for what pins it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from yelmo_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
FAST_LIB_PATH = os.path.join(HERE, "_build", "liboracle_fast.so")
_libs = {}
_use_fast = False


def build(force: bool = False) -> str:
    """Compile liboracle.so (the oracle the tests compare with) and liboracle_fast.so (the timed CPU
    baseline) with the Makefile beside this file."""
    src = os.path.getmtime(os.path.join(HERE, "yelmo_oracle.c"))
    if force or any(not os.path.exists(p) or os.path.getmtime(p) < src for p in (LIB_PATH, FAST_LIB_PATH)):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def timing_flags() -> str:
    """Compiler flags of the timed build (liboracle_fast.so) on this host."""
    r = subprocess.run(["make", "-s", "-C", HERE, "flags"], capture_output=True, text=True)
    return r.stdout.strip()


class timing_build:
    """Context manager: the oracle calls inside it run liboracle_fast.so (-O3,
    tuned for the host CPU, FMA contraction), the build the CPU baseline times;
    outside it they run the reference build (liboracle.so)."""

    def __enter__(self):
        global _use_fast
        self._prev = _use_fast
        _use_fast = True
        return self

    def __exit__(self, *exc):
        global _use_fast
        _use_fast = self._prev
        return False


def lib():
    path = FAST_LIB_PATH if _use_fast else LIB_PATH
    if path not in _libs:
        build()
        L = C.CDLL(path)
        abi.declare_velocity(L.orc_calc_velocity_ssa, abi.SSA_ARGS)
        abi.declare_velocity(L.orc_calc_velocity_diva, abi.DIVA_ARGS)
        abi.declare_velocity(L.orc_calc_velocity_diva_hook, abi.DIVA_ARGS)
        L.orc_calc_velocity_diva_hook.argtypes = L.orc_calc_velocity_diva_hook.argtypes + [abi.NEFF_HOOK, C.c_void_p]
        abi.declare_inputs(L.orc_calc_dyn_inputs)
        abi.declare_inputs(L.orc_calc_dyn_inputs_bg, bg=True)
        abi.declare_masks(L.orc_set_ssa_masks)
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.orc_assemble_csr.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int] + \
            [dp] * 4 + [dp, ip, ip] + [dp] * 8 + [C.c_int, ip, ip, dp, dp, dp, ip]
        L.orc_assemble_csr.restype = C.c_int
        L.orc_linear_solve.argtypes = [C.c_int, ip, ip, dp, dp, dp, C.c_int, C.c_int, C.c_int,
                                       C.c_double, C.c_int, ip, dp]
        L.orc_linear_solve.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_calc_dyn_diagnostics.argtypes = [C.POINTER(abi.DynDiag), C.c_int]
        L.orc_calc_dyn_diagnostics.restype = C.c_int
        L.orc_calc_advec2D_impl_lis.argtypes = [dp] * 5 + [ip, dp, C.c_double, C.c_double, C.c_double,
                                                           C.c_int, C.c_int, C.c_int, ip, ip]
        L.orc_calc_advec2D_impl_lis.restype = C.c_int
        L.orc_calc_gradient_column_ac.argtypes = [dp] * 5 + [ip, C.c_int, C.c_int, C.c_int]
        L.orc_calc_jacobian_vel_3D.argtypes = [C.POINTER(abi.JVel), C.c_int, C.c_int]
        L.orc_calc_uz_3D.argtypes = [C.POINTER(abi.Uz3D), C.c_int, C.c_int]
        L.orc_calc_strain_rate_tensor.argtypes = [C.POINTER(abi.Strain3D), C.c_int]
        _libs[path] = L
    return _libs[path]


def set_threads(n: int):
    lib().orc_set_threads(int(n))


def calc_dyn_inputs(inst) -> dict:
    """Oracle restatement of the fields calc_ydyn builds before the solve."""
    d = inst.input_buffers()
    p = inst.par
    bg = tuple(getattr(inst, "slope_bg", (0.0, 0.0)))
    fn = lib().orc_calc_dyn_inputs if bg == (0.0, 0.0) else lib().orc_calc_dyn_inputs_bg
    st = abi.call_inputs(fn, d, inst.dx, p.grad_lim, p.taud_lim, p.rho_ice, p.rho_sw, p.g,
                         abi.BOUNDARY_CODES[p.boundaries], None if bg == (0.0, 0.0) else bg)
    assert st == 0
    return d


def set_ssa_masks(mask_frnt, f_ice, f_grnd, lateral_bc: str, boundaries: str):
    nx, ny = f_ice.shape
    mx = np.zeros((nx, ny), dtype=np.int32, order="F")
    my = np.zeros((nx, ny), dtype=np.int32, order="F")
    lib().orc_set_ssa_masks(abi.ptr(mx, "i"), abi.ptr(my, "i"), abi.ptr(mask_frnt, "i"),
                            abi.ptr(f_ice, "d"), abi.ptr(f_grnd, "d"),
                            abi.LATBC_CODES[lateral_bc], abi.BOUNDARY_CODES[boundaries], nx, ny)
    return mx, my


def prepare(inst) -> dict:
    """Cold-start state of one solve with the oracle's prologue and masks."""
    inputs = calc_dyn_inputs(inst)
    f = inst.state(inputs)
    f["ssa_mask_acx"], f["ssa_mask_acy"] = set_ssa_masks(
        inputs["mask_frnt"], inputs["f_ice"], inputs["f_grnd"], inst.par.ssa_lat_bc, inst.par.boundaries)
    return f


def calc_velocity(fields: dict, inst, par=None, neff_hook=None) -> dict:
    """Run orc_calc_velocity_ssa / _diva on ``fields`` (updated in place);
    neff_hook(c_bed, ux_b, uy_b) as in yelmo_gb300.gpu.calc_velocity (DIVA)."""
    par = par or inst.par
    cpar = par.to_c()
    if par.solver == "ssa":
        return abi.call_velocity(lib().orc_calc_velocity_ssa, abi.SSA_ARGS, fields, inst.dx, inst.dx,
                                 inst.n_glen, cpar)
    if neff_hook:
        cb = abi.neff_hook(neff_hook)
        return abi.call_velocity(lib().orc_calc_velocity_diva_hook, abi.DIVA_ARGS, fields, inst.dx, inst.dx,
                                 inst.n_glen, cpar, extra=(cb, None))
    return abi.call_velocity(lib().orc_calc_velocity_diva, abi.DIVA_ARGS, fields, inst.dx, inst.dx,
                             inst.n_glen, cpar)


def assemble_csr(energy: bool, f: dict, dx: float, dy: float, boundaries: str, N_aa=None,
                 beta_acx=None, beta_acy=None, ux=None, uy=None):
    """CSR (0-based) of the residual or energy assembler on the given fields."""
    nx, ny = f["H_ice"].shape
    n = 2 * nx * ny
    cap = 64 * n
    ptr_ = np.zeros(n + 1, dtype=np.int32)
    idx = np.zeros(cap, dtype=np.int32)
    val = np.zeros(cap)
    b = np.zeros(n)
    x = np.zeros(n)
    cf = np.zeros(n, dtype=np.int32)
    g = lambda k: abi.ptr(f[k], "d")
    nnz = lib().orc_assemble_csr(
        int(energy), nx, ny, dx, dy, abi.BOUNDARY_CODES[boundaries],
        abi.ptr(ux if ux is not None else f["ux"], "d"), abi.ptr(uy if uy is not None else f["uy"], "d"),
        abi.ptr(beta_acx if beta_acx is not None else f["beta_acx"], "d"),
        abi.ptr(beta_acy if beta_acy is not None else f["beta_acy"], "d"),
        abi.ptr(N_aa if N_aa is not None else f["N_aa"], "d"),
        abi.ptr(f["ssa_mask_acx"], "i"), abi.ptr(f["ssa_mask_acy"], "i"),
        g("H_ice"), g("f_ice"), g("z_bed"), g("z_sl"), g("taud_acx"), g("taud_acy"),
        g("taul_int_acx"), g("taul_int_acy"), cap, abi.ptr(ptr_, "i"), abi.ptr(idx, "i"),
        abi.ptr(val, "d"), abi.ptr(b, "d"), abi.ptr(x, "d"), abi.ptr(cf, "i"))
    if nnz < 0:
        raise RuntimeError(f"orc_assemble_csr failed ({nnz})")
    return ptr_, idx[:nnz].copy(), val[:nnz].copy(), b, x, cf


def calc_dyn_diagnostics(arrays: dict, dx: float, dy: float, boundaries: str) -> dict:
    """orc_calc_dyn_diagnostics on the arrays of yelmo_gb300.gpu.diagnostics_arrays (filled in place)."""
    nx, ny = arrays["H_ice"].shape
    nz = arrays["zeta_aa"].shape[0] if "zeta_aa" in arrays else (arrays["ux"].shape[2] if "ux" in arrays else 1)
    D = abi.dyn_diag(arrays, nx, ny, nz, dx, dy)
    st = lib().orc_calc_dyn_diagnostics(C.byref(D), abi.BOUNDARY_CODES[boundaries])
    if st != 0:
        raise RuntimeError(f"orc_calc_dyn_diagnostics failed ({st})")
    return arrays


def calc_advec2D_impl_lis(var, ux, uy, var_dot, mask_ice, var_ref, dx, dy, dt, boundaries: str):
    """orc_calc_advec2D_impl_lis: (dvdt, lin_iter, lin_status); boundaries as for
    yelmo_gb300.gpu.calc_advec2D_impl_lis (\"mask\" has its own advection borders)."""
    nx, ny = var.shape
    dvdt = np.zeros((nx, ny), order="F")
    it, st = C.c_int(0), C.c_int(0)
    code = abi.ADV_BOUNDARY_CODES[boundaries]
    r = lib().orc_calc_advec2D_impl_lis(abi.ptr(dvdt, "d"), abi.ptr(var, "d"), abi.ptr(ux, "d"), abi.ptr(uy, "d"),
                                        abi.ptr(var_dot, "d"), abi.ptr(mask_ice, "i"), abi.ptr(var_ref, "d"),
                                        dx, dy, dt, code, nx, ny, C.byref(it), C.byref(st))
    if r < 0:
        raise RuntimeError(f"orc_calc_advec2D_impl_lis failed ({r})")
    return dvdt, it.value, st.value


def calc_gradient_column_ac(dvdx, dvdy, f_ice, mask_ocn, boundaries: str):
    """orc_calc_gradient_column_ac: (dvdx_c, dvdy_c)."""
    nx, ny = f_ice.shape
    gx = np.zeros((nx, ny), order="F")
    gy = np.zeros((nx, ny), order="F")
    ocn = np.asfortranarray(mask_ocn, dtype=np.int32)
    st = lib().orc_calc_gradient_column_ac(abi.ptr(gx, "d"), abi.ptr(gy, "d"), abi.ptr(dvdx, "d"),
                                           abi.ptr(dvdy, "d"), abi.ptr(f_ice, "d"), abi.ptr(ocn, "i"),
                                           abi.BOUNDARY_CODES[boundaries], nx, ny)
    if st != 0:
        raise RuntimeError(f"orc_calc_gradient_column_ac failed ({st})")
    return gx, gy


def calc_jacobian_vel_3D(arrays: dict, dx: float, dy: float, boundaries: str, terms: int = 3) -> dict:
    """orc_calc_jacobian_vel_3D on the arrays of yelmo_gb300.gpu.jacobian_arrays (filled in place)."""
    J = abi.jvel(arrays, dx, dy)
    st = lib().orc_calc_jacobian_vel_3D(C.byref(J), abi.BOUNDARY_CODES[boundaries], int(terms))
    if st != 0:
        raise RuntimeError(f"orc_calc_jacobian_vel_3D failed ({st})")
    return arrays

def calc_uz_3D(arrays: dict, dx: float, dy: float, boundaries: str, method: int = 1, use_bmb: bool = True) -> dict:
    """orc_calc_uz_3D on the arrays of yelmo_gb300.gpu.uz_arrays (filled in place)."""
    U = abi.uz3d(arrays, dx, dy, use_bmb)
    st = lib().orc_calc_uz_3D(C.byref(U), abi.BOUNDARY_CODES[boundaries], int(method))
    if st != 0:
        raise RuntimeError(f"orc_calc_uz_3D failed ({st})")
    return arrays

def calc_strain_rate_tensor(arrays: dict, dx: float, dy: float, boundaries: str, de_max: float = 0.5) -> dict:
    """orc_calc_strain_rate_tensor on the arrays of yelmo_gb300.gpu.strain_arrays (filled in place)."""
    S = abi.strain3d(arrays, dx, dy, de_max)
    st = lib().orc_calc_strain_rate_tensor(C.byref(S), abi.BOUNDARY_CODES[boundaries])
    if st != 0:
        raise RuntimeError(f"orc_calc_strain_rate_tensor failed ({st})")
    return arrays


def linear_solve(ptr_, idx, val, b, x, method, precond, maxiter, tol, initx_zeros=False):
    it = C.c_int(0)
    rr = C.c_double(0.0)
    st = lib().orc_linear_solve(len(b), abi.ptr(ptr_, "i"), abi.ptr(idx, "i"), abi.ptr(val, "d"),
                                abi.ptr(b, "d"), abi.ptr(x, "d"), method, precond, maxiter, tol,
                                int(initx_zeros), C.byref(it), C.byref(rr))
    return st, it.value, rr.value
