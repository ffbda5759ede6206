"""Python host binding of libyelmo_gpu.so (the sm_103a solver).

Mirrors the reference's solver interface for Python hosts:

* ``calc_velocity(fields, dx, n_glen, par)`` -- calc_velocity_ssa /
  calc_velocity_diva (velocity_ssa.f90:60, velocity_diva.f90:59) on a dict of
  Fortran-ordered numpy arrays named as in the reference; INOUT arrays are
  updated in place, the integer counters are returned.
* ``calc_dyn_inputs(inst)`` / ``set_ssa_masks(...)`` / ``prepare(inst)`` -- the
  fields calc_ydyn derives before the solve and set_ssa_masks, on the GPU.
* ``linear_solver_matrix_solve(...)`` -- the CSR seam of solver_linear.F90:151.
* ``calc_velocity_batch(fields_list, dx, n_glen, par)`` -- many host states
  in one call (one batched solve on the device).
* ``DeviceSolver`` -- solves on device-resident fields (no host copies).

There is no CPU fallback: if the library cannot be loaded, or no CUDA device is
present, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi
from .params import YdynParams

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libyelmo_gpu.so")
_lib = None

EXPORTS = [
    "ygpu_dyn_par_defaults", "ygpu_parse_lis_opt", "ygpu_boundary_code", "ygpu_last_error", "ygpu_version",
    "ygpu_calc_velocity_ssa", "ygpu_calc_velocity_diva", "ygpu_set_ssa_masks", "ygpu_calc_dyn_inputs",
    "ygpu_calc_dyn_inputs_bg",
    "ygpu_linear_solver_matrix_solve", "ygpu_ctx_create", "ygpu_ctx_destroy", "ygpu_ctx_stream",
    "ygpu_solve_device", "ygpu_solve_batch_device", "ygpu_solve_device_noalloc",
    "ygpu_server_create", "ygpu_server_destroy", "ygpu_server_add_member", "ygpu_server_submit",
    "ygpu_server_poll", "ygpu_server_wait", "ygpu_server_fetch", "ygpu_server_get_info",
    "ygpu_server_member_steps", "ygpu_server_set_member_steps", "ygpu_calc_dyn_inputs_bg_device",
    "ygpu_set_ssa_masks_device", "ygpu_kernel_launches", "ygpu_step_timing", "ygpu_step_timing_get", "ygpu_tuning_defaults",
    "ygpu_ctx_set_tuning", "ygpu_set_neff_hook", "ygpu_solve_batch_host", "ygpu_calc_dyn_diagnostics",
    "ygpu_calc_dyn_diagnostics_device", "ygpu_calc_advec2D_impl_lis", "ygpu_advec2D_impl_lis_device",
    "ygpu_calc_gradient_column_ac", "ygpu_calc_gradient_column_ac_device", "ygpu_calc_jacobian_vel_3D",
    "ygpu_calc_jacobian_vel_3D_device", "ygpu_calc_uz_3D", "ygpu_calc_uz_3D_device", "ygpu_lin_method_run",
    "ygpu_calc_strain_rate_tensor", "ygpu_calc_strain_rate_tensor_device",
]


class YgpuError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {msg}")


def lib(build_if_missing: bool = True):
    """Load libyelmo_gpu.so (building it with nvcc if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) and build_if_missing:
        from . import build
        build.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run python -m yelmo_gb300.build")
    L = C.CDLL(LIB_PATH)
    abi.declare_velocity(L.ygpu_calc_velocity_ssa, abi.SSA_ARGS)
    abi.declare_velocity(L.ygpu_calc_velocity_diva, abi.DIVA_ARGS)
    abi.declare_inputs(L.ygpu_calc_dyn_inputs)
    abi.declare_inputs(L.ygpu_calc_dyn_inputs_bg, bg=True)
    abi.declare_masks(L.ygpu_set_ssa_masks)
    L.ygpu_last_error.restype = C.c_char_p
    L.ygpu_version.restype = C.c_char_p
    L.ygpu_boundary_code.argtypes = [C.c_char_p]
    L.ygpu_parse_lis_opt.argtypes = [C.c_char_p, C.POINTER(abi.DynPar)]
    L.ygpu_dyn_par_defaults.argtypes = [C.POINTER(abi.DynPar)]
    L.ygpu_ctx_create.restype = C.c_void_p
    L.ygpu_ctx_create.argtypes = [C.c_int]
    L.ygpu_ctx_destroy.argtypes = [C.c_void_p]
    L.ygpu_ctx_stream.restype = C.c_void_p
    L.ygpu_ctx_stream.argtypes = [C.c_void_p]
    L.ygpu_solve_device.argtypes = [C.c_void_p, C.c_int, C.POINTER(abi.DynPar), C.POINTER(abi.Fields),
                                    C.POINTER(abi.Stats)]
    L.ygpu_solve_batch_device.argtypes = [C.c_void_p, C.c_int, C.POINTER(abi.DynPar), C.c_int,
                                          C.POINTER(abi.Fields), C.POINTER(abi.Stats)]
    L.ygpu_calc_dyn_diagnostics.argtypes = [C.POINTER(abi.DynDiag), C.c_int]
    L.ygpu_calc_dyn_diagnostics_device.argtypes = [C.c_void_p, C.POINTER(abi.DynDiag), C.c_int]
    L.ygpu_solve_batch_host.argtypes = [C.c_int, C.POINTER(abi.DynPar), C.c_int, C.POINTER(abi.Fields),
                                        C.POINTER(abi.Stats)]
    L.ygpu_solve_device_noalloc.argtypes = [C.c_int, C.POINTER(abi.DynPar), C.POINTER(abi.Fields),
                                            C.POINTER(abi.Stats), C.c_void_p]
    ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
    L.ygpu_calc_advec2D_impl_lis.argtypes = [dp] * 5 + [ip, dp, C.c_double, C.c_double, C.c_double,
                                                        C.c_int, C.c_int, C.c_int, ip, ip]
    L.ygpu_advec2D_impl_lis_device.argtypes = [C.c_void_p] + [C.c_void_p] * 7 + [C.c_double, C.c_double, C.c_double,
                                                                              C.c_int, C.c_int, C.c_int, ip, ip]
    L.ygpu_linear_solver_matrix_solve.argtypes = [C.c_int, ip, ip, dp, dp, dp, C.c_char_p, ip, ip, dp]
    L.ygpu_calc_gradient_column_ac.argtypes = [dp] * 5 + [ip, C.c_int, C.c_int, C.c_int]
    L.ygpu_calc_gradient_column_ac_device.argtypes = [C.c_void_p] * 7 + [C.c_int, C.c_int, C.c_int]
    L.ygpu_calc_jacobian_vel_3D.argtypes = [C.POINTER(abi.JVel), C.c_int, C.c_int]
    L.ygpu_calc_jacobian_vel_3D_device.argtypes = [C.c_void_p, C.POINTER(abi.JVel), C.c_int, C.c_int]
    L.ygpu_calc_uz_3D.argtypes = [C.POINTER(abi.Uz3D), C.c_int, C.c_int]
    L.ygpu_calc_uz_3D_device.argtypes = [C.c_void_p, C.POINTER(abi.Uz3D), C.c_int, C.c_int]
    L.ygpu_server_create.restype = C.c_void_p
    L.ygpu_server_create.argtypes = [C.POINTER(abi.ServerCfg)]
    L.ygpu_server_destroy.argtypes = [C.c_void_p]
    L.ygpu_server_add_member.argtypes = [C.c_void_p, C.POINTER(abi.Fields), ip]
    L.ygpu_server_submit.argtypes = [C.c_void_p, C.c_int, C.c_ulonglong, ip]
    L.ygpu_server_poll.argtypes = [C.c_void_p, C.c_int]
    L.ygpu_server_wait.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(abi.Stats), dp]
    L.ygpu_server_fetch.argtypes = [C.c_void_p, C.c_int, C.c_int, dp]
    L.ygpu_server_get_info.argtypes = [C.c_void_p, C.POINTER(abi.ServerInfo)]
    L.ygpu_calc_dyn_inputs_bg_device.argtypes = [C.c_void_p] + [C.c_void_p] * 16 + [C.c_double] * 8 + \
        [C.c_int] * 3
    L.ygpu_set_ssa_masks_device.argtypes = [C.c_void_p] * 6 + [C.c_int] * 4
    L.ygpu_server_member_steps.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_ulonglong)]
    L.ygpu_server_set_member_steps.argtypes = [C.c_void_p, C.c_int, C.c_ulonglong]
    L.ygpu_kernel_launches.restype = C.c_ulonglong
    L.ygpu_tuning_defaults.argtypes = [C.POINTER(abi.Tuning)]
    L.ygpu_set_neff_hook.argtypes = [abi.NEFF_HOOK, C.c_void_p]
    L.ygpu_set_neff_hook.restype = None
    L.ygpu_ctx_set_tuning.argtypes = [C.c_void_p, C.POINTER(abi.Tuning)]
    L.ygpu_step_timing.argtypes = [C.c_int]
    L.ygpu_step_timing_get.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
    L.ygpu_lin_method_run.argtypes = [C.POINTER(abi.DynPar), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.ygpu_lin_method_run.restype = None
    L.ygpu_calc_strain_rate_tensor.argtypes = [C.POINTER(abi.Strain3D), C.c_int]
    L.ygpu_calc_strain_rate_tensor_device.argtypes = [C.c_void_p, C.POINTER(abi.Strain3D), C.c_int]
    _lib = L
    return L


def last_error() -> str:
    return lib().ygpu_last_error().decode()


def _check(st, allow_linear=True):
    if st < 0 or (not allow_linear and st != 0):
        raise YgpuError(st, last_error())
    return st


def calc_velocity(fields: dict, dx: float, n_glen: float, par: YdynParams, dy: float | None = None,
                  neff_hook=None) -> dict:
    """calc_velocity_ssa / calc_velocity_diva on the GPU (host arrays, updated in place).

    neff_hook(c_bed, ux_b, uy_b): DIVA only, called after every Picard iteration to
    update c_bed in place (fields["c_bed"] is then in/out)."""
    L = lib()
    cpar = par.to_c()
    dy = dx if dy is None else dy
    if par.solver == "ssa":
        out = abi.call_velocity(L.ygpu_calc_velocity_ssa, abi.SSA_ARGS, fields, dx, dy, n_glen, cpar)
    else:
        cb = abi.neff_hook(neff_hook) if neff_hook else None
        if cb:
            L.ygpu_set_neff_hook(cb, None)
        try:
            out = abi.call_velocity(L.ygpu_calc_velocity_diva, abi.DIVA_ARGS, fields, dx, dy, n_glen, cpar)
        finally:
            if cb:
                L.ygpu_set_neff_hook(abi.NEFF_HOOK(), None)
    _check(out["status"])
    return out


_FIELDS_3D = {"ux", "uy", "ux_i", "uy_i", "visc_eff", "duxdz", "duydz", "ATT"}


def calc_velocity_batch(fields: list, dx, n_glen: float, par: YdynParams, neff_hook=None) -> list:
    """calc_velocity on a batch of host states in one call (ygpu_solve_batch_host).

    fields: dicts as for calc_velocity, updated in place; dx: one grid spacing or
    one per instance (dy = dx). neff_hook: as for calc_velocity, for a single
    DIVA state. Returns the per-instance stats dicts."""
    n = len(fields)
    if n == 0:
        return []
    dxs = list(dx) if isinstance(dx, (list, tuple)) else [dx] * n
    kind = abi.KIND_SSA if par.solver == "ssa" else abi.KIND_DIVA
    names = {a for a, t in (abi.SSA_ARGS if kind == abi.KIND_SSA else abi.DIVA_ARGS) if t != "s"}
    arr = (abi.Fields * n)()
    for k, f in enumerate(fields):
        nx, ny = f["H_ice"].shape
        nz = f["zeta_aa"].shape[0]
        F = arr[k]
        F.nx, F.ny, F.nz, F.dx, F.dy, F.n_glen = nx, ny, nz, dxs[k], dxs[k], n_glen
        for name, _ in abi.Fields._fields_[6:]:
            if name not in names:
                continue
            a = f[name]
            want = (nz,) if name == "zeta_aa" else (nx, ny, nz) if name in _FIELDS_3D else (nx, ny)
            if a.shape != want:
                raise ValueError(f"instance {k}, {name}: shape {a.shape}, expected {want}")
            abi.ptr(a, "i" if name.startswith("ssa_mask") else "d")
            setattr(F, name, a.ctypes.data)
    sts = (abi.Stats * n)()
    cpar = par.to_c()
    L = lib()
    cb = abi.neff_hook(neff_hook) if neff_hook else None
    if cb:
        L.ygpu_set_neff_hook(cb, None)
    try:
        _check(L.ygpu_solve_batch_host(kind, C.byref(cpar), n, arr, sts))
    finally:
        if cb:
            L.ygpu_set_neff_hook(abi.NEFF_HOOK(), None)
    return [s.as_dict() for s in sts]


def diagnostics_arrays(fields: dict, nz: int, want_3d: bool = True, want_avg: bool = True) -> dict:
    """Inputs of the post-solve diagnostics taken from a solve's field dict, with
    zeroed output arrays (the groups: depth averages from ux_i, 3D magnitudes from ux)."""
    nx, ny = fields["H_ice"].shape
    out = {k: fields[k] for k in abi.DIAG_INPUTS[:11]}
    if want_avg and "ux_i" in fields:
        out.update(ux_i=fields["ux_i"], uy_i=fields["uy_i"], zeta_aa=fields["zeta_aa"])
    if want_3d and "ux" in fields:
        out.update(ux=fields["ux"], uy=fields["uy"])
    for k in abi.DIAG_OUTPUTS:
        if k == "uxy":
            if "ux" in out:
                out[k] = np.zeros((nx, ny, nz), order="F")
        elif k in ("ux_s", "uy_s", "uxy_s", "f_vbvs") and "ux" not in out:
            continue
        elif k in ("ux_i_bar", "uy_i_bar", "uxy_i_bar") and "ux_i" not in out:
            continue
        else:
            out[k] = np.zeros((nx, ny), order="F")
    return out


def calc_dyn_diagnostics(arrays: dict, dx: float, dy: float, boundaries: str) -> dict:
    """Post-solve diagnostics on the GPU (ygpu_calc_dyn_diagnostics); the output
    arrays of `arrays` (see diagnostics_arrays) are filled in place."""
    nx, ny = arrays["H_ice"].shape
    nz = arrays["zeta_aa"].shape[0] if "zeta_aa" in arrays else (arrays["ux"].shape[2] if "ux" in arrays else 1)
    D = abi.dyn_diag(arrays, nx, ny, nz, dx, dy)
    _check(lib().ygpu_calc_dyn_diagnostics(C.byref(D), abi.BOUNDARY_CODES[boundaries]))
    return arrays


def calc_advec2D_impl_lis(var, ux, uy, var_dot, mask_ice, var_ref, dx: float, dy: float, dt: float,
                          boundaries: str):
    """calc_advec2D(solver = "impl-lis") on the GPU (ygpu_calc_advec2D_impl_lis):
    returns (dvdt, lin_iter, lin_status). mask_ice: int32 MASK_ICE_* (0 none,
    1 fixed, 2 dynamic)."""
    nx, ny = var.shape
    dvdt = np.zeros((nx, ny), order="F")
    it, st = C.c_int(0), C.c_int(0)
    r = lib().ygpu_calc_advec2D_impl_lis(abi.ptr(dvdt, "d"), abi.ptr(var, "d"), abi.ptr(ux, "d"), abi.ptr(uy, "d"),
                                         abi.ptr(var_dot, "d"), abi.ptr(mask_ice, "i"), abi.ptr(var_ref, "d"),
                                         dx, dy, dt, abi.ADV_BOUNDARY_CODES[boundaries], nx, ny,
                                         C.byref(it), C.byref(st))
    _check(r)
    return dvdt, it.value, st.value


def calc_gradient_column_ac(dvdx, dvdy, f_ice, mask_ocn, boundaries: str):
    """calc_gradient_column_ac on the GPU: (dvdx_c, dvdy_c). mask_ocn: nonzero
    where the bed lies below sea level."""
    nx, ny = f_ice.shape
    gx = np.zeros((nx, ny), order="F")
    gy = np.zeros((nx, ny), order="F")
    ocn = np.asfortranarray(mask_ocn, dtype=np.int32)
    _check(lib().ygpu_calc_gradient_column_ac(abi.ptr(gx, "d"), abi.ptr(gy, "d"), abi.ptr(dvdx, "d"),
                                              abi.ptr(dvdy, "d"), abi.ptr(f_ice, "d"), abi.ptr(ocn, "i"),
                                              abi.BOUNDARY_CODES[boundaries], nx, ny))
    return gx, gy


def jacobian_arrays(inputs: dict, terms: int = abi.JAC_UXY | abi.JAC_UZ) -> dict:
    """`inputs` (JAC_INPUTS names) with zeroed output arrays for `terms`."""
    nx, ny = inputs["H_ice"].shape
    out = dict(inputs)
    nza = inputs["zeta_aa"].shape[0] if "zeta_aa" in inputs else 0
    nzc = inputs["zeta_ac"].shape[0] if "zeta_ac" in inputs else 0
    if terms & abi.JAC_UXY:
        for n in abi.JAC_OUTPUTS[:6]:
            out[n] = np.zeros((nx, ny, nza), order="F")
    if nzc:
        for n in abi.JAC_OUTPUTS[6:]:
            out[n] = np.zeros((nx, ny, nzc), order="F")
    return out


def calc_jacobian_vel_3D(arrays: dict, dx: float, dy: float, boundaries: str,
                         terms: int = abi.JAC_UXY | abi.JAC_UZ) -> dict:
    """Velocity Jacobian on the GPU (ygpu_calc_jacobian_vel_3D); the output arrays
    of `arrays` (see jacobian_arrays) are filled in place."""
    J = abi.jvel(arrays, dx, dy)
    _check(lib().ygpu_calc_jacobian_vel_3D(C.byref(J), abi.BOUNDARY_CODES[boundaries], int(terms)))
    return arrays

def uz_arrays(inputs: dict, srf_err: bool = True) -> dict:
    """`inputs` (UZ_INPUTS names) with zeroed uz, uz_star (and uz_srf_err)."""
    nx, ny = inputs["H_ice"].shape
    nzc = inputs["zeta_ac"].shape[0]
    out = dict(inputs)
    out["uz"] = np.zeros((nx, ny, nzc), order="F")
    out["uz_star"] = np.zeros((nx, ny, nzc), order="F")
    if srf_err:
        out["uz_srf_err"] = np.zeros((nx, ny), order="F")
    return out


def calc_uz_3D(arrays: dict, dx: float, dy: float, boundaries: str, method: int = abi.UZ_AA,
               use_bmb: bool = True) -> dict:
    """Vertical velocity on the GPU (ygpu_calc_uz_3D, uz_method 1 to 4; method 3
    reads jac_dxx / jac_dyy); the output arrays of `arrays` (see uz_arrays) are
    filled in place."""
    U = abi.uz3d(arrays, dx, dy, use_bmb)
    _check(lib().ygpu_calc_uz_3D(C.byref(U), abi.BOUNDARY_CODES[boundaries], int(method)))
    return arrays

def strain_arrays(jac: dict, inputs: dict, want_2d: bool = True) -> dict:
    """The strain-rate tensor's inputs (the Jacobian's dxx ... dzy from `jac`, the
    geometry from `inputs`) with zeroed outputs."""
    nx, ny = inputs["H_ice"].shape
    nza = inputs["zeta_aa"].shape[0]
    out = {k: jac[k] for k in ("dxx", "dxy", "dxz", "dyx", "dyy", "dyz", "dzx", "dzy")}
    for k in ("H_ice", "f_ice", "f_grnd", "zeta_aa", "zeta_ac"):
        out[k] = inputs[k]
    for k in abi.STRAIN_OUTPUTS_3D:
        out[k] = np.zeros((nx, ny, nza), order="F")
    if want_2d:
        for k in abi.STRAIN_OUTPUTS_2D:
            out[k] = np.zeros((nx, ny), order="F")
    return out


def calc_strain_rate_tensor(arrays: dict, dx: float, dy: float, boundaries: str, de_max: float = 0.5) -> dict:
    """Strain-rate tensor on the GPU (ygpu_calc_strain_rate_tensor) on the arrays of
    strain_arrays (outputs filled in place)."""
    S = abi.strain3d(arrays, dx, dy, de_max)
    _check(lib().ygpu_calc_strain_rate_tensor(C.byref(S), abi.BOUNDARY_CODES[boundaries]))
    return arrays


def calc_dyn_inputs(inst) -> dict:
    d = inst.input_buffers()
    p = inst.par
    bg = tuple(getattr(inst, "slope_bg", (0.0, 0.0)))
    fn = lib().ygpu_calc_dyn_inputs if bg == (0.0, 0.0) else lib().ygpu_calc_dyn_inputs_bg
    _check(abi.call_inputs(fn, d, inst.dx, p.grad_lim, p.taud_lim, p.rho_ice, p.rho_sw, p.g,
                           abi.BOUNDARY_CODES[p.boundaries], None if bg == (0.0, 0.0) else bg))
    return d


def set_ssa_masks(mask_frnt, f_ice, f_grnd, lateral_bc: str, boundaries: str):
    nx, ny = f_ice.shape
    mx = np.zeros((nx, ny), dtype=np.int32, order="F")
    my = np.zeros((nx, ny), dtype=np.int32, order="F")
    _check(lib().ygpu_set_ssa_masks(abi.ptr(mx, "i"), abi.ptr(my, "i"), abi.ptr(mask_frnt, "i"),
                                    abi.ptr(f_ice, "d"), abi.ptr(f_grnd, "d"), abi.LATBC_CODES[lateral_bc],
                                    abi.BOUNDARY_CODES[boundaries], nx, ny))
    return mx, my


def prepare(inst) -> dict:
    """Cold-start state of one solve with the GPU prologue and masks."""
    inputs = calc_dyn_inputs(inst)
    f = inst.state(inputs)
    f["ssa_mask_acx"], f["ssa_mask_acy"] = set_ssa_masks(
        inputs["mask_frnt"], inputs["f_ice"], inputs["f_grnd"], inst.par.ssa_lat_bc, inst.par.boundaries)
    return f


def linear_solver_matrix_solve(a_ptr1, a_index1, a_value, b_value, x_value, lis_opt: str):
    """GPU solve of a 1-based CSR system (linear_solver_class arrays); x updated in place."""
    it, st, rr = C.c_int(0), C.c_int(0), C.c_double(0.0)
    ret = lib().ygpu_linear_solver_matrix_solve(
        len(b_value), abi.ptr(a_ptr1, "i"), abi.ptr(a_index1, "i"), abi.ptr(a_value, "d"),
        abi.ptr(b_value, "d"), abi.ptr(x_value, "d"), lis_opt.encode(), C.byref(it), C.byref(st), C.byref(rr))
    _check(ret)
    return st.value, it.value, rr.value


# ---------------------------------------------------------------------------
# device-resident solves (torch tensors as device memory)
# ---------------------------------------------------------------------------
FIELD_NAMES_2D = ["ux_bar", "uy_bar", "ux_b", "uy_b", "taub_acx", "taub_acy", "beta", "beta_acx", "beta_acy",
                  "beta_eff", "visc_eff_int", "ssa_err_acx", "ssa_err_acy", "c_bed", "f_slide", "taud_acx",
                  "taud_acy", "taul_int_acx", "taul_int_acy", "H_ice", "f_ice", "H_grnd", "f_grnd",
                  "f_grnd_acx", "f_grnd_acy", "z_sl", "z_bed", "z_srf"]
FIELD_NAMES_3D = ["ux", "uy", "ux_i", "uy_i", "visc_eff", "duxdz", "duydz", "ATT"]
INT_NAMES = ["ssa_mask_acx", "ssa_mask_acy"]
STATE_NAMES = ["ux_bar", "uy_bar", "ux_b", "uy_b", "taub_acx", "taub_acy", "beta", "beta_acx", "beta_acy",
               "visc_eff"]


def to_device(fields: dict, device: str = "cuda"):
    """Copy a field dict to torch device tensors (same memory layout as the Fortran arrays)."""
    import torch
    out = {}
    for k, a in fields.items():
        if not isinstance(a, np.ndarray):
            continue
        flat = np.ravel(a, order="F")
        out[k] = torch.from_numpy(np.ascontiguousarray(flat)).to(device)
    return out


def make_fields(dev: dict, nx, ny, nz, dx, dy, n_glen) -> abi.Fields:
    f = abi.Fields()
    f.nx, f.ny, f.nz, f.dx, f.dy, f.n_glen = nx, ny, nz, dx, dy, n_glen
    for name, _ in abi.Fields._fields_[6:]:
        t = dev.get(name)
        setattr(f, name, t.data_ptr() if t is not None else None)
    return f


def solve_device_noalloc(kind: int, par: YdynParams, fields: abi.Fields, stream: int = 0) -> dict:
    """ygpu_solve_device_noalloc: the solve with the library's fixed scratch array
    (no device allocation); ``stream`` is a cudaStream_t handle (0: default stream)."""
    st = abi.Stats()
    cpar = par.to_c()
    r = lib().ygpu_solve_device_noalloc(kind, C.byref(cpar), C.byref(fields), C.byref(st),
                                        C.c_void_p(stream) if stream else None)
    _check(r)
    out = st.as_dict()
    out["return"] = r
    return out


class DeviceSolver:
    """A solver context (one CUDA stream) for device-resident solves."""

    def __init__(self, device: int = 0):
        self.L = lib()
        self.ctx = self.L.ygpu_ctx_create(device)
        if not self.ctx:
            raise YgpuError(abi.ERR_CUDA, last_error())

    def close(self):
        if self.ctx:
            self.L.ygpu_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, kind: int, par: YdynParams, fields: abi.Fields) -> dict:
        st = abi.Stats()
        cpar = par.to_c()
        r = self.L.ygpu_solve_device(self.ctx, kind, C.byref(cpar), C.byref(fields), C.byref(st))
        _check(r)
        out = st.as_dict()
        out["return"] = r
        return out

    def set_tuning(self, check_every: int = 4, use_graphs: bool = True, unknowns_per_cta: int = 512,
                   max_active_unknowns: int = 1_500_000, spin_log2: int = 0, cluster_ctas: int = 0):
        """ygpu_ctx_set_tuning: host-check interval, chunk graphs, team size, queue threshold;
        spin_log2 > 0 lowers the team waits' spin budget to 2^spin_log2 polls (tests);
        cluster_ctas: Krylov teams as thread-block clusters of 2..16 CTAs (0 or -1: global teams)."""
        t = abi.Tuning(check_every, 1 if use_graphs else 0, unknowns_per_cta, max_active_unknowns, spin_log2,
                       cluster_ctas)
        _check(self.L.ygpu_ctx_set_tuning(self.ctx, C.byref(t)))
        self.tuning = {"check_every": check_every, "use_graphs": bool(use_graphs),
                       "unknowns_per_cta": unknowns_per_cta, "max_active_unknowns": max_active_unknowns,
                       "cluster_ctas": cluster_ctas}

    def solve_batch(self, kind: int, par: YdynParams, fields: list) -> list:
        n = len(fields)
        arr = (abi.Fields * n)(*fields)
        sts = (abi.Stats * n)()
        cpar = par.to_c()
        r = self.L.ygpu_solve_batch_device(self.ctx, kind, C.byref(cpar), n, arr, sts)
        _check(r)
        return [s.as_dict() for s in sts]


STEP_NAMES = ("setup", "pre", "krylov", "post", "final")


def kernel_launches() -> int:
    """Kernels the library has launched in this process."""
    return int(lib().ygpu_kernel_launches())


def step_timing(on: bool):
    """Switch CUDA-event timing of every solver step launch on (clearing the totals) or off."""
    lib().ygpu_step_timing(1 if on else 0)


def step_timing_get() -> dict:
    """{step: (device ms, launches)} since step_timing(True)."""
    ms = (C.c_double * 5)()
    n = (C.c_longlong * 5)()
    lib().ygpu_step_timing_get(ms, n)
    return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(STEP_NAMES)}


def host_io_bytes(kind: int, nx: int, ny: int, nz: int):
    """Bytes the host-pointer drop-in copies in and out (ygpu_calc_velocity_* staging)."""
    b2, b3, i2, bz = 8 * nx * ny, 8 * nx * ny * nz, 4 * nx * ny, 8 * nz
    inputs_common = 13 * b2 + b3 + bz + 2 * i2       # c_bed..z_srf (13 2D), ATT, zeta, masks
    if kind == abi.KIND_SSA:
        h2d = 7 * b2 + b3 + inputs_common             # ux_b, uy_b, taub x2, beta x3, visc
        d2h = 10 * b2 + b3                            # ux_b, uy_b, taub x2, visc_int, err x2, beta x3, visc
    else:
        h2d = 9 * b2 + b3 + inputs_common             # ux_bar, uy_bar, ux_b, uy_b, taub x2, beta x3, visc
        d2h = 13 * b2 + 7 * b3                        # 2D: ux_bar..uy_b(4), taub(2), beta(3), beta_eff, visc_int, err(2)
    return h2d, d2h


def algorithmic_bytes(stats: dict, kind: int, nx: int, ny: int, nz: int, mixed: bool, energy: bool = True,
                      cg: bool = True, by_step: bool = False, krylov64: bool = False, minimal: bool = False):
    """Algorithmic HBM bytes of one solve: every distinct array read once and
    written once per kernel pass, per cell (w = 8 B FP64, 4 B FP32):

    - pre step, per Picard iteration: strain rates 7w, column pass (3nz+14)w
      DIVA / (3nz+10)w SSA (read u, taub, H, f_ice, c_bed, f_slide, f_grnd,
      visc_prev, ATT; write visc, N, F2, beta), faces 20w+8, system 16w+8;
    - Krylov step, per active cell (a cell with a non-identity row; the
      iterations skip the others): pipelined CG iteration 42w+8 (read the operator input,
      N, N_ab, two drag arrays, the row flags, the preconditioner and eight
      recurrence vectors; write the eight vectors and the next operator
      input), BiCGSTAB iteration 62w+16 (two operator applies of 8w+8 and
      46w of vector passes); mixed mode, per active cell: each FP64
      defect-correction step 186 B (FP64 operator 66, residual 48,
      conversions 32, update 40);
    - mixed mode, pre step: the FP32 coefficient copies, 72 B per cell and
      Picard iteration;
    - post step, per Picard iteration: epilogue 16w+8.

    krylov64: the mixed mode's Krylov step runs in FP64 (BiCGSTAB with ILU(0) on
    the residual form). minimal: the Krylov bytes of the least-traffic form of the
    same method instead, per active cell and iteration: plain PCG 23w (per row the
    operator input, the coefficients' share and the output, x, r and p read and
    written, the preconditioner read and z written), BiCGSTAB 36w (two operator
    applies and the eight vector updates, each vector read or written once).

    Returns the total, or {step: bytes} with by_step."""
    n2 = nx * ny
    w = 8
    picard = stats["ssa_iter_now"]
    lin = stats["ssa_lin_iter"]
    col = (3 * nz + (14 if kind == abi.KIND_DIVA else 10)) * w
    pre = 7 * w + col + (20 * w + 8) + (16 * w + 8)
    post = 16 * w + 8
    wk = 4 if (mixed and not krylov64) else 8
    if minimal:
        it_bytes = (23 * wk) if cg else (36 * wk)
    else:
        it_bytes = (42 * wk + 8) if cg else (62 * wk + 16)
    n_act = stats.get("active_cells") or n2
    krylov = float(n_act) * lin * it_bytes
    if mixed:
        krylov += float(n_act) * stats.get("outer_iter", 0) * 186
        pre += 72
    steps = {"pre": float(n2) * picard * pre, "krylov": krylov, "post": float(n2) * picard * post}
    return steps if by_step else sum(steps.values())