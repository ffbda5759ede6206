"""ctypes mirror of ``include/yelmo_gpu.h`` (structs, codes, prototypes).

The C header is the interface; this module only restates its layouts so that
Python hosts (and the tests) can call the shared library with plain pointers.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

# status codes (yelmo_gpu.h; 0/2/4 are the LIS codes of solver_linear.F90:36-39)
OK, BREAKDOWN, MAXITER = 0, 2, 4
ERR_NONFINITE, ERR_BAD_ARG, ERR_CUDA, ERR_TIMEOUT = -1, -2, -3, -4
ERR_ADMISSION, ERR_NOMEM, ERR_BUSY = -5, -6, -7

STATUS_NAMES = {
    OK: "ok", BREAKDOWN: "BREAKDOWN", MAXITER: "MAXITER", ERR_NONFINITE: "NONFINITE",
    ERR_BAD_ARG: "BAD_ARG", ERR_CUDA: "CUDA_ERROR", ERR_TIMEOUT: "TIMEOUT",
    ERR_ADMISSION: "ADMISSION_REJECTED", ERR_NOMEM: "NOMEM", ERR_BUSY: "BUSY",
}

# boundary codes, yelmo_tools.f90:14-20 and boundary_code() :248-271
# boundary strings of the advection entry: "mask" has its own code there
ADV_BOUNDARY_CODES = {"zeros": 0, "infinite": 1, "MISMIP3D": 2, "TROUGH": 3, "periodic": 4,
                      "periodic-x": 5, "periodic-y": 6, "mask": 7}
BOUNDARY_CODES = {
    "zeros": 0, "infinite": 1, "mask": 1, "MISMIP3D": 2, "TROUGH": 3,
    "periodic": 4, "periodic-x": 5, "periodic-y": 6,
}
LATBC_CODES = {"none": 0, "floating": 1, "float": 1, "marine": 2, "all": 3}
SSA_SOLVER_CODES = {"residual": 0, "energy": 1}
VEL_LIM_CODES = {"clip": 0, "drag": 1}
LIN_CG, LIN_BICGSTAB, LIN_MINRES = 0, 1, 2
PRE_NONE, PRE_JACOBI, PRE_ILU0, PRE_TILE_BLOCK = 0, 1, 2, 3
PREC_FP64, PREC_MIXED = 0, 1
KIND_SSA, KIND_DIVA = 0, 1


class DynPar(C.Structure):
    """ygpu_dyn_par: ssa_param_class / diva_param_class + parsed ssa_lis_opt."""
    _fields_ = [
        ("ssa_solver", C.c_int), ("boundaries", C.c_int), ("no_slip", C.c_int),
        ("visc_method", C.c_int), ("visc_const", C.c_double),
        ("beta_method", C.c_int), ("beta_const", C.c_double), ("beta_q", C.c_double),
        ("beta_u0", C.c_double), ("beta_gl_scale", C.c_int), ("beta_gl_stag", C.c_int),
        ("beta_gl_f", C.c_double), ("H_grnd_lim", C.c_double), ("beta_min", C.c_double),
        ("eps_0", C.c_double), ("ssa_vel_lim_method", C.c_int), ("ssa_vel_lim_tau", C.c_double),
        ("ssa_vel_max", C.c_double), ("ssa_iter_max", C.c_int), ("ssa_iter_rel", C.c_double),
        ("ssa_iter_conv", C.c_double), ("ssa_write_log", C.c_int),
        ("rho_ice", C.c_double), ("rho_sw", C.c_double), ("g", C.c_double),
        ("lin_solver", C.c_int), ("lin_precond", C.c_int), ("lin_maxiter", C.c_int),
        ("lin_tol", C.c_double), ("lin_initx_zeros", C.c_int),
        ("precision", C.c_int), ("inner_maxiter", C.c_int), ("inner_tol", C.c_double),
    ]


class Stats(C.Structure):
    """ygpu_stats."""
    _fields_ = [
        ("ssa_iter_now", C.c_int), ("ssa_lin_iter", C.c_int), ("ssa_lin_fail", C.c_int),
        ("ssa_lim_n", C.c_int), ("ssa_resid", C.c_double), ("lin_resid", C.c_double),
        ("outer_iter", C.c_int), ("status", C.c_int), ("device_ms", C.c_double),
        ("phase_ms", C.c_double * 10), ("active_cells", C.c_int),
        ("lin_solver_run", C.c_int), ("lin_precond_run", C.c_int),
    ]

    PHASES = ("setup", "strain", "column", "faces", "system", "krylov", "epilogue", "final", "sync_all",
              "sync_krylov")

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "phase_ms"}
        d["phase_ms"] = {n: float(self.phase_ms[i]) for i, n in enumerate(self.PHASES)}
        return d


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

DIAG_INPUTS = ("ux_bar", "uy_bar", "ux_b", "uy_b", "taub_acx", "taub_acy", "taud_acx", "taud_acy",
               "H_ice", "f_ice", "f_grnd", "ux_i", "uy_i", "zeta_aa", "ux", "uy")
DIAG_OUTPUTS = ("ux_i_bar", "uy_i_bar", "qq_acx", "qq_acy", "qq", "qq_gl_acx", "qq_gl_acy", "taub", "taud",
                "uxy_b", "uxy_i_bar", "uxy_bar", "uxy", "ux_s", "uy_s", "uxy_s", "f_vbvs")


class DynDiag(C.Structure):
    """ygpu_dyn_diag: arrays of the post-solve diagnostics."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("dx", C.c_double), ("dy", C.c_double)] + \
        [(n, C.c_void_p) for n in DIAG_INPUTS + DIAG_OUTPUTS]


def dyn_diag(arrays: dict, nx: int, ny: int, nz: int, dx: float, dy: float) -> DynDiag:
    """A DynDiag over the numpy arrays of `arrays` (absent names stay NULL)."""
    D = DynDiag()
    D.nx, D.ny, D.nz, D.dx, D.dy = nx, ny, nz, dx, dy
    for n in DIAG_INPUTS + DIAG_OUTPUTS:
        a = arrays.get(n)
        if a is None:
            continue
        want = (nz,) if n == "zeta_aa" else (nx, ny, nz) if n in ("ux_i", "uy_i", "ux", "uy", "uxy") else (nx, ny)
        if a.shape != want:
            raise ValueError(f"{n}: shape {a.shape}, expected {want}")
        ptr(a, "d")
        setattr(D, n, a.ctypes.data)
    return D


JAC_INPUTS = ("ux", "uy", "uz", "H_ice", "f_ice", "dzsdx", "dzsdy", "dzbdx", "dzbdy", "zeta_aa", "zeta_ac")
JAC_OUTPUTS = ("dxx", "dxy", "dxz", "dyx", "dyy", "dyz", "dzx", "dzy", "dzz")
JAC_UXY, JAC_UZ = 1, 2


class JVel(C.Structure):
    """ygpu_jvel: arrays of the velocity Jacobian."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz_aa", C.c_int), ("nz_ac", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double)] + [(n, C.c_void_p) for n in JAC_INPUTS + JAC_OUTPUTS]


def jvel(arrays: dict, dx: float, dy: float) -> JVel:
    """A JVel over the numpy arrays of `arrays` (absent names stay NULL); the
    layer counts come from zeta_aa / zeta_ac."""
    nx, ny = arrays["H_ice"].shape
    nza = arrays["zeta_aa"].shape[0] if "zeta_aa" in arrays else 0
    nzc = arrays["zeta_ac"].shape[0] if "zeta_ac" in arrays else (arrays["dzz"].shape[2] if "dzz" in arrays else 0)
    J = JVel()
    J.nx, J.ny, J.nz_aa, J.nz_ac, J.dx, J.dy = nx, ny, nza, nzc, dx, dy
    for n in JAC_INPUTS + JAC_OUTPUTS:
        a = arrays.get(n)
        if a is None:
            continue
        if n == "zeta_aa":
            want = (nza,)
        elif n == "zeta_ac":
            want = (nzc,)
        elif n in ("ux", "uy", "dxx", "dxy", "dxz", "dyx", "dyy", "dyz"):
            want = (nx, ny, nza)
        elif n in ("uz", "dzx", "dzy", "dzz"):
            want = (nx, ny, nzc)
        else:
            want = (nx, ny)
        if a.shape != want:
            raise ValueError(f"{n}: shape {a.shape}, expected {want}")
        ptr(a, "d")
        setattr(J, n, a.ctypes.data)
    return J

UZ_INPUTS = ("ux", "uy", "H_ice", "f_ice", "smb", "bmb", "dzbdt", "dzsdt", "dzsdx", "dzsdy", "dzbdx", "dzbdy",
             "zeta_aa", "zeta_ac", "ux_bar", "uy_bar", "dHidt_dyn", "mask_kin")
UZ_OUTPUTS = ("uz", "uz_star", "uz_srf_err")
UZ_JAC_INPUTS = ("jac_dxx", "jac_dyy")
UZ_AA, UZ_NODES, UZ_JAC, UZ_FLUX = 1, 2, 3, 4


class Uz3D(C.Structure):
    """ygpu_uz3d: arrays of the vertical velocity."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz_aa", C.c_int), ("nz_ac", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("use_bmb", C.c_int)] + \
        [(n, C.c_void_p) for n in UZ_INPUTS + UZ_OUTPUTS + UZ_JAC_INPUTS]


def uz3d(arrays: dict, dx: float, dy: float, use_bmb: bool = True) -> Uz3D:
    """A Uz3D over the numpy arrays of `arrays` (absent names stay NULL)."""
    nx, ny = arrays["H_ice"].shape
    nza, nzc = arrays["zeta_aa"].shape[0], arrays["zeta_ac"].shape[0]
    U = Uz3D()
    U.nx, U.ny, U.nz_aa, U.nz_ac, U.dx, U.dy, U.use_bmb = nx, ny, nza, nzc, dx, dy, int(bool(use_bmb))
    for n in UZ_INPUTS + UZ_OUTPUTS + UZ_JAC_INPUTS:
        a = arrays.get(n)
        if a is None:
            continue
        want = {"zeta_aa": (nza,), "zeta_ac": (nzc,), "ux": (nx, ny, nza), "uy": (nx, ny, nza),
                "uz": (nx, ny, nzc), "uz_star": (nx, ny, nzc), "jac_dxx": (nx, ny, nza),
                "jac_dyy": (nx, ny, nza)}.get(n, (nx, ny))
        if a.shape != want:
            raise ValueError(f"{n}: shape {a.shape}, expected {want}")
        ptr(a, "i" if n == "mask_kin" else "d")
        setattr(U, n, a.ctypes.data)
    return U

STRAIN_INPUTS = ("dxx", "dxy", "dxz", "dyx", "dyy", "dyz", "dzx", "dzy", "H_ice", "f_ice", "f_grnd",
                 "zeta_aa", "zeta_ac")
STRAIN_OUTPUTS_3D = ("s_dxx", "s_dyy", "s_dxy", "s_dxz", "s_dyz", "s_de", "s_div", "s_f_shear")
STRAIN_OUTPUTS_2D = ("a_dxx", "a_dyy", "a_dxy", "a_dxz", "a_dyz", "a_de", "a_div", "a_f_shear", "eps_eig_1",
                     "eps_eig_2")


class Strain3D(C.Structure):
    """ygpu_strain3d: arrays of the strain-rate tensor."""
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz_aa", C.c_int), ("nz_ac", C.c_int),
                ("dx", C.c_double), ("dy", C.c_double), ("de_max", C.c_double)] + \
        [(n, C.c_void_p) for n in STRAIN_INPUTS + STRAIN_OUTPUTS_3D + STRAIN_OUTPUTS_2D]


def strain3d(arrays: dict, dx: float, dy: float, de_max: float) -> Strain3D:
    """A Strain3D over the numpy arrays of `arrays` (absent names stay NULL)."""
    nx, ny = arrays["H_ice"].shape
    nza, nzc = arrays["zeta_aa"].shape[0], arrays["zeta_ac"].shape[0]
    S = Strain3D()
    S.nx, S.ny, S.nz_aa, S.nz_ac, S.dx, S.dy, S.de_max = nx, ny, nza, nzc, dx, dy, de_max
    for n in STRAIN_INPUTS + STRAIN_OUTPUTS_3D + STRAIN_OUTPUTS_2D:
        a = arrays.get(n)
        if a is None:
            continue
        if n == "zeta_aa":
            want = (nza,)
        elif n == "zeta_ac":
            want = (nzc,)
        elif n in ("dzx", "dzy"):
            want = (nx, ny, nzc)
        elif n in STRAIN_OUTPUTS_3D or n in ("dxx", "dxy", "dxz", "dyx", "dyy", "dyz"):
            want = (nx, ny, nza)
        else:
            want = (nx, ny)
        if a.shape != want:
            raise ValueError(f"{n}: shape {a.shape}, expected {want}")
        ptr(a, "d")
        setattr(S, n, a.ctypes.data)
    return S


class Fields(C.Structure):
    """ygpu_fields: device pointers of one instance."""
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("n_glen", C.c_double),
    ] + [(n, C.c_void_p) for n in (
        "ux", "uy", "ux_bar", "uy_bar", "ux_b", "uy_b", "ux_i", "uy_i",
        "taub_acx", "taub_acy", "beta", "beta_acx", "beta_acy", "beta_eff",
        "visc_eff", "visc_eff_int", "duxdz", "duydz", "ssa_err_acx", "ssa_err_acy",
        "ssa_mask_acx", "ssa_mask_acy",
        "c_bed", "f_slide", "taud_acx", "taud_acy", "taul_int_acx", "taul_int_acy",
        "H_ice", "f_ice", "H_grnd", "f_grnd", "f_grnd_acx", "f_grnd_acy",
        "ATT", "zeta_aa", "z_sl", "z_bed", "z_srf")]


class Tuning(C.Structure):
    """ygpu_tuning."""
    _fields_ = [("check_every", C.c_int), ("use_graphs", C.c_int), ("unknowns_per_cta", C.c_int),
                ("max_active_unknowns", C.c_ulonglong), ("spin_log2", C.c_int), ("cluster_ctas", C.c_int)]


class ServerCfg(C.Structure):
    """ygpu_server_cfg."""
    _fields_ = [
        ("device", C.c_int), ("kind", C.c_int), ("par", DynPar),
        ("grad_lim", C.c_double), ("taud_lim", C.c_double), ("lateral_bc", C.c_int),
        ("dH_sigma", C.c_double), ("hbm_budget", C.c_ulonglong), ("max_slots", C.c_int),
        ("max_active_unknowns", C.c_ulonglong),
    ]


class ServerInfo(C.Structure):
    """ygpu_server_info."""
    _fields_ = [
        ("members", C.c_int), ("slots", C.c_int), ("active", C.c_int), ("pending", C.c_int),
        ("ticks", C.c_longlong), ("completed", C.c_longlong), ("bytes_held", C.c_ulonglong),
    ]


SRV_UX, SRV_UY, SRV_VISC, SRV_H, SRV_UXB, SRV_UYB = 0, 1, 2, 3, 4, 5
SRV_TAUBX, SRV_TAUBY, SRV_BETA, SRV_BETAX, SRV_BETAY = 6, 7, 8, 9, 10


# Argument names of calc_velocity_ssa (velocity_ssa.f90:60) and
# calc_velocity_diva (velocity_diva.f90:59), in order, with their C type.
SSA_ARGS = [
    ("ux_b", "d"), ("uy_b", "d"), ("taub_acx", "d"), ("taub_acy", "d"),
    ("visc_eff", "d"), ("visc_eff_int", "d"), ("ssa_mask_acx", "i"), ("ssa_mask_acy", "i"),
    ("ssa_err_acx", "d"), ("ssa_err_acy", "d"),
    ("ssa_iter_now", "s"), ("ssa_lin_iter", "s"), ("ssa_lin_fail", "s"), ("ssa_lim_n", "s"),
    ("beta", "d"), ("beta_acx", "d"), ("beta_acy", "d"), ("c_bed", "d"), ("f_slide", "d"),
    ("taud_acx", "d"), ("taud_acy", "d"), ("taul_int_acx", "d"), ("taul_int_acy", "d"),
    ("H_ice", "d"), ("f_ice", "d"), ("H_grnd", "d"), ("f_grnd", "d"),
    ("f_grnd_acx", "d"), ("f_grnd_acy", "d"), ("ATT", "d"), ("zeta_aa", "d"),
    ("z_sl", "d"), ("z_bed", "d"), ("z_srf", "d"),
]
DIVA_ARGS = [
    ("ux", "d"), ("uy", "d"), ("ux_bar", "d"), ("uy_bar", "d"),
    ("ux_b", "d"), ("uy_b", "d"), ("ux_i", "d"), ("uy_i", "d"),
    ("taub_acx", "d"), ("taub_acy", "d"),
    ("beta", "d"), ("beta_acx", "d"), ("beta_acy", "d"), ("beta_eff", "d"),
    ("visc_eff", "d"), ("visc_eff_int", "d"), ("duxdz", "d"), ("duydz", "d"),
    ("ssa_mask_acx", "i"), ("ssa_mask_acy", "i"), ("ssa_err_acx", "d"), ("ssa_err_acy", "d"),
    ("ssa_iter_now", "s"), ("ssa_lin_iter", "s"), ("ssa_lin_fail", "s"), ("ssa_lim_n", "s"),
    ("c_bed", "d"), ("f_slide", "d"),
    ("taud_acx", "d"), ("taud_acy", "d"), ("taul_int_acx", "d"), ("taul_int_acy", "d"),
    ("H_ice", "d"), ("f_ice", "d"), ("H_grnd", "d"), ("f_grnd", "d"),
    ("f_grnd_acx", "d"), ("f_grnd_acy", "d"), ("ATT", "d"), ("zeta_aa", "d"),
    ("z_sl", "d"), ("z_bed", "d"), ("z_srf", "d"),
]
INPUT_ARGS = [
    ("H_ice", "d"), ("z_bed", "d"), ("z_sl", "d"),
    ("f_ice", "d"), ("H_grnd", "d"), ("z_srf", "d"), ("f_grnd", "d"), ("f_grnd_acx", "d"),
    ("f_grnd_acy", "d"), ("mask_frnt", "i"), ("dzsdx", "d"), ("dzsdy", "d"),
    ("taud_acx", "d"), ("taud_acy", "d"), ("taul_int_acx", "d"), ("taul_int_acy", "d"),
]


def _ctype(t):
    return {"d": _dp, "i": _ip, "s": _ip}[t]


def declare_velocity(fn, args):
    fn.argtypes = [_ctype(t) for _, t in args] + [
        C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(DynPar)]
    fn.restype = C.c_int


def declare_inputs(fn, bg: bool = False):
    """ygpu_calc_dyn_inputs (bg: ygpu_calc_dyn_inputs_bg, two background slopes more)."""
    fn.argtypes = [_ctype(t) for _, t in INPUT_ARGS] + [C.c_double] * (8 if bg else 6) + [C.c_int] * 3
    fn.restype = C.c_int


def declare_masks(fn):
    fn.argtypes = [_ip, _ip, _ip, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_int]
    fn.restype = C.c_int


def ptr(a: np.ndarray, kind: str):
    """Pointer to a Fortran-ordered array (checked dtype and contiguity)."""
    want = np.float64 if kind == "d" else np.int32
    if a.dtype != want:
        raise TypeError(f"array of dtype {a.dtype}, expected {want}")
    if not (a.flags.f_contiguous or a.ndim <= 1):
        raise TypeError("arrays must be Fortran-contiguous (column-major, x fastest)")
    return a.ctypes.data_as(_dp if kind == "d" else _ip)


# neff_hook of calc_velocity_diva: (user, c_bed in/out, ux_b, uy_b, nx, ny)
NEFF_HOOK = C.CFUNCTYPE(None, C.c_void_p, _dp, _dp, _dp, C.c_int, C.c_int)


def neff_hook(fn):
    """Wrap fn(c_bed, ux_b, uy_b) -- (nx, ny) Fortran-ordered views, c_bed
    updated in place -- as a C callback (keep the result alive during the call)."""
    def _cb(user, cb, ub, vb, nx, ny):
        n = nx * ny
        view = lambda p: np.ctypeslib.as_array(p, shape=(n,)).reshape((nx, ny), order="F")
        fn(view(cb), view(ub), view(vb))
    return NEFF_HOOK(_cb)


def call_velocity(fn, args, fields: dict, dx, dy, n_glen, par: DynPar, extra=()):
    """Call a calc_velocity_* style entry with a dict of named numpy arrays.

    Scalars ssa_iter_now etc. are returned in a dict; arrays are updated in place.
    `extra` arguments are appended after the parameters.
    """
    nx, ny = fields["H_ice"].shape
    nz = fields["zeta_aa"].shape[0]
    scal = {n: C.c_int(0) for n, t in args if t == "s"}
    cargs = []
    for n, t in args:
        if t == "s":
            cargs.append(C.pointer(scal[n]))
        else:
            cargs.append(ptr(fields[n], t))
    st = fn(*cargs, C.c_double(dx), C.c_double(dy), C.c_double(n_glen),
            C.c_int(nx), C.c_int(ny), C.c_int(nz), C.byref(par), *extra)
    out = {n: v.value for n, v in scal.items()}
    out["status"] = int(st)
    return out


def call_inputs(fn, fields: dict, dx, grad_lim, taud_lim, rho_ice, rho_sw, g, bc, slope_bg=None):
    """Call ygpu_calc_dyn_inputs, or the _bg entry with slope_bg = (slope_bg_x, slope_bg_y)."""
    nx, ny = fields["H_ice"].shape
    cargs = [ptr(fields[n], t) for n, t in INPUT_ARGS]
    bg = () if slope_bg is None else (C.c_double(slope_bg[0]), C.c_double(slope_bg[1]))
    return int(fn(*cargs, C.c_double(dx), C.c_double(grad_lim), C.c_double(taud_lim),
                  C.c_double(rho_ice), C.c_double(rho_sw), C.c_double(g), *bg,
                  C.c_int(bc), C.c_int(nx), C.c_int(ny)))
