"""ydyn parameters of the velocity solve.

``YdynParams`` holds the &ydyn namelist keys that the SSA/DIVA solve reads
(input/yelmo_defaults.nml:140-172; copied into ssa_param_class /
diva_param_class at src/yelmo_dynamics.f90:472-502 and :597-628) plus the
physical constants of &Earth (input/yelmo_phys_const.nml). ``to_c()`` gives the
``ygpu_dyn_par`` struct of include/yelmo_gpu.h, with the LIS option string of
the chosen assembler parsed the way ``ygpu_parse_lis_opt`` does.
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace

from . import abi


def parse_lis_opt(opts: str) -> dict:
    """Parse "-i cg -p jacobi -maxiter 200 -tol 1.0e-2 -initx_zeros false"."""
    tok = opts.split()
    if len(tok) % 2:
        raise ValueError(f"bad LIS option string: {opts!r}")
    out = {}
    solvers = {"cg": abi.LIN_CG, "1": abi.LIN_CG, "bicgstab": abi.LIN_BICGSTAB, "3": abi.LIN_BICGSTAB,
               "minres": abi.LIN_MINRES, "5": abi.LIN_MINRES}
    pres = {"none": abi.PRE_NONE, "0": abi.PRE_NONE, "jacobi": abi.PRE_JACOBI, "1": abi.PRE_JACOBI,
            "ilu": abi.PRE_ILU0, "2": abi.PRE_ILU0}
    for k, v in zip(tok[::2], tok[1::2]):
        if k == "-i":
            if v not in solvers:
                raise ValueError(f"LIS solver {v!r} not supported")
            out["lin_solver"] = solvers[v]
        elif k == "-p":
            if v not in pres:
                raise ValueError(f"LIS preconditioner {v!r} not supported")
            out["lin_precond"] = pres[v]
        elif k == "-maxiter":
            out["lin_maxiter"] = int(v)
        elif k == "-tol":
            out["lin_tol"] = float(v)
        elif k == "-initx_zeros":
            out["lin_initx_zeros"] = int(v in ("true", "1"))
    return out


@dataclass
class YdynParams:
    solver: str = "diva"                 # "ssa" | "diva" | "diva-noslip"
    visc_method: int = 1
    visc_const: float = 1e7
    beta_method: int = 1
    beta_const: float = 1e3
    beta_q: float = 1.0
    beta_u0: float = 100.0
    beta_gl_scale: int = 0
    beta_gl_stag: int = 1
    beta_gl_f: float = 1.0
    H_grnd_lim: float = 500.0
    beta_min: float = 100.0
    eps_0: float = 1e-6
    ssa_solver: str = "energy"
    ssa_lis_opt_residual: str = "-i minres -p jacobi -maxiter 100 -tol 1.0e-2 -initx_zeros false"
    ssa_lis_opt_energy: str = "-i cg -p jacobi -maxiter 200 -tol 1.0e-2 -initx_zeros false"
    ssa_lat_bc: str = "all"
    ssa_vel_lim_method: str = "drag"
    ssa_vel_max: float = 10000.0
    ssa_vel_lim_tau: float = 1e5
    ssa_iter_max: int = 20
    ssa_iter_rel: float = 0.7
    ssa_iter_conv: float = 1e-2
    taud_lim: float = 2e5
    boundaries: str = "zeros"
    ssa_write_log: bool = False
    # &Earth constants
    rho_ice: float = 910.0
    rho_sw: float = 1028.0
    g: float = 9.81
    # ytopo
    grad_lim: float = 0.5
    # GPU solve only
    precision: str = "fp64"              # "fp64" | "mixed"
    inner_maxiter: int = 0
    inner_tol: float = 0.0

    def with_(self, **kw) -> "YdynParams":
        return replace(self, **kw)

    @property
    def kind(self) -> int:
        return abi.KIND_SSA if self.solver == "ssa" else abi.KIND_DIVA

    @property
    def lis_opt(self) -> str:
        return self.ssa_lis_opt_energy if self.ssa_solver == "energy" else self.ssa_lis_opt_residual

    def to_c(self) -> abi.DynPar:
        if self.boundaries not in abi.BOUNDARY_CODES:
            raise ValueError(f"boundaries {self.boundaries!r} not recognised")
        p = abi.DynPar()
        p.ssa_solver = abi.SSA_SOLVER_CODES[self.ssa_solver]
        p.boundaries = abi.BOUNDARY_CODES[self.boundaries]
        p.no_slip = int(self.solver == "diva-noslip")
        p.visc_method = self.visc_method
        p.visc_const = self.visc_const
        p.beta_method = self.beta_method
        p.beta_const = self.beta_const
        p.beta_q = self.beta_q
        p.beta_u0 = self.beta_u0
        p.beta_gl_scale = self.beta_gl_scale
        p.beta_gl_stag = self.beta_gl_stag
        p.beta_gl_f = self.beta_gl_f
        p.H_grnd_lim = self.H_grnd_lim
        p.beta_min = self.beta_min
        p.eps_0 = self.eps_0
        p.ssa_vel_lim_method = abi.VEL_LIM_CODES[self.ssa_vel_lim_method]
        p.ssa_vel_lim_tau = self.ssa_vel_lim_tau
        p.ssa_vel_max = self.ssa_vel_max
        p.ssa_iter_max = self.ssa_iter_max
        p.ssa_iter_rel = self.ssa_iter_rel
        p.ssa_iter_conv = self.ssa_iter_conv
        p.ssa_write_log = int(self.ssa_write_log)
        p.rho_ice, p.rho_sw, p.g = self.rho_ice, self.rho_sw, self.g
        p.lin_solver, p.lin_precond, p.lin_maxiter = abi.LIN_CG, abi.PRE_JACOBI, 200
        p.lin_tol, p.lin_initx_zeros = 1e-2, 0
        for k, v in parse_lis_opt(self.lis_opt).items():
            setattr(p, k, v)
        p.precision = abi.PREC_MIXED if self.precision == "mixed" else abi.PREC_FP64
        p.inner_maxiter = self.inner_maxiter
        p.inner_tol = self.inner_tol
        return p
