"""Synthetic velocity-solve workloads (seeded, platform independent).

Each builder returns an ``Instance``: the raw fields a Yelmo run would hold
before calc_ydyn (ice thickness, bed, sea level, rate factor, friction inputs,
sigma grid) plus the solver parameters. ``Instance.state()`` allocates the
INOUT fields of calc_velocity_ssa / calc_velocity_diva at their cold-start
values (ydyn_alloc, src/yelmo_dynamics.f90:1165: visc_eff = 1e3, velocities 0).
The fields that calc_ydyn derives before the solve (masks, flotation,
driving and lateral stress) come from ``ygpu_calc_dyn_inputs`` (GPU) or the
oracle's restatement of it.

Workloads (sizes as the benchmark definitions):
  dome_ssa        81x81, dx 16 km, grounded dome, imposed beta     (SSA, residual, BiCGSTAB+ILU0)
  marine_diva     161x161, dx 8 km, nz 10, marine dome with rough bed (DIVA)
  ensemble_member side n in {41,81,121,161}, 1280 km domain          (batched SSA)
  continent_diva  801x801, dx 4 km, nz 20, spectral bed, power-law friction (DIVA)
Any builder takes ``n`` to scale the grid for tests.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .params import YdynParams

T0 = 273.15

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n outputs of the splitmix64 generator started at ``seed`` (uint64)."""
    with np.errstate(over="ignore"):
        s = np.uint64(seed) + np.uint64(0x9E3779B97F4A7C15) * np.arange(1, n + 1, dtype=np.uint64)
        z = s
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed: int, n: int) -> np.ndarray:
    """Uniform doubles in (0, 1) from the top 53 bits of splitmix64."""
    return ((splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 2.0**53)


def normal(seed: int, n: int) -> np.ndarray:
    """Standard normal deviates (Box-Muller on splitmix64 uniforms)."""
    m = (n + 1) // 2
    u = uniform01(seed, 2 * m)
    r = np.sqrt(-2.0 * np.log(u[:m]))
    t = 2.0 * np.pi * u[m:]
    return np.concatenate([r * np.cos(t), r * np.sin(t)])[:n]


def gaussian_field(nx, ny, dx, sigma, ell, seed):
    """Gaussian-correlated noise: white noise filtered with exp(-(r/ell)^2), std sigma."""
    w = normal(seed, nx * ny).reshape((nx, ny), order="F")
    kx = np.fft.fftfreq(nx, d=dx) * 2.0 * np.pi
    ky = np.fft.fftfreq(ny, d=dx) * 2.0 * np.pi
    k2 = kx[:, None] ** 2 + ky[None, :] ** 2
    f = np.real(np.fft.ifft2(np.fft.fft2(w) * np.exp(-k2 * ell * ell / 4.0)))
    f = f - f.mean()
    sd = f.std()
    return np.asfortranarray(f * (sigma / sd if sd > 0 else 0.0))


def spectral_field(nx, ny, dx, rms, mean, seed, slope=-2.0):
    """Noise with power spectrum ~ k^slope, given rms and mean."""
    w = normal(seed, nx * ny).reshape((nx, ny), order="F")
    kx = np.fft.fftfreq(nx, d=dx)
    ky = np.fft.fftfreq(ny, d=dx)
    k = np.sqrt(kx[:, None] ** 2 + ky[None, :] ** 2)
    k[0, 0] = np.inf
    f = np.real(np.fft.ifft2(np.fft.fft2(w) * k ** (slope / 2.0)))
    f = f - f.mean()
    return np.asfortranarray(mean + f * (rms / f.std()))


def calc_zeta(nz: int, scale: str = "exp", zeta_exp: float = 2.0) -> np.ndarray:
    """zeta_aa of calc_zeta (yelmo_grid.f90:41-121)."""
    z = np.array([k / (nz - 1) for k in range(nz)], dtype=np.float64)
    if scale == "exp":
        z = z ** zeta_exp
    elif scale == "exp-inv":
        z = (1.0 - z ** zeta_exp)[::-1].copy()
    elif scale == "tanh":
        z = np.tanh(np.pi * (z - 0.5))
        z = z - z.min()
        z = z / z.max()
    return z


def rate_factor(T_ice, T_pmp, enh=1.0):
    """calc_rate_factor (deformation.f90:305-341), Kelvin, n = 3."""
    Tp = np.clip(T_ice - T_pmp + T0, 220.0, T0)
    A1 = enh * 1.25671e-05 * np.exp(-60.0e3 / (8.314 * Tp))
    A2 = enh * 6.0422976e10 * np.exp(-139.0e3 / (8.314 * Tp))
    return np.where(Tp <= 263.15, A1, A2)


def _F(a):
    return np.asfortranarray(a, dtype=np.float64)


@dataclass
class Instance:
    """Raw fields of one velocity solve (Fortran-ordered numpy arrays)."""
    name: str
    par: YdynParams
    dx: float
    H_ice: np.ndarray
    z_bed: np.ndarray
    z_sl: np.ndarray
    ATT: np.ndarray
    zeta_aa: np.ndarray
    beta: np.ndarray          # imposed beta on aa-nodes (beta_method = -1), else zeros
    c_bed: np.ndarray
    f_slide: np.ndarray
    n_glen: float = 3.0
    extra: dict = field(default_factory=dict)
    # uniform background slope (ytopo slope_bg_x, slope_bg_y) not contained in z_bed
    slope_bg: tuple = (0.0, 0.0)

    @property
    def nx(self):
        return self.H_ice.shape[0]

    @property
    def ny(self):
        return self.H_ice.shape[1]

    @property
    def nz(self):
        return self.zeta_aa.shape[0]

    def input_buffers(self) -> dict:
        """Empty output buffers of ygpu_calc_dyn_inputs, plus the three inputs."""
        s2 = (self.nx, self.ny)
        d = {k: np.zeros(s2, order="F") for k in (
            "f_ice", "H_grnd", "z_srf", "f_grnd", "f_grnd_acx", "f_grnd_acy", "dzsdx", "dzsdy",
            "taud_acx", "taud_acy", "taul_int_acx", "taul_int_acy")}
        d["mask_frnt"] = np.zeros(s2, dtype=np.int32, order="F")
        d["H_ice"], d["z_bed"], d["z_sl"] = self.H_ice, self.z_bed, self.z_sl
        return d

    def state(self, inputs: dict) -> dict:
        """All arrays of one calc_velocity_* call, cold start, given the prologue fields."""
        s2, s3 = (self.nx, self.ny), (self.nx, self.ny, self.nz)
        f = {}
        for k in ("ux_b", "uy_b", "ux_bar", "uy_bar", "taub_acx", "taub_acy", "visc_eff_int",
                  "ssa_err_acx", "ssa_err_acy", "beta_acx", "beta_acy", "beta_eff"):
            f[k] = np.zeros(s2, order="F")
        for k in ("ux", "uy", "ux_i", "uy_i", "duxdz", "duydz"):
            f[k] = np.zeros(s3, order="F")
        f["visc_eff"] = np.full(s3, 1e3, order="F")
        f["beta"] = _F(self.beta.copy())
        f["ssa_mask_acx"] = np.zeros(s2, dtype=np.int32, order="F")
        f["ssa_mask_acy"] = np.zeros(s2, dtype=np.int32, order="F")
        for k in ("c_bed", "f_slide", "H_ice", "z_bed", "z_sl", "ATT", "zeta_aa"):
            f[k] = getattr(self, k)
        for k in ("taud_acx", "taud_acy", "taul_int_acx", "taul_int_acy", "f_ice", "H_grnd",
                  "f_grnd", "f_grnd_acx", "f_grnd_acy", "z_srf", "mask_frnt"):
            f[k] = inputs[k]
        return f


def _lin(lo, hi, n):
    return np.array([lo + (hi - lo) * i / (n - 1) for i in range(n)])


def dome_ssa(n: int = 81, seed: int = 1234, nz: int = 10) -> Instance:
    """Plain single SSA solve: grounded dome on a flat bed, imposed beta."""
    dx = 16e3 * 80.0 / (n - 1)
    x = (np.arange(n) - (n - 1) / 2.0) * dx
    r = np.sqrt(x[:, None] ** 2 + x[None, :] ** 2)
    H = 3000.0 * np.sqrt(np.maximum(0.0, 1.0 - (r / 600e3) ** 2))
    u = uniform01(seed, n * n).reshape((n, n), order="F")
    beta = 10.0 ** (2.0 + 2.0 * u)            # log-uniform in [1e2, 1e4]
    zeta = calc_zeta(nz)
    par = YdynParams(
        solver="ssa", ssa_solver="residual", visc_method=1, beta_method=-1, beta_gl_stag=1,
        ssa_iter_max=50, ssa_iter_conv=1e-4,
        ssa_lis_opt_residual="-i bicgstab -p ilu -maxiter 1000 -tol 1.0e-8 -initx_zeros false",
        boundaries="zeros")
    return Instance("dome_ssa", par, dx, _F(H), _F(np.zeros((n, n))), _F(np.zeros((n, n))),
                    _F(np.full((n, n, nz), 1e-16)), zeta, _F(beta), _F(np.zeros((n, n))),
                    _F(np.ones((n, n))))


def _marine_geometry(n, dx, seed):
    x = (np.arange(n) - (n - 1) / 2.0) * dx
    r = np.sqrt(x[:, None] ** 2 + x[None, :] ** 2)
    L = (n - 1) * dx
    bed = 200.0 - 1000.0 * (x[:, None] - x[0]) / L + np.zeros((1, n))
    bed = bed + gaussian_field(n, n, dx, 100.0, 40e3, seed)
    H = 3500.0 * np.sqrt(np.maximum(0.0, 1.0 - (r / 700e3) ** 2))
    H = np.where(r > 600e3, 0.0, H)
    return _F(H), _F(bed)


def _temperature_att(H, zeta, Ts=-30.0, Tb=-2.0):
    """A(T) with T linear in depth from Ts (surface) to Tb (base), homologous."""
    T = Tb + (Ts - Tb) * zeta[None, None, :] + 0.0 * H[:, :, None]
    return _F(rate_factor(T0 + T, T0))


def marine_diva(n: int = 161, seed: int = 2024, nz: int = 10) -> Instance:
    """Marine single DIVA solve: dome over a seaward-deepening rough bed."""
    dx = 8e3 * 160.0 / (n - 1)
    H, bed = _marine_geometry(n, dx, seed)
    zeta = calc_zeta(nz)
    ATT = _temperature_att(H, zeta)
    u = uniform01(seed + 7, n * n).reshape((n, n), order="F")
    beta = 10.0 ** (2.0 + 2.0 * u)
    floating = H < -(1028.0 / 910.0) * bed
    beta = np.where(floating, 0.0, beta)
    par = YdynParams(solver="diva", ssa_solver="energy", beta_method=-1, beta_gl_stag=1)
    return Instance("marine_diva", par, dx, H, bed, _F(np.zeros((n, n))), ATT, zeta, _F(beta),
                    _F(np.zeros((n, n))), _F(np.ones((n, n))))


def ensemble_member(i: int, seed: int = 77, nz: int = 10, sides=(41, 81, 121, 161)) -> Instance:
    """Member i of the batched ensemble: side drawn from ``sides``, 1280 km domain, SSA."""
    side = int(sides[int(uniform01(seed + i, 1)[0] * len(sides)) % len(sides)])
    dx = 1280e3 / (side - 1)
    H, bed = _marine_geometry(side, dx, seed + i)
    zeta = calc_zeta(nz)
    ATT = _temperature_att(H, zeta)
    u = uniform01(seed + 1000 + i, side * side).reshape((side, side), order="F")
    beta = np.where(H < -(1028.0 / 910.0) * bed, 0.0, 10.0 ** (2.0 + 2.0 * u))
    par = YdynParams(solver="ssa", ssa_solver="energy", beta_method=-1, beta_gl_stag=1)
    return Instance(f"ensemble_{i}", par, dx, H, bed, _F(np.zeros((side, side))), ATT, zeta,
                    _F(beta), _F(np.zeros((side, side))), _F(np.ones((side, side))))


def served_member(i: int, seed: int = 99, nz: int = 10, lo: int = 64, hi: int = 321) -> Instance:
    """Member i of the served ensemble stream: side uniform in [lo, hi], 1280 km
    domain, geometry, roughness and friction as the batched ensemble, SSA."""
    side = lo + int(uniform01(seed + i, 1)[0] * (hi - lo + 1))
    side = min(max(side, lo), hi)
    dx = 1280e3 / (side - 1)
    H, bed = _marine_geometry(side, dx, seed + i)
    zeta = calc_zeta(nz)
    ATT = _temperature_att(H, zeta)
    u = uniform01(seed + 1000 + i, side * side).reshape((side, side), order="F")
    beta = np.where(H < -(1028.0 / 910.0) * bed, 0.0, 10.0 ** (2.0 + 2.0 * u))
    par = YdynParams(solver="ssa", ssa_solver="energy", beta_method=-1, beta_gl_stag=1)
    return Instance(f"served_{i}", par, dx, H, bed, _F(np.zeros((side, side))), ATT, zeta,
                    _F(beta), _F(np.zeros((side, side))), _F(np.ones((side, side))))


def continent_diva(n: int = 801, seed: int = 4242, nz: int = 20) -> Instance:
    """Large DIVA solve: spectral bed (k^-2, rms 600 m, mean -200 m), twelve
    seeded domes (3000 m, radii 5-11 % of the domain) over a 300 m ice sheet
    inside 45 % of the domain radius, capped at 4000 m. About 30 % of the ice
    floats (28.5 % at 801 x 801). Power-law friction, q = 1/3."""
    dx = 4e3 * 800.0 / (n - 1)
    bed = spectral_field(n, n, dx, 600.0, -200.0, seed)
    x = (np.arange(n) - (n - 1) / 2.0) * dx
    H = np.zeros((n, n))
    cen = uniform01(seed + 1, 24).reshape(12, 2)
    rad = uniform01(seed + 2, 12)
    L = (n - 1) * dx
    for (cx, cy), rr in zip(cen, rad):
        x0, y0, R = (cx - 0.5) * 0.6 * L, (cy - 0.5) * 0.6 * L, (0.05 + 0.06 * rr) * L
        d = np.sqrt((x[:, None] - x0) ** 2 + (x[None, :] - y0) ** 2)
        H = H + 3000.0 * np.sqrt(np.maximum(0.0, 1.0 - (d / R) ** 2))
    r = np.sqrt(x[:, None] ** 2 + x[None, :] ** 2)
    H = np.where(r < 0.45 * L, np.maximum(H, 300.0), H)
    H = np.minimum(H, 4000.0)
    zeta = calc_zeta(nz)
    ATT = _temperature_att(H, zeta, Ts=-25.0, Tb=-1.0)
    cb = 1e4 * 10.0 ** (uniform01(seed + 3, n * n).reshape((n, n), order="F") - 0.5)
    par = YdynParams(solver="diva", ssa_solver="energy", beta_method=2, beta_q=1.0 / 3.0,
                     beta_u0=100.0, beta_gl_stag=1)
    return Instance("continent_diva", par, dx, _F(H), _F(bed), _F(np.zeros((n, n))), ATT, zeta,
                    _F(np.zeros((n, n))), _F(cb), _F(np.ones((n, n))))


BUILDERS = {
    "dome_ssa": dome_ssa,
    "marine_diva": marine_diva,
    "continent_diva": continent_diva,
}


def radial_shelf(dx_km: float = 10.0, H: float = 400.0, R_s: float = 300e3, L: float = 400e3,
                 A: float = 1e-18, beta_reg: float = 1e-3, z_bed: float = -2000.0,
                 nz: int = 10) -> Instance:
    """A2 radial floating shelf (docs/dev/benchmark-protocol, tests/bench/src/shelf.jl):
    constant thickness H inside r < R_s on [-L, L]^2, uniform imposed friction beta_reg,
    par/yelmo_bench_SHELF-R.nml settings (beta_method = beta_gl_stag = -1, lat bc "marine").
    Exact solution: u = e x, v = e y, e = A S^n 3^(-(n+1)/2), S = rho_i g H (1 - rho_i/rho_w)/2."""
    dx = dx_km * 1e3
    n = int(round(2 * L / dx))
    xc = -L + dx / 2 + dx * np.arange(n)
    r = np.sqrt(xc[:, None] ** 2 + xc[None, :] ** 2)
    Hf = np.where(r < R_s, H, 0.0)
    zeta = calc_zeta(nz)
    par = YdynParams(solver="diva", ssa_solver="energy", beta_method=-1, beta_gl_stag=-1,
                     ssa_lat_bc="marine")
    inst = Instance("radial_shelf", par, dx, _F(Hf), _F(np.full((n, n), z_bed)), _F(np.zeros((n, n))),
                    _F(np.full((n, n, nz), A)), zeta, _F(np.full((n, n), beta_reg)),
                    _F(np.zeros((n, n))), _F(np.ones((n, n))))
    S = 0.5 * par.rho_ice * par.g * H * (1.0 - par.rho_ice / par.rho_sw)
    inst.extra = {"xc": xc, "strain_rate": A * S ** 3 * 3.0 ** (-2.0), "beta_reg": beta_reg}
    return inst


def schoof_slab_u(y, alpha: float, H0: float, A: float, W: float, m: float, rho_ice: float, g: float):
    """Schoof (2006) ice stream on a plastic bed, n = 3 (tests/yelmo_trough.f90:1349-1400):
    till yield stress tau_c = f |y/L|^m, f = rho g H alpha, L = W / (1+m)^(1/m), and the
    along-stream velocity u(y), zero for |y| > W. Returns (u, tau_c)."""
    y = np.asarray(y, dtype=np.float64)
    f = rho_ice * g * H0 * alpha
    B = A ** (-1.0 / 3.0)
    L = W / (1.0 + m) ** (1.0 / m)
    s = np.abs(y / L)
    m1 = m + 1.0
    bracket = ((y / L) ** 4 - m1 ** (4.0 / m)) / 4.0 \
        - 3.0 * (s ** (m + 4.0) - m1 ** (1.0 + 4.0 / m)) / (m1 * (m + 4.0)) \
        + 3.0 * (s ** (2.0 * m + 4.0) - m1 ** (2.0 + 4.0 / m)) / (m1 ** 2 * (2.0 * m + 4.0)) \
        - (s ** (3.0 * m + 4.0) - m1 ** (3.0 + 4.0 / m)) / (m1 ** 3 * (3.0 * m + 4.0))
    u = -2.0 * f ** 3 * L ** 4 / (B ** 3 * H0 ** 3) * bracket
    u = np.where(np.abs(y) > W, 0.0, u)
    return u, f * s ** m


def schoof_slab(dx_km: float = 2.0, lx: float = 100e3, ly: float = 80e3, alpha: float = 1e-3,
                H0: float = 1000.0, W: float = 25e3, m: float = 1.55, A: float = 1e-16,
                nz: int = 5) -> Instance:
    """Schoof (2006) slab (the reference's SLAB-S06 domain, tests/yelmo_trough.f90:174-182,
    259-307, par/yelmo_SLAB-S06.nml): periodic in x and y, uniform thickness H0 on a bed
    sloping down in x by alpha, SSA (energy form, visc_method 2) on a plastic bed
    (beta_method 4, q = 0, u0 = 1 m/a) whose c_bed is the analytic till yield stress.
    The slope enters only the driving stress, as the reference's uniform background
    slope: slab_state sets taud_acx = -rho g H0 alpha (grounded, flowing towards +x)."""
    dx = dx_km * 1e3
    nx, ny = int(round(lx / dx)), int(round(ly / dx))
    y = -(ny // 2) * dx + dx * np.arange(ny)
    par = YdynParams(solver="ssa", ssa_solver="energy", visc_method=2, beta_method=4, beta_q=0.0,
                     beta_u0=1.0, beta_gl_scale=0, beta_gl_stag=0, beta_gl_f=1.0, beta_min=0.0,
                     eps_0=1e-6, boundaries="periodic", ssa_lat_bc="marine", ssa_vel_max=10000.0)
    u, tauc = schoof_slab_u(y, alpha, H0, A, W, m, par.rho_ice, par.g)
    c_bed = np.broadcast_to(tauc[None, :], (nx, ny))
    inst = Instance("schoof_slab", par, dx, _F(np.full((nx, ny), H0)), _F(np.full((nx, ny), 10000.0)),
                    _F(np.zeros((nx, ny))), _F(np.full((nx, ny, nz), A)), calc_zeta(nz),
                    _F(np.zeros((nx, ny))), _F(c_bed), _F(np.ones((nx, ny))))
    inst.extra = {"y": y, "u": u, "taud": par.rho_ice * par.g * H0 * alpha, "W": W}
    return inst


ISMIPHOM_A = 2.140373e-7       # [Pa-1 a-1] rate factor of experiment F (n = 1)


def ismiphom_f(exp: int = 1, dx_km: float = 2.5, L_km: float = 100.0, nz: int = 10,
               alpha_deg: float = 3.0, bump: float = 100.0, sigma: float = 10e3) -> Instance:
    """ISMIP-HOM experiment F (tests/yelmo_ismiphom.f90:59-77,149-186, par/yelmo_ISMIPHOM.nml):
    a slab of mean thickness 1000 m on a mean slope alpha over a Gaussian bed bump,
    periodic square domain of side L centred on the bump (x0 = -L/2, dx = L/40), DIVA
    with linear rheology (n = 1, A = 2.140373e-7 Pa-1 a-1), zero mass balance.
    exp 1 (F1): no slip (solver "diva-noslip"); exp 2 (F2): slip ratio 1, imposed
    beta = 1/(A H0) on the aa-nodes (beta_method -1). The inclined plane is the
    background slope slope_bg_x = -tan(alpha); z_srf starts at 0 and z_bed holds the
    periodic part, z_bed = -1000 + bump exp(-(x^2+y^2)/sigma^2). z_sl = -10000 keeps
    every cell grounded. bump = 0 gives the unperturbed slab, whose surface speed is
    A rho g tan(alpha) H0^2 (F1) and twice that (F2)."""
    if exp not in (1, 2):
        raise ValueError("exp is 1 (F1, no slip) or 2 (F2, slip ratio 1)")
    dx = dx_km * 1e3
    n = int(round(L_km / dx_km))
    x = -0.5 * L_km * 1e3 + dx * np.arange(n)
    r2 = x[:, None] ** 2 + x[None, :] ** 2
    z_bed = -1000.0 + bump * np.exp(-r2 / sigma ** 2)
    H = 0.0 - z_bed
    H0 = 1000.0
    beta = np.full((n, n), 1000.0 if exp == 1 else 1.0 / (ISMIPHOM_A * H0))
    par = YdynParams(solver="diva-noslip" if exp == 1 else "diva", visc_method=1, beta_method=-1,
                     beta_gl_scale=0, beta_gl_stag=1, beta_gl_f=1.0, beta_min=0.0, eps_0=1e-6,
                     ssa_solver="energy", ssa_lat_bc="marine", ssa_vel_max=10000.0, ssa_iter_max=100,
                     ssa_iter_rel=0.7, ssa_iter_conv=1e-5, taud_lim=1e6, grad_lim=0.5,
                     boundaries="periodic", rho_ice=910.0, rho_sw=1028.0, g=9.81)
    inst = Instance(f"ismiphom_f{exp}", par, dx, _F(H), _F(z_bed), _F(np.full((n, n), -10000.0)),
                    _F(np.full((n, n, nz), ISMIPHOM_A)), calc_zeta(nz, "linear"), _F(beta),
                    _F(np.zeros((n, n))), _F(np.ones((n, n))), n_glen=1.0,
                    slope_bg=(-np.tan(np.deg2rad(alpha_deg)), 0.0))
    tau = par.rho_ice * par.g * H0 * np.tan(np.deg2rad(alpha_deg))
    u_def = ISMIPHOM_A * tau * H0          # n = 1: 2A/(n+1) tau^n H0
    inst.extra = {"x": x, "exp": exp, "u_s_slab": u_def if exp == 1 else 2.0 * u_def}
    return inst


def slab_state(inst: Instance, inputs: dict) -> dict:
    """State of the Schoof slab: the driving stress of the background slope, and the
    analytic velocity as the start (as the reference initialises ux_b, ux_bar)."""
    f = inst.state(inputs)
    f["taud_acx"][:] = -inst.extra["taud"]
    f["taud_acy"][:] = 0.0
    u = np.broadcast_to(inst.extra["u"][None, :], (inst.nx, inst.ny))
    for k in ("ux_b", "ux_bar"):
        f[k][:] = u
    return f


def shelf_state(inst: Instance, inputs: dict) -> dict:
    """Cold state of the A2 shelf with the imposed staggered friction (beta_gl_stag = -1)."""
    f = inst.state(inputs)
    f["beta_acx"][:] = inst.extra["beta_reg"]
    f["beta_acy"][:] = inst.extra["beta_reg"]
    return f
