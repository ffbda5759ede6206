"""A thickness time loop around the drop-in velocity solve, for the inclined-plane
steady states (ISMIP-HOM experiment F, tests/yelmo_ismiphom.f90:149-186,241-260).

Each step does what Yelmo's time loop does for these cases (topography solver
"impl-lis", zero mass balance, every cell grounded and dynamic):

1. the implicit upwind advection of H_ice with the depth-averaged velocity
   (calc_advec2D "impl-lis", ``ygpu_calc_advec2D_impl_lis``), H_ice += dt dH/dt;
2. the fields calc_ydyn builds from H_ice and z_bed, with the background slope
   added to the surface gradient before the limit (``ygpu_calc_dyn_inputs_bg``,
   yelmo_topography.f90:1373-1374) and the SSA masks;
3. the DIVA velocity solve, warm-started from the previous step's velocity and
   viscosity (``ygpu_calc_velocity_diva``).

Before the first step the velocity is solved once on the initial geometry (the
reference's yelmo_update_equil with topo_fixed, tests/yelmo_ismiphom.f90:228).

Yelmo integrates in time with an adaptive predictor-corrector (AB-SAM with a PI42
controller); this loop takes fixed backward-Euler thickness steps with the velocity
of the previous step. The steady state of both is the one where div(u H) = 0 for
the velocity of that H, which depends on the spatial discretisation only. The
lagged velocity makes the surface relaxation explicit, so dt must stay below
about dx^2 / (4 D), D ~ 2 A rho g H^3 / 3 the slab's diffusivity (about 1 a at
dx = 2.5 km); ``run`` reports the largest |dH/dt| of each step so a diverging
choice shows.

The calls go through a backend: the GPU library by default (``GpuBackend``).
Any object with the same four methods can stand in for it (a test passes the
oracle's functions to compare the two loops step by step).
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import gpu

_PROLOGUE = ("taud_acx", "taud_acy", "taul_int_acx", "taul_int_acy", "f_ice", "H_grnd", "f_grnd",
             "f_grnd_acx", "f_grnd_acy", "z_srf", "mask_frnt")


class GpuBackend:
    """The drop-in GPU calls of one time step (host arrays)."""

    def inputs(self, inst) -> dict:
        return gpu.calc_dyn_inputs(inst)

    def masks(self, mask_frnt, f_ice, f_grnd, lateral_bc: str, boundaries: str):
        return gpu.set_ssa_masks(mask_frnt, f_ice, f_grnd, lateral_bc, boundaries)

    def velocity(self, fields: dict, inst) -> dict:
        return gpu.calc_velocity(fields, inst.dx, inst.n_glen, inst.par)

    def advect(self, H, ux, uy, smb, mask_ice, H_ref, dx, dt, boundaries: str):
        return gpu.calc_advec2D_impl_lis(H, ux, uy, smb, mask_ice, H_ref, dx, dx, dt, boundaries)


def surface_speed_aa(ux_s: np.ndarray, uy_s: np.ndarray) -> np.ndarray:
    """|u_s| on the aa-nodes of a periodic grid: ux_s on the acx-nodes (i+1/2) and
    uy_s on the acy-nodes (j+1/2) averaged onto the cell centres."""
    uxa = 0.5 * (ux_s + np.roll(ux_s, 1, axis=0))
    uya = 0.5 * (uy_s + np.roll(uy_s, 1, axis=1))
    return np.sqrt(uxa ** 2 + uya ** 2)


def _refresh(be, inst, f):
    inputs = be.inputs(inst)
    for k in _PROLOGUE:
        f[k] = inputs[k]
    f["ssa_mask_acx"], f["ssa_mask_acy"] = be.masks(inputs["mask_frnt"], inputs["f_ice"], inputs["f_grnd"],
                                                    inst.par.ssa_lat_bc, inst.par.boundaries)
    return inputs


def run(inst, dt: float, t_end: float, backend=None, dhdt_tol: float = 0.0, on_step=None) -> dict:
    """Integrate H_ice of ``inst`` (a copy; inst is not changed) from t = 0 to t_end
    in steps of dt [a], or until max |dH/dt| < dhdt_tol [m/a] (0: never).

    Returns the final state: t, steps, H_ice, z_srf, ux_bar, uy_bar, ux_s, uy_s (the
    top layer of the 3D velocity), us_aa (surface speed on the aa-nodes), the
    solve's fields, and per step max |dH/dt|, Picard iterations and the
    advection's linear iterations. on_step(step, t, fields, dHdt) is called after
    every step. A solve or an advection that fails raises (the library's status)."""
    be = backend or GpuBackend()
    st = dataclasses.replace(inst, H_ice=np.array(inst.H_ice, dtype=np.float64, order="F", copy=True))
    H = st.H_ice
    nx, ny = H.shape
    f = st.state(be.inputs(st))
    _refresh(be, st, f)
    be.velocity(f, st)
    mask_ice = np.full((nx, ny), 2, dtype=np.int32, order="F")     # MASK_ICE_DYNAMIC
    smb = np.zeros((nx, ny), order="F")
    n_steps = int(np.ceil(t_end / dt - 1e-9))
    hist = {"dhdt_max": [], "picard": [], "adv_iter": []}
    t, k = 0.0, 0
    for k in range(1, n_steps + 1):
        dHdt, it_adv, st_adv = be.advect(H, f["ux_bar"], f["uy_bar"], smb, mask_ice, H, st.dx, dt,
                                         st.par.boundaries)
        if st_adv != 0:
            raise RuntimeError(f"advection linear solve failed at step {k} (status {st_adv})")
        H += dt * dHdt
        t = k * dt
        _refresh(be, st, f)
        out = be.velocity(f, st)
        if out["status"] != 0:
            raise RuntimeError(f"velocity solve failed at step {k} (status {out['status']})")
        m = float(np.max(np.abs(dHdt)))
        hist["dhdt_max"].append(m)
        hist["picard"].append(out["ssa_iter_now"])
        hist["adv_iter"].append(it_adv)
        if on_step:
            on_step(k, t, f, dHdt)
        if not np.isfinite(m):
            raise RuntimeError(f"thickness diverged at step {k} (t = {t} a): reduce dt")
        if dhdt_tol > 0.0 and m < dhdt_tol:
            break
    ux_s, uy_s = f["ux"][:, :, -1].copy(order="F"), f["uy"][:, :, -1].copy(order="F")
    return {"t": t, "steps": k, "H_ice": H.copy(order="F"), "z_srf": f["z_srf"].copy(order="F"),
            "ux_bar": f["ux_bar"].copy(order="F"), "uy_bar": f["uy_bar"].copy(order="F"),
            "ux_s": ux_s, "uy_s": uy_s, "us_aa": surface_speed_aa(ux_s, uy_s), "fields": f,
            "history": {kk: np.asarray(v) for kk, v in hist.items()}}
