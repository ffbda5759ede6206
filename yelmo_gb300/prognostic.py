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
oracle's functions to compare the two loops step by step). ``run_device`` is the
same loop with every field resident on the GPU: the device entry points of the
library on one context stream, and the thickness update as a torch operation
on that stream; only max |dH/dt| and the statuses come back to the host.
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


def run_device(inst, dt: float, t_end: float, device: int = 0, dhdt_tol: float = 0.0,
               tuning: dict | None = None) -> dict:
    """``run`` with the fields on the GPU (device tensors, no host staging per step):
    ygpu_advec2D_impl_lis_device, the thickness update, ygpu_calc_dyn_inputs_bg_device,
    ygpu_set_ssa_masks_device and ygpu_solve_device on one context's stream. Returns
    what ``run`` returns, without the solve's field dict ("fields"). tuning: keyword
    arguments of DeviceSolver.set_tuning for the context (None: its defaults)."""
    import ctypes as C

    import torch

    from . import abi
    p = inst.par
    nx, ny, nz = inst.nx, inst.ny, inst.nz
    dev_name = f"cuda:{device}"
    st = dataclasses.replace(inst, H_ice=np.array(inst.H_ice, dtype=np.float64, order="F", copy=True))
    d = gpu.to_device(gpu.prepare(st), dev_name)
    z2 = lambda: torch.zeros(nx * ny, dtype=torch.float64, device=dev_name)
    dzsdx, dzsdy, dvdt, smb = z2(), z2(), z2(), z2()
    mask_ice = torch.full((nx * ny,), 2, dtype=torch.int32, device=dev_name)       # MASK_ICE_DYNAMIC
    solver = gpu.DeviceSolver(device)
    if tuning:
        solver.set_tuning(**tuning)
    L = solver.L
    ptr = lambda k: C.c_void_p(d[k].data_ptr())
    try:
        stream = torch.cuda.ExternalStream(L.ygpu_ctx_stream(solver.ctx), device=dev_name)
        fields = gpu.make_fields(d, nx, ny, nz, st.dx, st.dx, st.n_glen)
        bc = abi.BOUNDARY_CODES[p.boundaries]
        latbc = abi.LATBC_CODES[p.ssa_lat_bc]
        sbx, sby = (float(v) for v in st.slope_bg)
        torch.cuda.synchronize(dev_name)
        solver.solve(p.kind, p, fields)
        n_steps = int(np.ceil(t_end / dt - 1e-9))
        hist = {"dhdt_max": [], "picard": [], "adv_iter": []}
        it, ls = C.c_int(0), C.c_int(0)
        t, k = 0.0, 0
        for k in range(1, n_steps + 1):
            gpu._check(L.ygpu_advec2D_impl_lis_device(
                solver.ctx, C.c_void_p(dvdt.data_ptr()), ptr("H_ice"), ptr("ux_bar"), ptr("uy_bar"),
                C.c_void_p(smb.data_ptr()), C.c_void_p(mask_ice.data_ptr()), ptr("H_ice"), st.dx, st.dx, dt,
                abi.ADV_BOUNDARY_CODES[p.boundaries], nx, ny, C.byref(it), C.byref(ls)))
            if ls.value != 0:
                raise RuntimeError(f"advection linear solve failed at step {k} (status {ls.value})")
            with torch.cuda.stream(stream):
                d["H_ice"].add_(dvdt, alpha=dt)
                m = dvdt.abs().max()
            gpu._check(L.ygpu_calc_dyn_inputs_bg_device(
                solver.ctx, ptr("H_ice"), ptr("z_bed"), ptr("z_sl"), ptr("f_ice"), ptr("H_grnd"), ptr("z_srf"),
                ptr("f_grnd"), ptr("f_grnd_acx"), ptr("f_grnd_acy"), ptr("mask_frnt"),
                C.c_void_p(dzsdx.data_ptr()), C.c_void_p(dzsdy.data_ptr()), ptr("taud_acx"), ptr("taud_acy"),
                ptr("taul_int_acx"), ptr("taul_int_acy"), st.dx, p.grad_lim, p.taud_lim, p.rho_ice, p.rho_sw,
                p.g, sbx, sby, bc, nx, ny))
            gpu._check(L.ygpu_set_ssa_masks_device(solver.ctx, ptr("ssa_mask_acx"), ptr("ssa_mask_acy"),
                                                   ptr("mask_frnt"), ptr("f_ice"), ptr("f_grnd"), latbc, bc,
                                                   nx, ny))
            out = solver.solve(p.kind, p, fields)
            if out["status"] != 0:
                raise RuntimeError(f"velocity solve failed at step {k} (status {out['status']})")
            t = k * dt
            mv = float(m.item())
            hist["dhdt_max"].append(mv)
            hist["picard"].append(out["ssa_iter_now"])
            hist["adv_iter"].append(it.value)
            if not np.isfinite(mv):
                raise RuntimeError(f"thickness diverged at step {k} (t = {t} a): reduce dt")
            if dhdt_tol > 0.0 and mv < dhdt_tol:
                break
        torch.cuda.synchronize(dev_name)
        host = lambda key, shape: d[key].cpu().numpy().reshape(shape, order="F")
        ux = host("ux", (nx, ny, nz))
        uy = host("uy", (nx, ny, nz))
        ux_s, uy_s = np.asfortranarray(ux[:, :, -1]), np.asfortranarray(uy[:, :, -1])
        return {"t": t, "steps": k, "H_ice": host("H_ice", (nx, ny)), "z_srf": host("z_srf", (nx, ny)),
                "ux_bar": host("ux_bar", (nx, ny)), "uy_bar": host("uy_bar", (nx, ny)), "ux_s": ux_s,
                "uy_s": uy_s, "us_aa": surface_speed_aa(ux_s, uy_s),
                "history": {kk: np.asarray(v) for kk, v in hist.items()}}
    finally:
        solver.close()
