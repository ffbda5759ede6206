"""The converged oracle solve against the reference's analytic benchmark A2.

A2 radial floating shelf (docs/dev/benchmark-protocol/index.md:70-86,
tests/bench/src/shelf.jl): u = e x, v = e y with e = A S^3 / 9. The reference
matches it to ~0.07 % rms at dx = 10 km (index.md:270); the oracle must too.
"""
import numpy as np
import pytest

import oracle
from yelmo_gb300 import configs


@pytest.mark.parametrize("ssa_solver,lis", [
    ("energy", "-i cg -p jacobi -maxiter 4000 -tol 1.0e-10"),
    ("residual", "-i bicgstab -p ilu -maxiter 4000 -tol 1.0e-10"),
    ("energy", "-i minres -p jacobi -maxiter 4000 -tol 1.0e-10"),
])
def test_radial_shelf_matches_analytic(ssa_solver, lis):
    inst = configs.radial_shelf(dx_km=10.0)
    inputs = oracle.calc_dyn_inputs(inst)
    f = configs.shelf_state(inst, inputs)
    f["ssa_mask_acx"], f["ssa_mask_acy"] = oracle.set_ssa_masks(
        inputs["mask_frnt"], inputs["f_ice"], inputs["f_grnd"], "marine", "zeros")
    par = inst.par.with_(ssa_solver=ssa_solver, ssa_iter_max=100, ssa_iter_conv=1e-7,
                         ssa_lis_opt_energy=lis, ssa_lis_opt_residual=lis)
    out = oracle.calc_velocity(f, inst, par)
    # The first Picard iterations of a free-floating shelf are nearly singular
    # (beta_reg = 1e-3); the residual form may break down there, the last solve may not.
    assert out["status"] == 0
    if ssa_solver == "energy":
        assert out["ssa_lin_fail"] == 0
    xc, e, dx = inst.extra["xc"], inst.extra["strain_rate"], inst.dx
    ux_ex = e * (xc + dx / 2)[:, None] * np.ones((1, len(xc)))
    uy_ex = e * (xc + dx / 2)[None, :] * np.ones((len(xc), 1))
    mx, my = f["ssa_mask_acx"] > 0, f["ssa_mask_acy"] > 0
    num = np.concatenate([(f["ux_bar"] - ux_ex)[mx], (f["uy_bar"] - uy_ex)[my]])
    den = np.concatenate([ux_ex[mx], uy_ex[my]])
    rms = np.sqrt(np.mean(num ** 2)) / np.sqrt(np.mean(den ** 2))
    assert rms < 2e-3, rms
