"""Schoof (2006) ice stream on a plastic bed: the reference's SLAB-S06 benchmark
(tests/yelmo_trough.f90:259-307, analytic solution :1349-1400, par/yelmo_SLAB-S06.nml).

A periodic slab of uniform thickness on a slope, SSA with the energy form and a
plastic bed (beta_method 4, q = 0) whose till yield stress is the analytic one.
The converged discrete solve approaches the analytic velocity as the grid is
refined (about second order: 8.7 % relative L2 at the reference's 2 km, 2.5 % at
1 km). CPU: the oracle against the analytic profile. GPU: FP64 and mixed solves
against the oracle (the parity bar, 1e-6 relative L2) and against the profile."""
import numpy as np
import pytest

import oracle
from tests.cases import rel_l2
from yelmo_gb300 import configs, gpu

TIGHT = dict(ssa_iter_max=300, ssa_iter_conv=1e-7, ssa_lis_opt_energy="-i cg -p jacobi -maxiter 5000 -tol 1e-9")


def _state(inst, prologue):
    inputs = prologue.calc_dyn_inputs(inst)
    f = configs.slab_state(inst, inputs)
    f["ssa_mask_acx"], f["ssa_mask_acy"] = prologue.set_ssa_masks(
        inputs["mask_frnt"], inputs["f_ice"], inputs["f_grnd"], inst.par.ssa_lat_bc, inst.par.boundaries)
    return f


def _err(inst, f):
    u = inst.extra["u"][None, :]
    return float(np.sqrt(np.mean((f["ux_b"] - u) ** 2)) / np.sqrt(np.mean(u ** 2)))


def test_analytic_profile():
    """Symmetric in y, zero outside the stream, the yield stress equal to the driving
    stress where |y| = L, and the centre speed of the closed form."""
    inst = configs.schoof_slab(dx_km=1.0)
    y, W = inst.extra["y"], inst.extra["W"]
    u, tauc = configs.schoof_slab_u(y, 1e-3, 1000.0, 1e-16, W, 1.55, inst.par.rho_ice, inst.par.g)
    np.testing.assert_array_equal(u[np.abs(y) > W], 0.0)
    inner = (np.abs(y) < W) & (y != 0)
    ym = y[inner]
    u2, _ = configs.schoof_slab_u(-ym, 1e-3, 1000.0, 1e-16, W, 1.55, inst.par.rho_ice, inst.par.g)
    np.testing.assert_allclose(u[inner], u2, rtol=0, atol=1e-12 * u.max())   # the closed form cancels near |y| = W
    L = W / 2.55 ** (1 / 1.55)
    _, t_L = configs.schoof_slab_u(np.array([L]), 1e-3, 1000.0, 1e-16, W, 1.55, inst.par.rho_ice, inst.par.g)
    np.testing.assert_allclose(t_L, inst.extra["taud"], rtol=1e-12)
    assert u.max() == pytest.approx(910.836, rel=1e-5)


def test_oracle_converges_to_schoof():
    errs = {}
    for dxk in (2.0, 1.0):
        inst = configs.schoof_slab(dx_km=dxk)
        f = _state(inst, oracle)
        out = oracle.calc_velocity(f, inst, inst.par.with_(**TIGHT))
        assert out["status"] == 0 and out["ssa_lin_fail"] == 0
        assert np.max(np.abs(f["uy_b"])) < 1e-6            # no cross-stream flow
        errs[dxk] = _err(inst, f)
    assert errs[2.0] < 0.10, errs
    assert errs[1.0] < 0.03, errs
    assert np.log2(errs[2.0] / errs[1.0]) > 1.5, errs      # refinement order


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_slab_matches_oracle_and_analytic(precision):
    inst = configs.schoof_slab(dx_km=2.0)
    par = inst.par.with_(**TIGHT)
    fo = _state(inst, oracle)
    oracle.calc_velocity(fo, inst, par)
    fg = _state(inst, gpu)
    out = gpu.calc_velocity(fg, inst.dx, inst.n_glen, par.with_(precision=precision))
    assert out["status"] == 0
    assert rel_l2(fg["ux_b"], fo["ux_b"]) < 1e-6
    assert abs(_err(inst, fg) - _err(inst, fo)) < 1e-4
