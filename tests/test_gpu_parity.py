"""GPU solver against the oracle (FP64 restatement of the reference).

Bit-exact: the calc_ydyn prologue (flotation H_grnd, grounded fractions, ice
front mask, driving and lateral stress) and the SSA masks. Converged solve:
velocities, viscosity and friction within 1e-6 relative L2 of the oracle when
both are converged tightly (the parity bar), FP64 and mixed precision.
"""
import numpy as np
import pytest

import oracle
from tests.cases import SOLVE_CASES, case, rel_l2
from yelmo_gb300 import abi, configs, gpu

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _prepare_shared(inst):
    """Oracle prologue and masks (the same inputs go to both solvers)."""
    if inst.name == "radial_shelf":
        inputs = oracle.calc_dyn_inputs(inst)
        f = configs.shelf_state(inst, inputs)
        f["ssa_mask_acx"], f["ssa_mask_acy"] = oracle.set_ssa_masks(
            inputs["mask_frnt"], inputs["f_ice"], inputs["f_grnd"], inst.par.ssa_lat_bc, inst.par.boundaries)
        return f
    return oracle.prepare(inst)


def _copy(f):
    return {k: (v.copy(order="F") if isinstance(v, np.ndarray) else v) for k, v in f.items()}


@pytest.mark.parametrize("name", ["dome_ssa_residual", "marine_diva", "continent_diva", "shelf_diva"])
@pytest.mark.parametrize("bc", ["zeros", "infinite", "periodic", "MISMIP3D", "periodic-x"])
def test_prologue_bit_exact(name, bc):
    inst = case(name)
    inst.par = inst.par.with_(boundaries=bc)
    a = oracle.calc_dyn_inputs(inst)
    b = gpu.calc_dyn_inputs(inst)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    for lat in ("all", "marine", "floating", "none"):
        ma = oracle.set_ssa_masks(a["mask_frnt"], a["f_ice"], a["f_grnd"], lat, bc)
        mb = gpu.set_ssa_masks(a["mask_frnt"], a["f_ice"], a["f_grnd"], lat, bc)
        assert np.array_equal(ma[0], mb[0]) and np.array_equal(ma[1], mb[1])


def _compare(inst, fo, fg, outo, outg, tol):
    vel = ("ux_b", "uy_b") if inst.par.solver == "ssa" else ("ux_bar", "uy_bar", "ux_b", "uy_b")
    assert outg["status"] == 0, outg
    errs = {k: rel_l2(fg[k], fo[k]) for k in vel + ("visc_eff", "visc_eff_int", "taub_acx", "taub_acy")}
    if inst.par.solver != "ssa":
        errs.update({k: rel_l2(fg[k], fo[k]) for k in ("ux", "uy", "duxdz", "duydz", "beta_eff")})
    for k, e in errs.items():
        assert e <= tol, (k, e, errs)
    assert outg["ssa_lim_n"] == outo["ssa_lim_n"] or abs(outg["ssa_lim_n"] - outo["ssa_lim_n"]) <= 2


@pytest.mark.parametrize("name", SOLVE_CASES)
def test_solve_fp64_matches_oracle(name):
    inst = case(name)
    f0 = _prepare_shared(inst)
    fo, fg = _copy(f0), _copy(f0)
    outo = oracle.calc_velocity(fo, inst)
    assert outo["status"] == 0
    outg = gpu.calc_velocity(fg, inst.dx, inst.n_glen, inst.par)
    _compare(inst, fo, fg, outo, outg, TOL)


@pytest.mark.parametrize("name", ["dome_ssa_energy", "marine_diva", "continent_diva", "dome_ssa_residual"])
def test_solve_mixed_matches_oracle(name):
    inst = case(name)
    f0 = _prepare_shared(inst)
    fo, fg = _copy(f0), _copy(f0)
    outo = oracle.calc_velocity(fo, inst)
    outg = gpu.calc_velocity(fg, inst.dx, inst.n_glen, inst.par.with_(precision="mixed"))
    _compare(inst, fo, fg, outo, outg, TOL)


def test_default_tolerances_run_and_agree_loosely():
    """Reference defaults (Picard 1e-2, CG 1e-2): both solvers stop early; the
    answers agree to the accuracy those tolerances imply."""
    inst = configs.marine_diva(n=33, nz=6)
    f0 = oracle.prepare(inst)
    fo, fg = _copy(f0), _copy(f0)
    outo = oracle.calc_velocity(fo, inst)
    outg = gpu.calc_velocity(fg, inst.dx, inst.n_glen, inst.par)
    assert outg["status"] in (0, abi.MAXITER)
    assert rel_l2(fg["ux_bar"], fo["ux_bar"]) < 5e-2


def test_csr_seam_matches_oracle():
    inst = case("marine_diva")
    f = _prepare_shared(inst)
    fo = _copy(f)
    oracle.calc_velocity(fo, inst.__class__(**{**inst.__dict__, "par": inst.par.with_(ssa_iter_max=3)}))
    ptr, idx, val, b, x, cf = oracle.assemble_csr(True, {**fo, "N_aa": fo["visc_eff_int"],
                                                         "ux": fo["ux_bar"], "uy": fo["uy_bar"]},
                                                  inst.dx, inst.dx, inst.par.boundaries)
    xo = x.copy()
    st, it, rr = oracle.linear_solve(ptr, idx, val, b, xo, 0, 1, 20000, 1e-12)
    assert st == 0
    xg = x.copy()
    stg, itg, rrg = gpu.linear_solver_matrix_solve((ptr + 1).astype(np.int32), (idx + 1).astype(np.int32),
                                                   val, b, xg, "-i cg -p jacobi -maxiter 20000 -tol 1e-12")
    assert stg == 0 and rrg <= 1e-12
    assert rel_l2(xg, xo) < 1e-9
