"""Tile-block preconditioner (-p ilu on the energy form, FP64 and mixed precision).

The CG (the inner FP32 one in mixed precision) is preconditioned by the exact inverses of the 4 x 4-cell
tile blocks of the operator (block Jacobi). The converged solution must not
depend on the preconditioner: it matches the oracle's FP64 solve within the
parity bar, on grids whose sides are and are not multiples of the tile, and
the linear iterations drop below those of Jacobi."""
import numpy as np
import pytest

import oracle
from tests.cases import case, rel_l2
from tests.test_gpu_parity import TOL, _compare, _copy, _prepare_shared
from yelmo_gb300 import configs, gpu

pytestmark = pytest.mark.gpu

ILU = "-i cg -p ilu -maxiter 20000 -tol 1.0e-11"


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["dome_ssa_energy", "marine_diva", "continent_diva"])
def test_block_preconditioned_matches_oracle(name, precision):
    inst = case(name)
    f0 = _prepare_shared(inst)
    fo, fg, fj = _copy(f0), _copy(f0), _copy(f0)
    outo = oracle.calc_velocity(fo, inst)
    par_b = inst.par.with_(precision=precision, ssa_lis_opt_energy=ILU)
    outg = gpu.calc_velocity(fg, inst.dx, inst.n_glen, par_b)
    _compare(inst, fo, fg, outo, outg, TOL)
    # the same solve with Jacobi takes more linear iterations
    outj = gpu.calc_velocity(fj, inst.dx, inst.n_glen, inst.par.with_(precision=precision))
    assert outg["ssa_lin_iter"] < outj["ssa_lin_iter"], (outg["ssa_lin_iter"], outj["ssa_lin_iter"])


@pytest.mark.parametrize("side", [17, 18, 19, 22])
def test_partial_tiles(side):
    """Sides that leave partial tiles at the upper edges (and one that does not)."""
    inst = configs.ensemble_member(0, seed=3, nz=4, sides=(side,))
    inst.par = inst.par.with_(ssa_iter_max=400, ssa_iter_conv=1e-9,
                              ssa_lis_opt_energy="-i cg -p jacobi -maxiter 20000 -tol 1.0e-11")
    f0 = oracle.prepare(inst)
    fo, fg = _copy(f0), _copy(f0)
    outo = oracle.calc_velocity(fo, inst)
    outg = gpu.calc_velocity(fg, inst.dx, inst.n_glen, inst.par.with_(precision="mixed", ssa_lis_opt_energy=ILU))
    assert outg["status"] == 0
    for k in ("ux_b", "uy_b", "visc_eff"):
        assert rel_l2(fg[k], fo[k]) <= TOL, k
