"""Edge cases of the solve against the oracle: rectangular grids (nx != ny, in
both orientations, so swapped x/y indexing cannot pass), the smallest grid and
two layers, a domain without ice (zero forcing: the linear solves return x = 0
without iterating), ice everywhere up to the borders, and inputs the C ABI must
refuse."""
import numpy as np
import pytest

import oracle
from tests.cases import TIGHT, rel_l2
from tests.test_gpu_parity import TOL, _compare, _copy
from yelmo_gb300 import abi, configs, gpu

pytestmark = pytest.mark.gpu


def _slice(inst, nx, ny):
    """The instance restricted to its first nx x ny cells."""
    for k in ("H_ice", "z_bed", "z_sl", "beta", "c_bed", "f_slide"):
        setattr(inst, k, np.asfortranarray(getattr(inst, k)[:nx, :ny]))
    inst.ATT = np.asfortranarray(inst.ATT[:nx, :ny, :])
    inst.par = inst.par.with_(**TIGHT)
    return inst


def _solve_both(inst, precision="fp64"):
    f0 = oracle.prepare(inst)
    fo, fg = _copy(f0), _copy(f0)
    outo = oracle.calc_velocity(fo, inst)
    outg = gpu.calc_velocity(fg, inst.dx, inst.n_glen, inst.par.with_(precision=precision))
    return fo, fg, outo, outg


@pytest.mark.parametrize("shape", [(33, 21), (21, 33)])
@pytest.mark.parametrize("builder", ["marine_diva", "dome_ssa"])
def test_rectangular_grids(builder, shape):
    inst = getattr(configs, builder)(n=33, nz=5)
    inst = _slice(inst, *shape)
    fo, fg, outo, outg = _solve_both(inst)
    assert outo["status"] == 0
    _compare(inst, fo, fg, outo, outg, TOL)


def test_smallest_grid_two_layers():
    inst = _slice(configs.marine_diva(n=9, nz=2), 9, 9)
    fo, fg, outo, outg = _solve_both(inst)
    assert outo["status"] == 0
    _compare(inst, fo, fg, outo, outg, TOL)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_no_ice(precision):
    inst = configs.marine_diva(n=17, nz=4)
    inst.H_ice = np.zeros_like(inst.H_ice, order="F")
    inst.par = inst.par.with_(**TIGHT)
    fo, fg, outo, outg = _solve_both(inst, precision)
    assert outg["status"] == outo["status"] == 0
    for k in ("ux_bar", "uy_bar", "ux_b", "uy_b"):
        assert np.all(fg[k] == 0.0) and np.all(fo[k] == 0.0), k
    assert outg["ssa_lin_iter"] == 0


def test_ice_to_the_borders():
    inst = configs.dome_ssa(n=21, nz=4)
    inst.H_ice = np.asfortranarray(np.full_like(inst.H_ice, 1000.0))
    inst.par = inst.par.with_(**TIGHT, boundaries="infinite")
    fo, fg, outo, outg = _solve_both(inst)
    assert outo["status"] == 0
    _compare(inst, fo, fg, outo, outg, TOL)


def test_bad_inputs_are_refused():
    inst = configs.marine_diva(n=9, nz=3)
    f = gpu.prepare(inst)
    with pytest.raises(gpu.YgpuError) as e:
        gpu.calc_velocity(f, -1.0, inst.n_glen, inst.par)          # dx <= 0
    assert e.value.status == abi.ERR_BAD_ARG
    with pytest.raises(gpu.YgpuError) as e:
        gpu.calc_velocity(f, inst.dx, inst.n_glen, inst.par.with_(ssa_iter_max=-1))
    assert e.value.status == abi.ERR_BAD_ARG
    small = {k: (v[:2, :2].copy(order="F") if isinstance(v, np.ndarray) and v.ndim >= 2 else v)
             for k, v in f.items()}
    with pytest.raises(gpu.YgpuError) as e:
        gpu.calc_velocity(small, inst.dx, inst.n_glen, inst.par)   # 2 x 2 grid
    assert e.value.status == abi.ERR_BAD_ARG
