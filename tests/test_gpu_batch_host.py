"""Batched solve on host arrays (ygpu_solve_batch_host): a list of host states of
uneven size goes to the device, is solved as one batch and comes back. Each
instance must match its own host drop-in solve (calc_velocity_ssa / _diva on
the same state) and the oracle, with every in/out array written back and the
input arrays left untouched."""
import numpy as np
import pytest

import oracle
from tests.cases import TIGHT, rel_l2
from tests.test_gpu_parity import TOL, _copy
from yelmo_gb300 import configs, gpu

pytestmark = pytest.mark.gpu

OUT = {"ssa": ("ux_b", "uy_b", "taub_acx", "taub_acy", "visc_eff", "visc_eff_int", "beta"),
       "diva": ("ux", "uy", "ux_bar", "uy_bar", "ux_b", "uy_b", "ux_i", "duxdz", "beta_eff", "visc_eff",
                "visc_eff_int", "taub_acy")}


def _instances(solver, n=5):
    out = []
    for i in range(n):
        inst = configs.ensemble_member(i, seed=17, nz=5, sides=(17, 25, 33))
        inst.par = inst.par.with_(**TIGHT, solver=solver)
        out.append(inst)
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("solver", ["ssa", "diva"])
def test_batch_host_equals_single_calls(solver, precision):
    insts = _instances(solver)
    par = insts[0].par.with_(precision=precision)
    states = [oracle.prepare(inst) for inst in insts]
    single = [_copy(f) for f in states]
    batch = [_copy(f) for f in states]
    inputs_before = [{k: f[k].copy() for k in ("H_ice", "c_bed", "taud_acx", "ATT")} for f in batch]
    outs = [gpu.calc_velocity(f, inst.dx, inst.n_glen, par) for f, inst in zip(single, insts)]
    sts = gpu.calc_velocity_batch(batch, [inst.dx for inst in insts], insts[0].n_glen, par)
    tol = 1e-9 if precision == "fp64" else 1e-6
    for k, (fb, fs, o, st) in enumerate(zip(batch, single, outs, sts)):
        assert st["status"] == 0, (k, st)
        if precision == "fp64":
            assert st["ssa_iter_now"] == o["ssa_iter_now"], (k, st, o)
        for name in OUT[solver]:
            assert np.all(np.isfinite(fb[name])), (k, name)
            e = rel_l2(fb[name], fs[name])
            assert e <= tol, (k, name, e)
        for name, ref in inputs_before[k].items():
            np.testing.assert_array_equal(fb[name], ref)
    # and the oracle, on the smallest and the largest instance
    for k in (0, len(insts) - 1):
        fo = _copy(states[k])
        oracle.calc_velocity(fo, insts[k])
        for name in ("ux_b", "uy_b", "visc_eff"):
            assert rel_l2(batch[k][name], fo[name]) <= TOL, (k, name)


def test_batch_host_refuses_bad_shapes():
    insts = _instances("ssa", 2)
    states = [gpu.prepare(inst) for inst in insts]
    states[1]["visc_eff"] = states[1]["visc_eff"][:, :, :2].copy(order="F")
    with pytest.raises(ValueError):
        gpu.calc_velocity_batch(states, insts[0].dx, insts[0].n_glen, insts[0].par)
