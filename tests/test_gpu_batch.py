"""Batched solve: many instances of uneven size in one persistent launch, each
solved by a team of CTAs that takes instances from a device work queue. Every
instance's result must equal its own single-instance solve."""
import numpy as np
import pytest

from tests.cases import TIGHT, rel_l2
from yelmo_gb300 import abi, configs, gpu

pytestmark = pytest.mark.gpu


def _instances(n=7):
    out = []
    for i in range(n):
        inst = configs.ensemble_member(i, seed=11, nz=5, sides=(17, 25, 33, 41))
        inst.par = inst.par.with_(**TIGHT)
        out.append(inst)
    return out


def _device(inst):
    f0 = gpu.prepare(inst)
    dev = gpu.to_device(f0)
    return dev, gpu.make_fields(dev, inst.nx, inst.ny, inst.nz, inst.dx, inst.dx, inst.n_glen)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_equals_single(precision):
    torch = pytest.importorskip("torch")
    insts = _instances()
    par = insts[0].par.with_(precision=precision)
    solver = gpu.DeviceSolver(0)
    try:
        single = []
        for inst in insts:
            dev, f = _device(inst)
            torch.cuda.synchronize()
            st = solver.solve(abi.KIND_SSA, par, f)
            assert st["status"] == 0
            single.append({k: dev[k].cpu().numpy() for k in ("ux_b", "uy_b", "visc_eff", "taub_acx")})
        devs, fields = zip(*[_device(inst) for inst in insts])
        torch.cuda.synchronize()
        sts = solver.solve_batch(abi.KIND_SSA, par, list(fields))
        for k, (d, st) in enumerate(zip(devs, sts)):
            assert st["status"] == 0, (k, st)
            for name, ref in single[k].items():
                e = rel_l2(d[name].cpu().numpy(), ref)
                assert e <= 1e-6, (k, name, e)
    finally:
        solver.close()
