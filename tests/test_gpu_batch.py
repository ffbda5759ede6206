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


@pytest.mark.parametrize("queue", [False, True])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_equals_single(precision, queue):
    """Lockstep batch, and the queue (continuous batching: at most ~2 instances'
    unknowns on the GPU at once, the rest admitted as others finish)."""
    torch = pytest.importorskip("torch")
    insts = _instances()
    par = insts[0].par.with_(precision=precision)
    solver = gpu.DeviceSolver(0)
    if queue:
        solver.set_tuning(max_active_unknowns=2 * 2 * 41 * 41)
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


def test_graph_chunks_equal_step_launches():
    """Chunks of Picard iterations replayed as CUDA graphs give the same bits as
    one launch per step, with the same number of kernel launches counted."""
    torch = pytest.importorskip("torch")
    insts = _instances(5)
    par = insts[0].par.with_(precision="mixed")
    out = {}
    for graphs in (False, True):
        solver = gpu.DeviceSolver(0)
        try:
            solver.set_tuning(check_every=4, use_graphs=graphs, unknowns_per_cta=512)
            devs, fields = zip(*[_device(inst) for inst in insts])
            torch.cuda.synchronize()
            n0 = gpu.kernel_launches()
            sts = solver.solve_batch(abi.KIND_SSA, par, list(fields))
            n1 = gpu.kernel_launches()
            assert all(st["status"] == 0 for st in sts)
            out[graphs] = ([d["ux_b"].cpu().numpy() for d in devs], [st["ssa_iter_now"] for st in sts], n1 - n0)
        finally:
            solver.close()
    for a, b in zip(out[False][0], out[True][0]):
        np.testing.assert_array_equal(a, b)
    assert out[False][1] == out[True][1]
    assert out[False][2] == out[True][2] > 0


def test_tuning_rejects_out_of_range():
    solver = gpu.DeviceSolver(0)
    try:
        with pytest.raises(gpu.YgpuError):
            solver.set_tuning(check_every=0)
        with pytest.raises(gpu.YgpuError):
            solver.set_tuning(unknowns_per_cta=1)
    finally:
        solver.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cluster_teams_equal_global_teams(precision):
    """The Krylov step on thread-block clusters (cluster barrier, all-reduce in
    distributed shared memory; opt-in through ygpu_tuning.cluster_ctas) gives the
    solution of the default global-memory teams."""
    torch = pytest.importorskip("torch")
    insts = _instances(5)
    par = insts[0].par.with_(precision=precision)
    out = {}
    for cl in (0, 4):
        solver = gpu.DeviceSolver(0)
        try:
            solver.set_tuning(unknowns_per_cta=512, cluster_ctas=cl)
            devs, fields = zip(*[_device(inst) for inst in insts])
            torch.cuda.synchronize()
            sts = solver.solve_batch(abi.KIND_SSA, par, list(fields))
            assert all(st["status"] == 0 for st in sts), [st["status"] for st in sts]
            out[cl] = [d["ux_b"].cpu().numpy() for d in devs]
        finally:
            solver.close()
    for a, b in zip(out[0], out[4]):
        assert rel_l2(b, a) <= 1e-6


def test_autotune_picks_launch_shape_and_inner_tolerance():
    """The autotuner's trials leave the fields as reset() restores them; in mixed
    precision it picks the inner tolerance from its candidates, and a solve with that
    choice still meets the parity bar against the FP64 solve."""
    torch = pytest.importorskip("torch")
    from yelmo_gb300.autotune import DEFAULT_INNER_TOLS, autotune
    insts = _instances(4)
    devs, fields = zip(*[_device(inst) for inst in insts])
    pristine = [{k: d[k].clone() for k in gpu.STATE_NAMES} for d in devs]

    def reset():
        for d, p in zip(devs, pristine):
            for k in gpu.STATE_NAMES:
                d[k].copy_(p[k])

    solver = gpu.DeviceSolver(0)
    try:
        par64 = insts[0].par.with_(precision="fp64")
        reset()
        assert all(st["status"] == 0 for st in solver.solve_batch(abi.KIND_SSA, par64, list(fields)))
        ref = [d["ux_b"].cpu().numpy() for d in devs]
        par = insts[0].par.with_(precision="mixed")
        grid = {"unknowns_per_cta": (512, 1024), "check_every": (4,), "use_graphs": (True,)}
        out = autotune(solver, abi.KIND_SSA, par, list(fields), reset, iters=4, grid=grid)
        assert out["tuning"]["unknowns_per_cta"] in (512, 1024)
        assert out["inner_tol"] in DEFAULT_INNER_TOLS
        assert set(out["inner_tol_ms"]) == {f"{t:g}" for t in DEFAULT_INNER_TOLS}
        for d, p in zip(devs, pristine):          # left reset
            assert torch.equal(d["ux_b"], p["ux_b"])
        sts = solver.solve_batch(abi.KIND_SSA, par.with_(inner_tol=out["inner_tol"]), list(fields))
        for k, (d, st) in enumerate(zip(devs, sts)):
            assert st["status"] == 0, (k, st)
            assert rel_l2(d["ux_b"].cpu().numpy(), ref[k]) <= 1e-6
    finally:
        solver.close()
