"""Serving loop: requests from many ensemble members, continuous batching.

Each request advances its member's thickness by a seeded perturbation, rebuilds
the solve inputs on the device and solves warm from the member's previous
velocity and viscosity. The tests check that a served solve equals the plain
device solve of the same state, that a member's results are the same alone and
in a mix of other members' requests that join and leave the GPU around it, and
that admission refuses what does not fit the HBM budget."""
import time

import numpy as np
import pytest

from tests.cases import TIGHT, rel_l2
from yelmo_gb300 import abi, configs, gpu
from yelmo_gb300.serving import Server, member_state

pytestmark = pytest.mark.gpu


def _members(n, precision="fp64"):
    out = []
    for i in range(n):
        inst = configs.served_member(i, seed=5, nz=5, lo=24, hi=48)
        inst.par = inst.par.with_(**TIGHT).with_(precision=precision)
        out.append(inst)
    return out


def _server(insts, **kw):
    srv = Server(insts[0].par, dH_sigma=5.0, **kw)
    ids = [srv.add_member(member_state(inst), inst.dx) for inst in insts]
    return srv, ids


def test_served_solve_equals_plain_solve():
    torch = pytest.importorskip("torch")
    inst = _members(1)[0]
    with Server(inst.par, dH_sigma=5.0) as srv:
        m = srv.add_member(member_state(inst), inst.dx)
        H0 = srv.fetch(m, "H_ice")
        rid = srv.submit(m, seed=123)
        status, stats, lat = srv.wait(rid, timeout=120.0)
        assert status == 0, stats
        assert stats["ssa_iter_now"] > 1 and lat > 0.0
        H1 = srv.fetch(m, "H_ice")
        ux, uy = srv.fetch(m, "ux"), srv.fetch(m, "uy")
    # the step changed the ice thickness only where there was ice
    assert np.any(H1 != H0) and np.all(H1[H0 == 0.0] == 0.0) and np.all(H1 >= 0.0)
    # the plain device solve of the perturbed state (cold start, as the member was)
    inst.H_ice = H1
    f0 = gpu.prepare(inst)
    dev = gpu.to_device(f0)
    fields = gpu.make_fields(dev, inst.nx, inst.ny, inst.nz, inst.dx, inst.dx, inst.n_glen)
    solver = gpu.DeviceSolver(0)
    try:
        torch.cuda.synchronize()
        st = solver.solve(abi.KIND_SSA, inst.par, fields)
        assert st["status"] == 0
        ref_x = dev["ux_b"].cpu().numpy().reshape((inst.nx, inst.ny), order="F")
        ref_y = dev["uy_b"].cpu().numpy().reshape((inst.nx, inst.ny), order="F")
    finally:
        solver.close()
    assert st["ssa_iter_now"] == stats["ssa_iter_now"]
    assert rel_l2(ux, ref_x) <= 1e-9
    assert rel_l2(uy, ref_y) <= 1e-9


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-6)])
def test_same_result_alone_and_in_mix(precision, tol):
    insts = _members(6, precision)
    # alone: member 0 takes two steps with nothing else on the GPU
    srv, ids = _server(insts)
    try:
        for seed in (1, 2):
            status, _, _ = srv.wait(srv.submit(ids[0], seed), timeout=120.0)
            assert status == 0
        alone = {k: srv.fetch(ids[0], k) for k in ("ux", "uy", "visc_eff", "H_ice")}
    finally:
        srv.close()
    # in a mix: other members' requests are on the GPU when member 0 arrives,
    # more arrive while it runs, and its second step queues behind its first
    srv, ids = _server(insts, max_slots=4)
    try:
        rids = [srv.submit(ids[k], 10 + k) for k in (1, 2, 3)]
        time.sleep(0.002)
        r0 = srv.submit(ids[0], 1)
        rids += [srv.submit(ids[k], 20 + k) for k in (4, 5, 1)]
        r1 = srv.submit(ids[0], 2)
        rids += [srv.submit(ids[k], 30 + k) for k in (2, 3)]
        for r in rids + [r0, r1]:
            status, _, _ = srv.wait(r, timeout=300.0)
            assert status == 0, r
        mix = {k: srv.fetch(ids[0], k) for k in ("ux", "uy", "visc_eff", "H_ice")}
        info = srv.info()
    finally:
        srv.close()
    assert info["completed"] == len(rids) + 2
    assert info["slots"] <= 4
    np.testing.assert_array_equal(mix["H_ice"], alone["H_ice"])
    for k in ("ux", "uy", "visc_eff"):
        assert rel_l2(mix[k], alone[k]) <= tol, k


def test_admission_by_hbm_budget():
    inst = _members(1)[0]
    big = configs.served_member(3, seed=5, nz=5, lo=300, hi=321)
    big.par = inst.par
    with Server(inst.par, hbm_budget=64e6) as srv:
        srv.add_member(member_state(inst), inst.dx)
        with pytest.raises(gpu.YgpuError) as e:
            srv.add_member(member_state(big), big.dx)
        assert e.value.status == abi.ERR_ADMISSION
        assert srv.info()["bytes_held"] <= 64e6


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-6)])
def test_member_resumes_from_checkpoint(precision, tol, tmp_path):
    """Checkpoint every member after two steps, write the restart file, restore the
    members into a new server and run the last two steps there: thickness equal, the
    velocities and viscosity those of the uninterrupted server."""
    insts = _members(3, precision)
    seeds = [[11, 12, 13, 14], [21, 22, 23, 24], [31, 32, 33, 34]]

    def run(srv, ids, steps):
        for k in steps:
            rids = [srv.submit(m, seeds[i][k]) for i, m in enumerate(ids)]
            for r in rids:
                status, stats, _ = srv.wait(r, timeout=120.0)
                assert status == 0, stats

    def final(srv, ids):
        return [{k: srv.fetch(m, k) for k in ("H_ice", "ux", "uy", "visc_eff")} for m in ids]

    srv, ids = _server(insts)
    with srv:
        run(srv, ids, (0, 1))
        cks = [srv.checkpoint(m) for m in ids]
        assert [int(ck["steps"]) for ck in cks] == [2, 2, 2]
        run(srv, ids, (2, 3))
        ref = final(srv, ids)
    path = tmp_path / "restart.npz"
    np.savez(path, **{f"m{i}_{k}": v for i, ck in enumerate(cks) for k, v in ck.items()})
    z = np.load(path)
    cks = [{k: z[f"m{i}_{k}"] for k in cks[0]} for i in range(len(insts))]
    with Server(insts[0].par, dH_sigma=5.0) as srv2:
        ids2 = [srv2.restore(member_state(inst), ck, inst.dx) for inst, ck in zip(insts, cks)]
        assert ids2 == ids and [srv2.steps(m) for m in ids2] == [2, 2, 2]
        run(srv2, ids2, (2, 3))
        got = final(srv2, ids2)
        # a member with a request waiting cannot have its step count set
        rid = srv2.submit(ids2[0], 99)
        st = srv2.L.ygpu_server_set_member_steps(srv2.srv, ids2[0], 0)
        assert st in (0, abi.ERR_BUSY)
        assert srv2.wait(rid, timeout=120.0)[0] == 0
    for a, b in zip(got, ref):
        assert np.array_equal(a["H_ice"], b["H_ice"])
        for k in ("ux", "uy", "visc_eff"):
            assert rel_l2(a[k], b[k]) <= tol, k
