"""Failure statuses of the GPU solve, produced in forms that fault, trap or hang
no GPU, each against the oracle where it has the same status.

- NaN / Inf in the velocity the solve starts from: the solve ends with
  YGPU_ERR_NONFINITE, as velocity_general.f90:2114-2152 stops on a non-finite
  velocity; NaN / Inf in the driving stress: the first linear solve breaks down
  (LIS's BREAKDOWN, 2) and the velocity stays finite, as in the oracle. Neither
  hangs, and a later solve on the same thread's context is correct.
- A singular system through the lower seam (linear_solver_matrix_solve): CG and
  BiCGSTAB end with LIS's BREAKDOWN (2), solver_linear.F90:36-39.
- A tiny -maxiter: every linear solve ends at MAXITER (4), counted in
  ssa_lin_fail, and the solve returns the last linear status, as the oracle.
- A team wait that runs out: the spin budget of the team barrier is lowered to two
  polls (ygpu_tuning.spin_log2), so a wait gives up; the kernel sets the abort flag,
  every other wait returns, and the solve reports YGPU_ERR_TIMEOUT. The same
  context then solves correctly with the default budget.
"""
import numpy as np
import pytest

import oracle
from tests.cases import rel_l2
from yelmo_gb300 import abi, configs, gpu

pytestmark = pytest.mark.gpu


def _copy(f):
    return {k: (v.copy(order="F") if isinstance(v, np.ndarray) else v) for k, v in f.items()}


def _case(n=25, nz=4, **kw):
    inst = configs.marine_diva(n=n, nz=nz)
    inst.par = inst.par.with_(ssa_iter_max=300, ssa_iter_conv=1e-9,
                              ssa_lis_opt_energy="-i cg -p jacobi -maxiter 20000 -tol 1.0e-11").with_(**kw)
    return inst


@pytest.mark.parametrize("field,want", [("ux_bar", abi.ERR_NONFINITE), ("taud_acx", abi.BREAKDOWN)])
@pytest.mark.parametrize("bad", [np.nan, np.inf])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nonfinite_input_gives_failure_status(field, want, bad, precision):
    inst = _case()
    f0 = oracle.prepare(inst)
    ice = np.argwhere(f0["f_ice"] == 1.0)
    i, j = ice[len(ice) // 2]
    f0[field][i, j] = bad
    fo = _copy(f0)
    outo = oracle.calc_velocity(fo, inst)
    assert outo["status"] == want, outo
    fg = _copy(f0)
    try:
        outg = gpu.calc_velocity(fg, inst.dx, inst.n_glen, inst.par.with_(precision=precision))
        st = outg["status"]
    except gpu.YgpuError as e:
        st = e.status
    assert st == want
    if want == abi.BREAKDOWN:
        assert outg["ssa_lin_fail"] == outo["ssa_lin_fail"] and np.all(np.isfinite(fg["ux_bar"]))
    # the thread's context is still usable
    inst2 = _case()
    g0 = oracle.prepare(inst2)
    fo2, fg2 = _copy(g0), _copy(g0)
    oracle.calc_velocity(fo2, inst2)
    out = gpu.calc_velocity(fg2, inst2.dx, inst2.n_glen, inst2.par.with_(precision=precision))
    assert out["status"] == 0
    assert rel_l2(fg2["ux_bar"], fo2["ux_bar"]) <= 1e-6


@pytest.mark.parametrize("method", ["cg", "bicgstab"])
def test_singular_system_gives_breakdown(method):
    """A = [[1, 1], [1, 1]], b = [1, -1]: the first search direction is in the null
    space (p.Ap = 0 for CG, rt.A p = 0 for BiCGSTAB)."""
    ptr = np.array([0, 2, 4], dtype=np.int32)
    idx = np.array([0, 1, 0, 1], dtype=np.int32)
    val = np.ones(4)
    b = np.array([1.0, -1.0])
    code = {"cg": abi.LIN_CG, "bicgstab": abi.LIN_BICGSTAB}[method]
    st_o, _, _ = oracle.linear_solve(ptr, idx, val, b, np.zeros(2), code, abi.PRE_JACOBI, 100, 1e-10, True)
    assert st_o == abi.BREAKDOWN
    x = np.zeros(2)
    st_g, it_g, _ = gpu.linear_solver_matrix_solve(ptr + 1, idx + 1, val, b, x,
                                                   f"-i {method} -p jacobi -maxiter 100 -tol 1e-10")
    assert st_g == abi.BREAKDOWN, (st_g, it_g)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tiny_maxiter_counts_linear_failures(precision):
    inst = _case(ssa_iter_max=5, ssa_lis_opt_energy="-i cg -p jacobi -maxiter 2 -tol 1.0e-12")
    f0 = oracle.prepare(inst)
    fo, fg = _copy(f0), _copy(f0)
    outo = oracle.calc_velocity(fo, inst)
    outg = gpu.calc_velocity(fg, inst.dx, inst.n_glen, inst.par.with_(precision=precision))
    assert outo["status"] == abi.MAXITER and outo["ssa_lin_fail"] == 5, outo
    assert outg["status"] == abi.MAXITER, outg
    assert outg["ssa_lin_fail"] == outo["ssa_lin_fail"] and outg["ssa_iter_now"] == outo["ssa_iter_now"], outg


def test_team_wait_timeout_is_reported_and_context_recovers():
    pytest.importorskip("torch")
    import torch
    inst = _case(n=41, nz=6)
    f0 = gpu.prepare(inst)
    solver = gpu.DeviceSolver(0)
    try:
        def run():
            dev = gpu.to_device(f0)
            fields = gpu.make_fields(dev, inst.nx, inst.ny, inst.nz, inst.dx, inst.dx, inst.n_glen)
            torch.cuda.synchronize()
            try:
                st = solver.solve(abi.KIND_DIVA, inst.par, fields)
            except gpu.YgpuError as e:
                return e.status, None
            return st["status"], dev["ux_bar"].cpu().numpy()

        # several CTAs per team (128 unknowns each), two polls per wait
        solver.set_tuning(unknowns_per_cta=128, spin_log2=1)
        st, _ = run()
        assert st == abi.ERR_TIMEOUT, st
        assert "timeout" in gpu.last_error() or "limit" in gpu.last_error()
        # the default budget on the same context: a normal, correct solve
        solver.set_tuning(unknowns_per_cta=128, spin_log2=0)
        st, ux = run()
        assert st == 0
        fo = _copy(oracle.prepare(inst))
        oracle.calc_velocity(fo, inst)
        assert rel_l2(ux, np.ravel(fo["ux_bar"], order="F")) <= 1e-6
    finally:
        solver.close()
