"""ILU(0) preconditioning of BiCGSTAB on the residual form (-p ilu, the option
config 1 hands to LIS, solver_linear.F90:246-395). The GPU factorizes the
operator in a six-colour ordering (cell colour (i - j) mod 3, then the
component) so that each colour group factors and solves in parallel; the
oracle factorizes in the natural ordering. The preconditioners differ, the
converged solutions agree."""
import numpy as np
import pytest

import oracle
from tests.cases import TIGHT, rel_l2
from yelmo_gb300 import abi, configs, gpu

pytestmark = pytest.mark.gpu


def _dome(n, **kw):
    inst = configs.dome_ssa(n=n, nz=4)
    inst.par = inst.par.with_(**TIGHT).with_(**kw)
    return inst


def _copy(f):
    return {k: (v.copy(order="F") if isinstance(v, np.ndarray) else v) for k, v in f.items()}


def _gpu_solve(inst, f0):
    """Device solve of the prepared state f0: (outputs on the host, ygpu_stats)."""
    torch = pytest.importorskip("torch")
    dev = gpu.to_device(_copy(f0))
    fields = gpu.make_fields(dev, inst.nx, inst.ny, inst.nz, inst.dx, inst.dx, inst.n_glen)
    solver = gpu.DeviceSolver(0)
    try:
        torch.cuda.synchronize()
        st = solver.solve(abi.KIND_SSA, inst.par, fields)
    finally:
        solver.close()
    out = {k: dev[k].cpu().numpy().reshape(f0[k].shape, order="F") for k in ("ux_b", "uy_b", "visc_eff", "taub_acx")}
    return out, st


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-8), ("mixed", 1e-6)])
def test_ilu_solve_matches_oracle_ilu(precision, tol):
    """-i bicgstab -p ilu: the GPU's multicolour ILU(0) BiCGSTAB converges to the
    oracle's natural-order ILU(0) answer, and the stats name ILU(0) as what ran."""
    inst = _dome(33, precision=precision)
    f0 = oracle.prepare(inst)
    fo = _copy(f0)
    outo = oracle.calc_velocity(fo, inst)
    fg, st = _gpu_solve(inst, f0)
    assert st["status"] == 0 and outo["status"] == 0
    assert st["lin_solver_run"] == abi.LIN_BICGSTAB and st["lin_precond_run"] == abi.PRE_ILU0
    for k, v in fg.items():
        assert rel_l2(v, fo[k]) <= tol, (k, rel_l2(v, fo[k]))


def test_ilu_needs_fewer_iterations_than_jacobi():
    """The same FP64 solve with -p ilu takes fewer BiCGSTAB iterations than with
    -p jacobi, and both reach the same solution."""
    st, vel = {}, {}
    for pc in ("ilu", "jacobi"):
        inst = _dome(33, ssa_lis_opt_residual=f"-i bicgstab -p {pc} -maxiter 20000 -tol 1.0e-11")
        out, st[pc] = _gpu_solve(inst, oracle.prepare(inst))
        vel[pc] = out["ux_b"]
        assert st[pc]["status"] == 0
    assert st["ilu"]["lin_precond_run"] == abi.PRE_ILU0 and st["jacobi"]["lin_precond_run"] == abi.PRE_JACOBI
    assert st["ilu"]["ssa_lin_iter"] < st["jacobi"]["ssa_lin_iter"], (st["ilu"]["ssa_lin_iter"],
                                                                      st["jacobi"]["ssa_lin_iter"])
    assert rel_l2(vel["ilu"], vel["jacobi"]) <= 1e-7


def test_ilu_falls_back_to_jacobi_on_uncolourable_periodic_grid():
    """A periodic direction whose length is not a multiple of 3 breaks the
    six-colour ordering: the solve runs Jacobi, says so, and still matches."""
    inst = _dome(25, boundaries="periodic")
    f0 = oracle.prepare(inst)
    fo = _copy(f0)
    oracle.calc_velocity(fo, inst)
    fg, st = _gpu_solve(inst, f0)
    assert st["status"] == 0 and st["lin_precond_run"] == abi.PRE_JACOBI
    assert rel_l2(fg["ux_b"], fo["ux_b"]) <= 1e-6
