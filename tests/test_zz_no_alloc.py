"""The allocation-free entry point (ygpu_solve_device_noalloc) against the
context entry point (ygpu_solve_device), through the C ABI.

Callers that cannot allocate device memory (work captured into a CUDA graph, a
host whose device memory belongs to another runtime, a server that must not
grow after start-up) use ygpu_solve_device_noalloc: its scratch lives in a fixed
array inside the library. It must give the same solution as the context entry
point, and keep doing so on a second call that finds the array holding the
first call's contents. The file sorts last so that a failure here leaves every
other test already run.
"""
import numpy as np
import pytest

from yelmo_gb300 import abi, configs, gpu

pytestmark = pytest.mark.gpu

TOL = 1e-6      # relative L2, the tolerance of the parity tests


def _rel(a, b):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / n if n > 0 else np.linalg.norm(a - b)


def _instance():
    inst = configs.marine_diva(n=41, nz=6)
    inst.par = inst.par.with_(ssa_iter_max=300, ssa_iter_conv=1e-9,
                              ssa_lis_opt_energy="-i cg -p jacobi -maxiter 20000 -tol 1.0e-11")
    return inst


def _solve(entry, inst, f0):
    import torch
    dev = gpu.to_device(f0)
    fields = gpu.make_fields(dev, inst.nx, inst.ny, inst.nz, inst.dx, inst.dx, inst.n_glen)
    torch.cuda.synchronize()
    st = entry(fields)
    torch.cuda.synchronize()
    out = {k: dev[k].cpu().numpy() for k in ("ux_bar", "uy_bar", "visc_eff", "taub_acx", "ux", "duxdz")}
    return st, out


def test_noalloc_matches_context_entry_twice():
    pytest.importorskip("torch")
    inst = _instance()
    f0 = gpu.prepare(inst)
    par = inst.par
    solver = gpu.DeviceSolver(0)
    try:
        st_ref, ref = _solve(lambda fl: solver.solve(abi.KIND_DIVA, par, fl), inst, f0)
    finally:
        solver.close()
    assert st_ref["status"] == 0
    for call in range(2):
        st, out = _solve(lambda fl: gpu.solve_device_noalloc(abi.KIND_DIVA, par, fl), inst, f0)
        assert st["status"] == 0, (call, st)
        assert st["ssa_iter_now"] == st_ref["ssa_iter_now"]
        for k in ref:
            assert _rel(out[k], ref[k]) <= TOL, (call, k, _rel(out[k], ref[k]))


def test_noalloc_rejects_oversized_instance():
    pytest.importorskip("torch")
    import torch
    inst = configs.marine_diva(n=801, nz=20)
    dev = {k: torch.zeros(1, dtype=torch.float64, device="cuda") for k in ("x",)}
    f = abi.Fields()
    f.nx, f.ny, f.nz, f.dx, f.dy, f.n_glen = inst.nx, inst.ny, inst.nz, inst.dx, inst.dx, 3.0
    for name, _ in abi.Fields._fields_[6:]:
        setattr(f, name, dev["x"].data_ptr())
    with pytest.raises(gpu.YgpuError) as e:
        gpu.solve_device_noalloc(abi.KIND_DIVA, inst.par, f)
    assert e.value.status == abi.ERR_BAD_ARG
    assert "scratch" in str(e.value)
