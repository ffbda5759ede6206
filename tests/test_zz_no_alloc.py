"""The allocation-free entry point (ygpu_solve_device_noalloc) against the
context entry point (ygpu_solve_device), through the C ABI.

Some callers of this library cannot allocate device memory: a host whose device
memory belongs to another runtime, or to a pool allocator that must account for
every byte, and a server that must not grow after start-up. They use
ygpu_solve_device_noalloc, whose scratch lives in a fixed array inside the
library. It must give the same solution as the context entry point, and keep
doing so on a second call that finds the array holding the first call's
contents. It must also work as the first call of a fresh process (no context
created, the default stack limit), leave the stack limit as it found it, and
take no device memory on a repeated call. The file sorts last so that a failure
here leaves every other test already run.
"""
import os
import subprocess
import sys
import warnings

import numpy as np
import pytest

from yelmo_gb300 import abi, configs, gpu

pytestmark = pytest.mark.gpu

TOL = 1e-6      # relative L2, the tolerance of the parity tests
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


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


def test_noalloc_refuses_a_neff_hook():
    """The entry point does not run a neff hook: with one set on the calling
    thread a DIVA solve is refused instead of silently solving with a fixed c_bed."""
    pytest.importorskip("torch")
    inst = _instance()
    f0 = gpu.prepare(inst)
    L = gpu.lib()
    cb = abi.neff_hook(lambda c_bed, ux_b, uy_b: None)
    L.ygpu_set_neff_hook(cb, None)
    try:
        with pytest.raises(gpu.YgpuError) as e:
            _solve(lambda fl: gpu.solve_device_noalloc(abi.KIND_DIVA, inst.par, fl), inst, f0)
        assert e.value.status == abi.ERR_BAD_ARG and "neff hook" in str(e.value)
    finally:
        L.ygpu_set_neff_hook(abi.NEFF_HOOK(), None)
    st, _ = _solve(lambda fl: gpu.solve_device_noalloc(abi.KIND_DIVA, inst.par, fl), inst, f0)
    assert st["status"] == 0


def test_noalloc_refuses_a_capturing_stream():
    """The entry point synchronises its stream, which a capture forbids: on a
    stream being captured it is refused before anything is enqueued, the capture
    stays valid, and the same call on a plain stream afterwards solves."""
    pytest.importorskip("torch")
    import torch
    inst = _instance()
    f0 = gpu.prepare(inst)
    dev = gpu.to_device(f0)
    fields = gpu.make_fields(dev, inst.nx, inst.ny, inst.nz, inst.dx, inst.dx, inst.n_glen)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    err = None
    with torch.cuda.stream(s):
        g.capture_begin()
        try:
            gpu.solve_device_noalloc(abi.KIND_DIVA, inst.par, fields, stream=s.cuda_stream)
        except gpu.YgpuError as e:
            err = e
        finally:
            # the graph is empty (nothing was enqueued), which torch reports
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                g.capture_end()
    assert err is not None and err.status == abi.ERR_BAD_ARG and "captured" in str(err)
    torch.cuda.synchronize()
    st = gpu.solve_device_noalloc(abi.KIND_DIVA, inst.par, fields, stream=s.cuda_stream)
    torch.cuda.synchronize()
    assert st["status"] == 0


_FRESH = r"""
import ctypes, json, sys
sys.path.insert(0, sys.argv[1])
import numpy as np, torch
import oracle
from yelmo_gb300 import abi, configs, gpu

def cudart():
    for line in open("/proc/self/maps"):
        p = line.split()[-1]
        if "libcudart.so" in p:
            return ctypes.CDLL(p)
    raise RuntimeError("libcudart not mapped")

inst = configs.marine_diva(n=41, nz=6)
inst.par = inst.par.with_(ssa_iter_max=300, ssa_iter_conv=1e-9,
                          ssa_lis_opt_energy="-i cg -p jacobi -maxiter 20000 -tol 1.0e-11")
f0 = oracle.prepare(inst)       # the prologue on the CPU: no context of the library exists yet
torch.cuda.init()
dev = gpu.to_device(f0)
fields = gpu.make_fields(dev, inst.nx, inst.ny, inst.nz, inst.dx, inst.dx, inst.n_glen)
torch.cuda.synchronize()
rt = cudart()
lim = ctypes.c_size_t(0)
rt.cudaDeviceGetLimit(ctypes.byref(lim), 0)          # cudaLimitStackSize
stack0 = lim.value
res = {"stack0": stack0}
try:
    st = gpu.solve_device_noalloc(abi.KIND_DIVA, inst.par, fields)
    res["first"] = st["status"]
except gpu.YgpuError as e:
    res["first_error"] = str(e)
torch.cuda.synchronize()
rt.cudaDeviceGetLimit(ctypes.byref(lim), 0)
res["stack1"] = lim.value
if "first" in res:
    ux1 = dev["ux_bar"].cpu().numpy().copy()
    free0 = torch.cuda.mem_get_info()[0]
    st = gpu.solve_device_noalloc(abi.KIND_DIVA, inst.par, fields)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    ux2 = dev["ux_bar"].cpu().numpy()
    res.update(second=st["status"], free_drop=int(free0 - free1),
               repeat_rel=float(np.linalg.norm(ux2 - ux1) / np.linalg.norm(ux1)))
print("RESULT " + json.dumps(res))
"""


def test_noalloc_first_call_in_a_fresh_process():
    """In a fresh process, before any context exists: the first call succeeds (or
    fails with the documented stack message), the stack limit is left as it was,
    and a second call takes no device memory and repeats the answer."""
    pytest.importorskip("torch")
    r = subprocess.run([sys.executable, "-c", _FRESH, ROOT], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("RESULT ")]
    assert line, r.stdout[-2000:] + r.stderr[-2000:]
    import json
    res = json.loads(line[-1][7:])
    print(res)
    assert res["stack1"] == res["stack0"], res
    if "first_error" in res:
        assert "bytes of stack per thread" in res["first_error"], res
        return
    assert res["first"] == 0 and res["second"] == 0, res
    assert res["free_drop"] <= 0, res
    assert res["repeat_rel"] <= TOL, res
