#!/usr/bin/env python
"""Benchmark: SSA/DIVA velocity solves per second on GB300.

Default workload: the marine single DIVA solve, 161 x 161 cells, dx 8 km, 10 sigma
layers. Each solve is a cold start, converged to a Picard change < 1e-7 and a linear
relative residual < 1e-9. That puts the velocity within 1e-6 (relative L2) of the FP64
oracle converged to 1e-10.

Modes:
- A *batched* step solves B independent instances of the workload in one persistent
  launch. The instances differ in the seed of the bed roughness and the friction field;
  teams of CTAs take them from a device queue.
- ``value`` is the mixed-precision throughput: B solves per step, with the fields
  resident in HBM. The mixed precision is FP32 viscosity and Krylov inside FP64 defect
  correction.
- The plain FP64 throughput, and single-solve latency p50/p99 for both precisions, are
  reported beside it.
- ``e2e`` times the batched C-ABI entry ``ygpu_solve_batch_host`` on host buffers (the
  same B solves per step, the host-device copies inside the timed region);
  ``e2e_single`` the drop-in ``ygpu_calc_velocity_diva``, one solve per step.

``--workload ensemble`` runs the batched uneven ensemble instead: 256 SSA instances with
sides in {41, 81, 121, 161}.

Multi-GPU: replicas only. Instances are independent, so there is no collective. Each
rank runs the same job on its own GPU and ``value`` sums over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "SSA/DIVA solves/s, p50/p99 latency; mixed-FP32 vs FP64 on GPU at 1e-6 rel err"
BENCH_TOL = dict(ssa_iter_max=300, ssa_iter_conv=1e-7,
                 ssa_lis_opt_energy="-i cg -p jacobi -maxiter 5000 -tol 1.0e-9 -initx_zeros false",
                 ssa_lis_opt_residual="-i bicgstab -p jacobi -maxiter 5000 -tol 1.0e-9 -initx_zeros false")


def make_instances(workload: str, batch: int):
    from yelmo_gb300 import configs
    if workload == "marine_diva":
        insts = [configs.marine_diva(seed=2024 + b) for b in range(batch)]
    elif workload == "dome_ssa":
        insts = [configs.dome_ssa(seed=1234 + b) for b in range(batch)]
    elif workload == "continent_diva":
        insts = [configs.continent_diva(seed=4242 + b) for b in range(batch)]
    elif workload == "ensemble":
        insts = [configs.ensemble_member(i) for i in range(batch)]
    else:
        raise SystemExit(f"unknown workload {workload}")
    for inst in insts:
        inst.par = inst.par.with_(**BENCH_TOL)
        if workload == "dome_ssa":
            # the plain SSA solve keeps its configured preconditioner: BiCGSTAB with ILU(0)
            inst.par = inst.par.with_(ssa_lis_opt_residual="-i bicgstab -p ilu -maxiter 5000 -tol 1.0e-9 "
                                                           "-initx_zeros false")
        if workload == "continent_diva":
            # power-law friction with q = 1/3 settles into a Picard 2-cycle at the
            # beta_min floor, so this workload runs the namelist's own Picard
            # settings (ssa_iter_max 20, ssa_iter_conv 1e-2): every solve is 20
            # Picard iterations, each with a linear solve to 1e-9
            inst.par = inst.par.with_(ssa_iter_max=20, ssa_iter_conv=1e-2)
    return insts


LARGE_CELLS = 200_000     # above this, CPU samples are a few Picard iterations of one solve


def _cpu_sample(inst, oracle, n_max=5, budget_s=20.0):
    """Seconds per full solve of the oracle: whole solves, or for large grids two
    Picard iterations scaled to ssa_iter_max (the iterations those solves take)."""
    f0 = oracle.prepare(inst)
    if inst.nx * inst.ny > LARGE_CELLS:
        k = 2
        f = _copy(f0)
        t = time.perf_counter()
        oracle.calc_velocity(f, inst, inst.par.with_(ssa_iter_max=k))
        per_solve = (time.perf_counter() - t) * inst.par.ssa_iter_max / k
        return [per_solve], f"{k} Picard iterations of one solve, scaled to {inst.par.ssa_iter_max}", f0
    times = []
    t_all = time.perf_counter()
    while True:
        f = _copy(f0)
        t = time.perf_counter()
        oracle.calc_velocity(f, inst)
        times.append(time.perf_counter() - t)
        if time.perf_counter() - t_all > budget_s or len(times) >= n_max:
            break
    return times, f"{len(times)} full solves of the same workload", f0


def describe(inst, batch):
    kind = "SSA" if inst.par.solver == "ssa" else "DIVA"
    if inst.name.startswith("ensemble"):
        return f"ensemble of {batch} {kind} instances, sides 41-161, 1280 km domain, cold solves"
    return f"{inst.name} {inst.nx}x{inst.ny}x{inst.nz} dx={inst.dx/1e3:g}km cold {kind} solve"


def max_over_ranks(ms: float, dist=None, device: str = "cpu") -> float:
    """The timed span of a replica run: the maximum over ranks (every rank gets it)."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world: int, batch: int, steps: int, max_ms: float) -> float:
    """Whole-job solves/s: every rank solves `batch` instances per step."""
    return world * batch * steps / (max_ms / 1e3)


# ncu captures behind roofline.traffic: DRAM bytes over algorithmic bytes of one
# Krylov launch of the same workload (profiles/<kernel>_<workload>.md)
TRAFFIC_PROFILES = {"marine_diva": "ygpu_k_krylov_marine_diva_b16.md"}


def dram_over_algorithmic(workload: str):
    name = TRAFFIC_PROFILES.get(workload)
    if not name:
        return None
    try:
        for line in open(os.path.join(ROOT, "profiles", name)):
            if line.startswith("dram_over_algorithmic:"):
                return float(line.split(":")[1])
    except OSError:
        return None
    return None


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


class ClockSampler:
    """nvidia-smi clock and throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index, self.proc, self.lines = index, None, []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def _copy(f):
    return {k: (v.copy(order="F") if isinstance(v, np.ndarray) else v) for k, v in f.items()}


def diagnostics_leg(device: str, steps: int, warmup: int) -> dict:
    """Time the post-solve diagnostics kernels (ygpu_calc_dyn_diagnostics_device)
    on one 801 x 801 x 20 field set resident in HBM (seeded values; every group
    on), CUDA events on the launching stream. Algorithmic bytes per cell: 31
    2D arrays (11 inputs, 16 outputs, and 4 re-read by the second kernel) and
    5 3D arrays (ux_i, uy_i, ux, uy in, uxy out) of 8 B."""
    import ctypes as C
    import torch
    from yelmo_gb300 import abi, gpu
    nx = ny = 801
    nz = 20
    gen = torch.Generator(device=device).manual_seed(7)
    arrays, keep = {}, []

    def field(n, *shape, scale=100.0):
        t = torch.rand(*shape, dtype=torch.float64, device=device, generator=gen) * scale
        keep.append(t)
        arrays[n] = t
    for n in abi.DIAG_INPUTS:
        if n == "zeta_aa":
            t = torch.linspace(0.0, 1.0, nz, dtype=torch.float64, device=device) ** 2
            keep.append(t)
            arrays[n] = t
        elif n in ("ux_i", "uy_i", "ux", "uy"):
            field(n, nz * nx * ny)
        else:
            field(n, nx * ny)
    arrays["f_ice"].copy_((arrays["f_ice"] > 30.0).double())
    arrays["f_grnd"].copy_((arrays["f_grnd"] > 50.0).double())
    for n in abi.DIAG_OUTPUTS:
        t = torch.zeros(nz * nx * ny if n == "uxy" else nx * ny, dtype=torch.float64, device=device)
        keep.append(t)
        arrays[n] = t
    D = abi.DynDiag()
    D.nx, D.ny, D.nz, D.dx, D.dy = nx, ny, nz, 4e3, 4e3
    for n, t in arrays.items():
        setattr(D, n, t.data_ptr())
    L = gpu.lib()
    stream = torch.cuda.current_stream(device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    times = []
    for s in range(warmup + steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = L.ygpu_calc_dyn_diagnostics_device(C.c_void_p(stream.cuda_stream), C.byref(D), 0)
        e1.record(stream)
        torch.cuda.synchronize(device)
        if st != 0:
            raise RuntimeError(f"diagnostics failed ({st}): {gpu.last_error()}")
        if s >= warmup:
            times.append(e0.elapsed_time(e1))
    ms = statistics.mean(times)
    alg = float(nx * ny) * (31 * 8 + 5 * nz * 8)
    return {"workload": "801x801x20 synthetic fields, every group", "ms_per_call": ms,
            "alg_bytes_per_call": alg, "achieved_gbs": alg / (ms / 1e3) / 1e9, "kernels": 2}


def jacobian_leg(device: str, steps: int, warmup: int) -> dict:
    """Time the velocity Jacobian (ygpu_calc_jacobian_vel_3D_device, both term
    sets) on one 801 x 801 field set resident in HBM: 20 layers (nz_aa) and 21
    layer interfaces (nz_ac), seeded velocities, ice on ~80 % of the cells with
    margins, CUDA events on the launching stream. Algorithmic bytes per cell:
    ux, uy, the six ux/uy components (8 nz_aa words), uz and dzx, dzy, dzz
    (4 nz_ac words), and six 2D inputs, of 8 B."""
    import ctypes as C
    import torch
    from yelmo_gb300 import abi, gpu
    nx = ny = 801
    nza, nzc = 20, 21
    n2 = nx * ny
    gen = torch.Generator(device=device).manual_seed(13)
    r = lambda *s: torch.randn(*s, dtype=torch.float64, device=device, generator=gen)
    f_ice = (torch.rand(n2, dtype=torch.float64, device=device, generator=gen) < 0.8).double()
    a = {"ux": r(nza * n2) * 100.0, "uy": r(nza * n2) * 100.0, "uz": r(nzc * n2),
         "H_ice": (r(n2).abs() * 1000.0 + 200.0) * f_ice, "f_ice": f_ice,
         "dzsdx": r(n2) * 1e-3, "dzsdy": r(n2) * 1e-3, "dzbdx": r(n2) * 1e-2, "dzbdy": r(n2) * 1e-2,
         "zeta_aa": torch.linspace(0.0, 1.0, nza, dtype=torch.float64, device=device) ** 2,
         "zeta_ac": torch.linspace(0.0, 1.0, nzc, dtype=torch.float64, device=device) ** 2}
    for n in abi.JAC_OUTPUTS:
        a[n] = torch.zeros((nza if n in abi.JAC_OUTPUTS[:6] else nzc) * n2, dtype=torch.float64, device=device)
    J = abi.JVel()
    J.nx, J.ny, J.nz_aa, J.nz_ac, J.dx, J.dy = nx, ny, nza, nzc, 4e3, 4e3
    for n, t in a.items():
        setattr(J, n, t.data_ptr())
    L = gpu.lib()
    stream = torch.cuda.current_stream(device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    times = []
    for s in range(warmup + steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = L.ygpu_calc_jacobian_vel_3D_device(C.c_void_p(stream.cuda_stream), C.byref(J), 0,
                                                abi.JAC_UXY | abi.JAC_UZ)
        e1.record(stream)
        torch.cuda.synchronize(device)
        if st != 0:
            raise RuntimeError(f"Jacobian failed ({st}): {gpu.last_error()}")
        if s >= warmup:
            times.append(e0.elapsed_time(e1))
    ms = statistics.mean(times)
    alg = float(n2) * 8.0 * (8 * nza + 4 * nzc + 6)
    return {"workload": "801x801, nz_aa 20, nz_ac 21, synthetic fields, ice on ~80 % of cells",
            "ms_per_call": ms, "alg_bytes_per_call": alg, "achieved_gbs": alg / (ms / 1e3) / 1e9, "kernels": 1}

def vertical_velocity_leg(device: str, steps: int, warmup: int) -> dict:
    """Time the vertical velocity (ygpu_calc_uz_3D_device, uz_method 1 and 4) on
    one 801 x 801 field set resident in HBM: 20 layers, 21 interfaces, seeded
    velocities and rates, ice on ~80 % of the cells, half of them with the column
    rate of the thickness step, CUDA events on the launching stream. Algorithmic
    bytes per cell: ux, uy (2 nz_aa words), uz, uz_star (2 nz_ac words), ten 2D
    inputs and uz_srf_err, of 8 B; uz_flux adds ux_bar, uy_bar, dHidt_dyn and the
    4-byte mask_kin."""
    import ctypes as C
    import torch
    from yelmo_gb300 import abi, gpu
    nx = ny = 801
    nza, nzc = 20, 21
    n2 = nx * ny
    gen = torch.Generator(device=device).manual_seed(17)
    r = lambda *s: torch.randn(*s, dtype=torch.float64, device=device, generator=gen)
    f_ice = (torch.rand(n2, dtype=torch.float64, device=device, generator=gen) < 0.8).double()
    za = torch.linspace(0.0, 1.0, nza, dtype=torch.float64, device=device) ** 2
    zc = torch.cat([za[:1], 0.5 * (za[1:] + za[:-1]), za[-1:]])
    a = {"ux": r(nza * n2) * 100.0, "uy": r(nza * n2) * 100.0, "H_ice": (r(n2).abs() * 1000.0 + 200.0) * f_ice,
         "f_ice": f_ice, "smb": r(n2) * 0.3, "bmb": r(n2) * 0.1, "dzbdt": r(n2) * 0.01, "dzsdt": r(n2) * 0.1,
         "dzsdx": r(n2) * 1e-3, "dzsdy": r(n2) * 1e-3, "dzbdx": r(n2) * 1e-2, "dzbdy": r(n2) * 1e-2,
         "zeta_aa": za, "zeta_ac": zc, "ux_bar": r(n2) * 50.0, "uy_bar": r(n2) * 50.0, "dHidt_dyn": r(n2) * 0.1,
         "mask_kin": (torch.rand(n2, device=device, generator=gen) < 0.5).int(),
         "uz": torch.zeros(nzc * n2, dtype=torch.float64, device=device),
         "uz_star": torch.zeros(nzc * n2, dtype=torch.float64, device=device),
         "uz_srf_err": torch.zeros(n2, dtype=torch.float64, device=device)}
    U = abi.Uz3D()
    U.nx, U.ny, U.nz_aa, U.nz_ac, U.dx, U.dy, U.use_bmb = nx, ny, nza, nzc, 4e3, 4e3, 1
    for n, t in a.items():
        setattr(U, n, t.data_ptr())
    L = gpu.lib()
    stream = torch.cuda.current_stream(device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    out = {}
    for name, method in (("uz_aa", abi.UZ_AA), ("uz_flux", abi.UZ_FLUX)):
        times = []
        for s in range(warmup + steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            st = L.ygpu_calc_uz_3D_device(C.c_void_p(stream.cuda_stream), C.byref(U), 0, method)
            e1.record(stream)
            torch.cuda.synchronize(device)
            if st != 0:
                raise RuntimeError(f"vertical velocity failed ({st}): {gpu.last_error()}")
            if s >= warmup:
                times.append(e0.elapsed_time(e1))
        ms = statistics.mean(times)
        alg = float(n2) * (8.0 * (2 * nza + 2 * nzc + 11) + (28.0 if method == abi.UZ_FLUX else 0.0))
        out[name] = {"ms_per_call": ms, "alg_bytes_per_call": alg, "achieved_gbs": alg / (ms / 1e3) / 1e9}
    out["workload"] = "801x801, nz_aa 20, nz_ac 21, synthetic fields, ice on ~80 % of cells"
    out["kernels"] = 1
    return out

def ismiphom_leg(years: float = 200.0) -> dict:
    """ISMIP-HOM F2 (40 x 40, dx 2.5 km, slip ratio 1, linear solves to 1e-8) for
    `years` 1-year steps of the thickness time loop (yelmo_gb300.prognostic) through
    the host drop-in calls on the GPU, the same loop with the fields resident on the
    GPU (run_device), and the same steps on the oracle as its CPU
    baseline and the values the GPU is compared with (4 threads: on 1600 cells more
    threads only add OpenMP overhead): wall time per step and the largest z_srf difference after the last
    step, relative to the surface relief."""
    import oracle
    from tests.golden.make_ismiphom_f_golden import OracleBackend, case
    from yelmo_gb300 import prognostic
    prognostic.run(case(2, "tight"), 1.0, 5.0)          # warm-up (library load, first launches)
    t0 = time.perf_counter()
    g = prognostic.run(case(2, "tight"), 1.0, years)
    t_gpu = time.perf_counter() - t0
    prognostic.run_device(case(2, "tight"), 1.0, 5.0)
    t0 = time.perf_counter()
    gd = prognostic.run_device(case(2, "tight"), 1.0, years)
    t_dev = time.perf_counter() - t0
    oracle.set_threads(4)
    t0 = time.perf_counter()
    o = prognostic.run(case(2, "tight"), 1.0, years, backend=OracleBackend())
    t_cpu = time.perf_counter() - t0
    err = float(np.max(np.abs(g["z_srf"] - o["z_srf"])) / np.max(np.abs(o["z_srf"])))
    return {"workload": f"ISMIP-HOM F2 40x40, {int(years)} one-year steps (advection, inputs, DIVA solve)",
            "gpu_ms_per_step": 1e3 * t_gpu / g["steps"], "oracle_ms_per_step": 1e3 * t_cpu / o["steps"],
            "gpu_device_resident_ms_per_step": 1e3 * t_dev / gd["steps"],
            "oracle_threads": 4, "zs_rel_diff_gpu_vs_oracle": err,
            "zs_rel_diff_device_resident_vs_oracle":
                float(np.max(np.abs(gd["z_srf"] - o["z_srf"])) / np.max(np.abs(o["z_srf"]))),
            "picard_iters": int(g["history"]["picard"].sum())}


def advection_leg(device: str, steps: int, warmup: int) -> dict:
    """Time calc_advec2D(impl-lis) on the device (ygpu_advec2D_impl_lis_device)
    on a 801 x 801 grid resident in HBM: seeded thickness, velocities and source,
    every cell dynamic, dt = 1 a. Algorithmic bytes per cell: assembly 108 B
    (6 inputs, 5 coefficients, b, x, the Jacobi diagonal), per BiCGSTAB
    iteration 224 B (two 5-point applies of 56 B and 14 vector streams of 8 B),
    and 36 B for the update and dvdt."""
    import ctypes as C
    import torch
    from yelmo_gb300 import gpu
    nx = ny = 801
    gen = torch.Generator(device=device).manual_seed(11)
    n = nx * ny
    r = lambda s: torch.randn(n, dtype=torch.float64, device=device, generator=gen) * s
    H = r(300.0).abs()
    ux, uy, F = r(150.0), r(150.0), r(0.5)
    mask = torch.full((n,), 2, dtype=torch.int32, device=device)
    dvdt = torch.zeros(n, dtype=torch.float64, device=device)
    solver = gpu.DeviceSolver(int(device.split(":")[1]))
    L = gpu.lib()
    it, st = C.c_int(0), C.c_int(0)
    times, iters = [], []
    try:
        # CUDA events on the context's stream, around the solve's launches
        ts = torch.cuda.ExternalStream(L.ygpu_ctx_stream(solver.ctx), device=device)
        for s in range(warmup + steps):
            torch.cuda.synchronize(device)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ts)
            rc = L.ygpu_advec2D_impl_lis_device(solver.ctx, dvdt.data_ptr(), H.data_ptr(), ux.data_ptr(), uy.data_ptr(),
                                                F.data_ptr(), mask.data_ptr(), H.data_ptr(), 4e3, 4e3, 1.0, 0, nx, ny,
                                                C.byref(it), C.byref(st))
            e1.record(ts)
            torch.cuda.synchronize(device)
            if rc != 0:
                raise RuntimeError(f"advection failed ({rc}): {gpu.last_error()}")
            if s >= warmup:
                times.append(e0.elapsed_time(e1))
                iters.append(it.value)
    finally:
        solver.close()
    ms = statistics.mean(times)
    alg = float(n) * (108 + statistics.mean(iters) * 224 + 36)
    return {"workload": "801x801 implicit upwind step, BiCGSTAB + Jacobi to 1e-12", "ms_per_call": ms,
            "bicgstab_iters": statistics.mean(iters), "alg_bytes_per_call": alg,
            "achieved_gbs": alg / (ms / 1e3) / 1e9, "status": st.value}


def run_reference(args, insts, rank, world):
    """CPU reference arm: the oracle (FP64 restatement of the reference path) on all host cores."""
    if rank != 0:
        return None
    import oracle
    cores = os.cpu_count() or 1
    inst = insts[0]
    f0 = oracle.prepare(inst)
    times, out = [], None
    large = inst.nx * inst.ny > LARGE_CELLS
    k = 2
    with oracle.timing_build():
        oracle.set_threads(cores)
        for s in range(args.warmup + args.steps):
            f = _copy(f0)
            t = time.perf_counter()
            if large:
                # bounded sample: two Picard iterations, scaled to the solve's ssa_iter_max
                out = oracle.calc_velocity(f, inst, inst.par.with_(ssa_iter_max=k))
                dt = (time.perf_counter() - t) * inst.par.ssa_iter_max / k
            else:
                out = oracle.calc_velocity(f, inst)
                dt = time.perf_counter() - t
            if s >= args.warmup:
                times.append(dt)
    flags = oracle.timing_flags()
    value = len(times) / sum(times)
    sample = (f"{k} Picard iterations per step scaled to {inst.par.ssa_iter_max}" if large
              else f"{len(times)} full solves")
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": describe(inst, 1), "picard_tol": inst.par.ssa_iter_conv, "lin": inst.par.lis_opt},
        "latency_ms": {"p50": 1e3 * float(np.percentile(times, 50)), "p99": 1e3 * float(np.percentile(times, 99))},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": f"{sample} (oracle: C FP64 restatement, OpenMP, {cores} threads, "
                                   f"gcc {flags})"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "picard_iters": out["ssa_iter_now"], "lin_iters": out["ssa_lin_iter"],
    }


def cpu_baseline_leg(inst, budget_s=20.0):
    """Oracle timed on the host cores (bounded sample), and its tightly converged
    solution, against which the GPU results are compared."""
    import oracle
    cores = os.cpu_count() or 1
    flags = oracle.timing_flags()
    with oracle.timing_build():
        oracle.set_threads(cores)
        times, sample, f0 = _cpu_sample(inst, oracle, budget_s=budget_s)
        base = {"value": len(times) / sum(times), "unit": "solves/s", "cores": cores, "kind": "port",
                "sample": f"{sample} (oracle: C FP64 restatement, OpenMP, {cores} threads, gcc {flags})"}
        # the same on one thread (one solve, or the two-iteration sample of large grids)
        oracle.set_threads(1)
        t1, sample1, _ = _cpu_sample(inst, oracle, n_max=1, budget_s=0.0)
        oracle.set_threads(cores)
    base["one_thread"] = {"value": len(t1) / sum(t1), "unit": "solves/s", "sample": sample1}
    oracle.set_threads(cores)
    if inst.nx * inst.ny > LARGE_CELLS:
        return base, None
    tight = _copy(f0)
    par_t = inst.par.with_(ssa_iter_max=800, ssa_iter_conv=1e-10,
                           ssa_lis_opt_energy="-i cg -p jacobi -maxiter 20000 -tol 1.0e-12",
                           ssa_lis_opt_residual="-i bicgstab -p jacobi -maxiter 20000 -tol 1.0e-12")
    oracle.calc_velocity(tight, inst, par_t)
    return base, tight


def run_served(args):
    """Served ensemble stream: Poisson arrivals of requests from many members.

    Each request advances one member's thickness by dH ~ N(0, 5 m) and solves it
    warm from the member's device-resident state (continuous batching in the
    library's serving loop). The same seeded request sequence runs through a
    mixed-precision server and a plain FP64 server; latency is submit to
    completion, throughput is completions over the span of a rate's run."""
    from yelmo_gb300 import configs
    from yelmo_gb300.serving import Server, member_state
    rates = [float(r) for r in args.rates.split(",")]
    n_mem = args.members
    t0 = time.perf_counter()
    insts = [configs.served_member(i) for i in range(n_mem)]
    for inst in insts:
        inst.par = inst.par.with_(**BENCH_TOL)
    states = [member_state(inst) for inst in insts]
    build_s = time.perf_counter() - t0
    cells = sum(i.nx * i.ny for i in insts)
    out = {}
    finals = {}
    for prec in ("mixed", "fp64"):
        par = insts[0].par.with_(precision=prec)
        with Server(par, dH_sigma=5.0, hbm_budget=150e9, max_slots=args.max_slots) as srv:
            ids = [srv.add_member(st, inst.dx) for st, inst in zip(states, insts)]
            # warm-up: one (cold) step of every member
            w = [srv.submit(m, 7) for m in ids]
            for r in w:
                srv.wait(r)
            per_rate = []
            for ri, rate in enumerate(rates):
                rng = np.random.default_rng(1000 + ri)
                n_req = int(min(max(rate * args.seconds, 20), args.max_requests))
                gaps = rng.exponential(1.0 / rate, n_req)
                who = rng.integers(0, n_mem, n_req)
                rids = []
                start = time.perf_counter()
                due = start
                for k in range(n_req):
                    due += gaps[k]
                    while True:
                        d = due - time.perf_counter()
                        if d <= 0:
                            break
                        time.sleep(min(d, 0.001))
                    rids.append(srv.submit(ids[who[k]], 100000 * (ri + 1) + k))
                lat, iters, bad = [], [], 0
                for r in rids:
                    status, st, l_ms = srv.wait(r)
                    bad += status != 0
                    lat.append(l_ms)
                    iters.append(st["ssa_iter_now"])
                span = time.perf_counter() - start
                per_rate.append({"offered_req_s": rate, "requests": n_req, "throughput": n_req / span,
                                 "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                                 "picard_mean": float(np.mean(iters)), "failed": int(bad)})
            info = srv.info()
            finals[prec] = [srv.fetch(m, "ux") for m in ids[:16]]
        out[prec] = {"rates": per_rate, "slots": info["slots"], "bytes_held": info["bytes_held"],
                     "ticks": info["ticks"]}
    err = max(rel_l2(a, b) for a, b in zip(finals["mixed"], finals["fp64"]))
    top_m, top_d = out["mixed"]["rates"][-1], out["fp64"]["rates"][-1]
    line = {
        "metric": METRIC, "value": top_m["throughput"], "unit": "solves/s", "n_gpus": 1,
        "steps": sum(r["requests"] for r in out["mixed"]["rates"]), "warmup": n_mem,
        "ms_per_step": 1e3 / top_m["throughput"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/f64 (FP32 viscosity and Krylov, FP64 defect correction)",
        "data": "synthetic (seeded members, Poisson arrivals, dH ~ N(0, 5 m))",
        "config": {"workload": f"served ensemble stream: {n_mem} SSA members, sides 64-321 "
                               f"({cells} cells resident), warm starts, continuous batching",
                   "rates_req_s": rates, "picard_tol": insts[0].par.ssa_iter_conv, "lin": insts[0].par.lis_opt,
                   "hbm_budget_gb": 150, "max_slots": args.max_slots or "one per SM", "max_active_unknowns": 1500000, "parallelism": "replicas x1"},
        "latency_ms": {"p50": top_m["p50_ms"], "p99": top_m["p99_ms"]},
        "served_mixed": out["mixed"], "served_fp64": out["fp64"],
        "mixed_over_fp64": top_m["throughput"] / top_d["throughput"],
        "rel_err_mixed_vs_fp64_max": err, "member_build_s": build_s,
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="marine_diva")
    ap.add_argument("--batch", type=int, default=0, help="instances per batched step (default 16; ensemble 256)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--members", type=int, default=512, help="served workload: ensemble members")
    ap.add_argument("--rates", default="10,100,500,2000", help="served workload: offered req/s")
    ap.add_argument("--seconds", type=float, default=5.0, help="served workload: arrival span per rate")
    ap.add_argument("--max-requests", type=int, default=1500, help="served workload: requests per rate")
    ap.add_argument("--max-slots", type=int, default=0, help="served workload: solves on the GPU at once (0: one per SM, load-limited by unknowns)")
    args = ap.parse_args()
    if args.workload == "served" and args.impl == "ours":
        if int(os.environ.get("RANK", "0")) == 0:
            run_served(args)
        return
    args.warmup = max(args.warmup, 3)
    batch = args.batch or {"ensemble": 256, "continent_diva": 1}.get(args.workload, 16)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    insts = make_instances(args.workload, batch)

    if args.impl == "reference":
        line = run_reference(args, insts, rank, world)
        if line is not None:
            print(json.dumps(line))
        return

    import torch
    from yelmo_gb300 import abi, gpu

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    ensemble = args.workload == "ensemble"
    cpu_base, tight = (None, None)
    if rank == 0 and not args.no_cpu and not ensemble:
        cpu_base, tight = cpu_baseline_leg(insts[0])

    kind = insts[0].par.kind
    hosts = [gpu.prepare(inst) for inst in insts]
    devs = [gpu.to_device(f, f"cuda:{local}") for f in hosts]
    pristine = [{k: d[k].clone() for k in gpu.STATE_NAMES} for d in devs]
    fields = [gpu.make_fields(d, i.nx, i.ny, i.nz, i.dx, i.dx, i.n_glen) for d, i in zip(devs, insts)]
    solver = gpu.DeviceSolver(local)          # batched steps
    solver1 = gpu.DeviceSolver(local)         # single-solve latency
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def reset(idx):
        for b in idx:
            for k in gpu.STATE_NAMES:
                devs[b][k].copy_(pristine[b][k])
        flush.zero_()               # L2 flush between timed steps
        torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    res = {}
    clocks = None
    tuned = {}
    from yelmo_gb300.autotune import autotune
    for prec in ("fp64", "mixed"):
        par = insts[0].par.with_(precision=prec)
        # launch tuning by measurement (untimed): the batch, and the single solve
        # (and, mixed, the inner tolerance by full solves)
        tb = autotune(solver, kind, par, fields, lambda: reset(range(batch)))
        t1 = None if ensemble else autotune(solver1, kind, par, fields[:1], lambda: reset([0]))
        tuned[prec] = {"batch": tb["tuning"], "single": t1["tuning"] if t1 else None}
        if tb["inner_tol"] is not None:
            tuned[prec]["inner_tol"] = {"batch": tb["inner_tol"], "single": t1["inner_tol"] if t1 else None,
                                        "batch_ms": tb["inner_tol_ms"]}
        par1 = par.with_(inner_tol=t1["inner_tol"]) if t1 and t1["inner_tol"] else par
        if tb["inner_tol"]:
            par = par.with_(inner_tol=tb["inner_tol"])
        # single-solve latency (instance 0)
        lat, st1 = [], None
        n_single = 0 if ensemble else args.warmup + args.steps
        for s in range(n_single):
            reset([0])
            st1 = solver1.solve(kind, par1, fields[0])
            if s >= args.warmup:
                lat.append(st1["device_ms"])
        u_single = None if ensemble else devs[0]["ux_bar" if kind == abi.KIND_DIVA else "ux_b"].cpu().numpy().reshape(
            (insts[0].nx, insts[0].ny), order="F")
        # batched throughput; the mixed arm also times every step kernel launch
        # with CUDA events on the solver stream and counts the launches
        barrier()
        clk = ClockSampler(local)
        step_ms, sts, all_sts = [], None, []
        launches = 0
        for s in range(args.warmup + args.steps):
            reset(range(batch))
            if s == args.warmup and prec == "mixed":
                clk.start()
                gpu.step_timing(True)
                launches = gpu.kernel_launches()
            sts = solver.solve_batch(kind, par, fields)
            if s >= args.warmup:
                step_ms.append(sts[0]["device_ms"])
                all_sts.append(sts)
        barrier()
        steps_timing = None
        if prec == "mixed":
            clocks = clk.stop()
            launches = gpu.kernel_launches() - launches
            steps_timing = gpu.step_timing_get()
            gpu.step_timing(False)
        vel = "ux_bar" if kind == abi.KIND_DIVA else "ux_b"
        vel_y = "uy_bar" if kind == abi.KIND_DIVA else "uy_b"
        u_batch = [d[vel].cpu().numpy().reshape((i.nx, i.ny), order="F") for d, i in zip(devs, insts)]
        v_batch = [d[vel_y].cpu().numpy().reshape((i.nx, i.ny), order="F") for d, i in zip(devs, insts)]
        # the batch's first instance, every checked output (flat, Fortran order)
        batch0 = {k: devs[0][k].cpu().numpy() for k in (vel, vel_y, "visc_eff", "beta_acx", "taub_acx")}
        tot_ms = max_over_ranks(sum(step_ms), dist, f"cuda:{local}")
        res[prec] = {"lat": lat, "st1": st1, "step_ms": step_ms, "tot_ms": tot_ms, "sts": sts,
                     "u_single": u_single, "u_batch": u_batch, "v_batch": v_batch, "batch0": batch0,
                     "all_sts": all_sts, "launches": launches, "steps_timing": steps_timing}

    # e2e: the batched C-ABI entry on host buffers (the whole batch per step, the
    # host-device copies inside the timed region), and the single-solve drop-in
    par_m = insts[0].par.with_(precision="mixed")
    if tuned["mixed"].get("inner_tol"):
        par_m = par_m.with_(inner_tol=tuned["mixed"]["inner_tol"]["batch"])
    par_m1 = par_m
    if tuned["mixed"].get("inner_tol") and tuned["mixed"]["inner_tol"]["single"]:
        par_m1 = par_m.with_(inner_tol=tuned["mixed"]["inner_tol"]["single"])
    n_e2e = args.warmup + max(3, args.steps)
    e2e_times, e2e1_times = [], []
    barrier()
    for s in range(n_e2e):
        fs = [_copy(h) for h in hosts]
        t = time.perf_counter()
        sts_h = gpu.calc_velocity_batch(fs, [i.dx for i in insts], insts[0].n_glen, par_m)
        dt = time.perf_counter() - t
        assert all(st["status"] == 0 for st in sts_h), sts_h
        if s >= args.warmup:
            e2e_times.append(dt)
    e2e_ms = max_over_ranks(1e3 * sum(e2e_times), dist, f"cuda:{local}")
    if not ensemble:
        for s in range(n_e2e):
            f = _copy(hosts[0])
            t = time.perf_counter()
            gpu.calc_velocity(f, insts[0].dx, insts[0].n_glen, par_m1)
            dt = time.perf_counter() - t
            if s >= args.warmup:
                e2e1_times.append(dt)
    diag = diagnostics_leg(f"cuda:{local}", max(3, args.steps), args.warmup) if rank == 0 else None
    adv = advection_leg(f"cuda:{local}", max(3, args.steps), args.warmup) if rank == 0 else None
    ismip = ismiphom_leg() if (rank == 0 and not args.no_cpu) else None
    jac = jacobian_leg(f"cuda:{local}", max(3, args.steps), args.warmup) if rank == 0 else None
    uzl = vertical_velocity_leg(f"cuda:{local}", max(3, args.steps), args.warmup) if rank == 0 else None
    i0 = insts[0]
    io = [gpu.host_io_bytes(kind, i.nx, i.ny, i.nz) for i in insts]
    h2d, d2h = sum(a for a, _ in io), sum(b for _, b in io)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    mixed, fp64 = res["mixed"], res["fp64"]
    K = len(mixed["step_ms"])
    value = replica_throughput(world, batch, K, mixed["tot_ms"])
    value64 = replica_throughput(world, batch, K, fp64["tot_ms"])
    # error of the mixed batch against the FP64 batch: every instance, both velocity components
    err_mixed_vs_fp64 = max(max(rel_l2(a, b) for a, b in zip(mixed["u_batch"], fp64["u_batch"])),
                            max(rel_l2(a, b) for a, b in zip(mixed["v_batch"], fp64["v_batch"])))
    err_vs_oracle = None
    if tight is not None:
        # against the oracle converged to 1e-10: the single solve's x velocity and
        # every checked output of the batch's first instance, both precisions
        vel = "ux_bar" if kind == abi.KIND_DIVA else "ux_b"
        err_vs_oracle = {"mixed": rel_l2(mixed["u_single"], tight[vel]), "fp64": rel_l2(fp64["u_single"], tight[vel])}
        for prec in ("mixed", "fp64"):
            err_vs_oracle[prec + "_batch_instance0"] = {
                k: rel_l2(v, np.ravel(tight[k], order="F")) for k, v in res[prec]["batch0"].items() if k in tight}
    # roofline of the dominant kernel (the Krylov step) over the timed batched
    # steps: algorithmic bytes of its launches / their CUDA-event time
    cg = insts[0].par.lis_opt.split("-i ")[1].split()[0] in ("cg", "minres")
    # BiCGSTAB with ILU(0) on the residual form runs in FP64 in the mixed mode too
    krylov64 = (not cg) and insts[0].par.ssa_solver != "energy" and " ilu" in insts[0].par.lis_opt
    alg_steps = {"pre": 0.0, "krylov": 0.0, "post": 0.0}
    kr_min = 0.0
    for sts_k in mixed["all_sts"]:
        for st, i in zip(sts_k, insts):
            for k, v in gpu.algorithmic_bytes(st, kind, i.nx, i.ny, i.nz, mixed=True, cg=cg, by_step=True,
                                              krylov64=krylov64).items():
                alg_steps[k] += v
            kr_min += gpu.algorithmic_bytes(st, kind, i.nx, i.ny, i.nz, mixed=True, cg=cg, by_step=True,
                                            krylov64=krylov64, minimal=True)["krylov"]
    tm = mixed["steps_timing"]
    kr_ms, kr_n = tm["krylov"]
    achieved = alg_steps["krylov"] / (kr_ms / 1e3) / 1e9 if kr_ms > 0 else None
    per_step = {k: {"launches": tm[k][1], "ms": tm[k][0],
                    "achieved_gbs": (alg_steps[k] / (tm[k][0] / 1e3) / 1e9) if k in alg_steps and tm[k][0] > 0
                    else None} for k in tm}
    avg_ms = statistics.mean(mixed["step_ms"])
    ratio = dram_over_algorithmic(args.workload)
    try:
        peak = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
        peak_src = "measured"
    except Exception:
        peak, peak_src = 6800.0, "fallback"
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": avg_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("f32/f64 (FP32 viscosity and coefficients, FP64 BiCGSTAB with ILU(0))" if krylov64
                  else "f32/f64 (FP32 viscosity and Krylov, FP64 defect correction)"),
        "data": "synthetic (seeded beds, geometry and friction)",
        "config": {"workload": describe(i0, batch), "batch": batch, "picard_tol": i0.par.ssa_iter_conv,
                   "lin": i0.par.lis_opt, "l2": "flushed (256 MB write) between timed steps",
                   "parallelism": f"replicas x{world}"},
        "latency_ms": ({"p50": float(np.percentile(mixed["lat"], 50)), "p99": float(np.percentile(mixed["lat"], 99))}
                       if mixed["lat"] else None),
        "fp64": {"value": value64, "unit": "solves/s", "ms_per_step": statistics.mean(fp64["step_ms"]),
                 "latency_ms": ({"p50": float(np.percentile(fp64["lat"], 50)),
                                 "p99": float(np.percentile(fp64["lat"], 99))} if fp64["lat"] else None)},
        "mixed_over_fp64": value / value64,
        "rel_err_vs_oracle": err_vs_oracle,
        "rel_err_mixed_vs_fp64_max": err_mixed_vs_fp64,
        "picard_iters": [s["ssa_iter_now"] for s in mixed["sts"][:4]],
        "gpu_launches": mixed["launches"],
        "e2e": {"value": replica_throughput(world, batch, len(e2e_times), e2e_ms), "unit": "solves/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "path": f"ygpu_solve_batch_host on host buffers, {batch} solves per step"},
        "e2e_single": ({"value": 1.0 / statistics.mean(e2e1_times), "unit": "solves/s",
                        "h2d_bytes_per_step": io[0][0], "d2h_bytes_per_step": io[0][1],
                        "path": ("ygpu_calc_velocity_diva" if kind == abi.KIND_DIVA else "ygpu_calc_velocity_ssa")
                        + " on host buffers, one solve per step"} if e2e1_times else None),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "traffic": (ratio * alg_steps["krylov"] / max(kr_n, 1)) if ratio else None,
                     "traffic_note": ("bytes per launch: DRAM/algorithmic ratio of the ncu capture in profiles/"
                                      + TRAFFIC_PROFILES.get(args.workload, "") + " times this run's average "
                                      "algorithmic bytes per launch") if ratio else None,
                     "kernel": "ygpu_k_krylov", "launches": kr_n,
                     "active_cells": mixed["sts"][0].get("active_cells"), "cells": i0.nx * i0.ny,
                     "alg_bytes_per_launch": alg_steps["krylov"] / max(kr_n, 1),
                     "alg_bytes_min_per_launch": kr_min / max(kr_n, 1),
                     "frac_min_traffic": ((kr_min / (kr_ms / 1e3) / 1e9) / peak) if kr_ms > 0 else None,
                     "min_traffic_note": "the same launches' bytes under the least-traffic form of the method "
                                         "(plain PCG 23w, BiCGSTAB 36w per active cell and iteration)",
                     "avg_launch_ms": kr_ms / max(kr_n, 1), "peak_source": peak_src},
        "step_kernels": per_step,
        "tuning": tuned,
        "phase_ms_single": mixed["st1"]["phase_ms"] if mixed["st1"] else None,
        "clocks": clocks,
        "diagnostics": (dict(diag, frac=diag["achieved_gbs"] / peak) if diag else None),
        "advection": (dict(adv, frac=adv["achieved_gbs"] / peak) if adv else None),
        "ismiphom_f": ismip,
        "jacobian": (dict(jac, frac=jac["achieved_gbs"] / peak) if jac else None),
        "vertical_velocity": ({k: (dict(v, frac=v["achieved_gbs"] / peak) if isinstance(v, dict) else v)
                               for k, v in uzl.items()} if uzl else None),
        "cpu_baseline": cpu_base,
    }
    print(json.dumps(line))
    solver.close()
    solver1.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
