#!/usr/bin/env python
"""Benchmark: SSA/DIVA velocity solves per second on GB300.

Workload (default): the marine single DIVA solve, 161 x 161, dx 8 km, 10 sigma
layers, cold start, converged to Picard change < 1e-7 and linear relative
residual < 1e-9 so that the velocity is within 1e-6 (relative L2) of the FP64
oracle converged to 1e-10. One step = one full solve. ``value`` is the
mixed-precision (FP32 Krylov inside FP64 defect correction) solves/s with the
fields resident in HBM; the plain FP64 solve is reported beside it. ``e2e`` is
the same solve through the C ABI drop-in (ygpu_calc_velocity_diva) from host
buffers, host-device copies included.

Multi-GPU: replicas only (instances are independent, no collective); each rank
solves K instances on its own GPU and ``value`` sums over ranks.
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


def bench_instance(name: str):
    from yelmo_gb300 import configs
    if name == "marine_diva":
        inst = configs.marine_diva()
    elif name == "dome_ssa":
        inst = configs.dome_ssa()
    elif name == "continent_diva":
        inst = configs.continent_diva()
    else:
        raise SystemExit(f"unknown workload {name}")
    inst.par = inst.par.with_(
        ssa_iter_max=300, ssa_iter_conv=1e-7,
        ssa_lis_opt_energy="-i cg -p jacobi -maxiter 5000 -tol 1.0e-9 -initx_zeros false",
        ssa_lis_opt_residual="-i bicgstab -p jacobi -maxiter 5000 -tol 1.0e-9 -initx_zeros false")
    return inst


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


class ClockSampler:
    """nvidia-smi clock and throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
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


def run_reference(args, inst, rank, world):
    """CPU reference arm: the oracle (FP64 restatement of the reference path) on all host cores."""
    if rank != 0:
        return None
    import oracle
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    f0 = oracle.prepare(inst)
    times = []
    for s in range(args.warmup + args.steps):
        f = {k: (v.copy(order="F") if isinstance(v, np.ndarray) else v) for k, v in f0.items()}
        t = time.perf_counter()
        out = oracle.calc_velocity(f, inst)
        dt = time.perf_counter() - t
        if s >= args.warmup:
            times.append(dt)
    tot = sum(times)
    value = len(times) / tot
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded marine dome over a rough, seaward-deepening bed)",
        "config": {"workload": f"{inst.name} {inst.nx}x{inst.ny}x{inst.nz} dx={inst.dx/1e3:g}km cold DIVA solve",
                   "picard_tol": inst.par.ssa_iter_conv, "lin": inst.par.lis_opt},
        "latency_ms": {"p50": 1e3 * float(np.percentile(times, 50)), "p99": 1e3 * float(np.percentile(times, 99))},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": f"{len(times)} full solves of the workload (oracle: C FP64 restatement, OpenMP)"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "picard_iters": out["ssa_iter_now"], "lin_iters": out["ssa_lin_iter"],
    }
    return line


def cpu_baseline_leg(inst, budget_s=20.0):
    """Oracle timed on the host cores (bounded sample), and its tightly converged
    solution as the checker of the GPU results."""
    import oracle
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    f0 = oracle.prepare(inst)
    times = []
    t_all = time.perf_counter()
    while True:
        f = {k: (v.copy(order="F") if isinstance(v, np.ndarray) else v) for k, v in f0.items()}
        t = time.perf_counter()
        oracle.calc_velocity(f, inst)
        times.append(time.perf_counter() - t)
        if time.perf_counter() - t_all > budget_s or len(times) >= 5:
            break
    tight = {k: (v.copy(order="F") if isinstance(v, np.ndarray) else v) for k, v in f0.items()}
    par_t = inst.par.with_(ssa_iter_max=600, ssa_iter_conv=1e-10,
                           ssa_lis_opt_energy="-i cg -p jacobi -maxiter 20000 -tol 1.0e-12",
                           ssa_lis_opt_residual="-i bicgstab -p jacobi -maxiter 20000 -tol 1.0e-12")
    oracle.calc_velocity(tight, inst, par_t)
    base = {"value": len(times) / sum(times), "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": f"{len(times)} full solves of the same workload (oracle: C FP64 restatement, "
                      f"OpenMP, {cores} threads)"}
    return base, tight, f0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="marine_diva")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    inst = bench_instance(args.workload)

    if args.impl == "reference":
        line = run_reference(args, inst, rank, world)
        if line is not None:
            print(json.dumps(line))
        return

    import torch
    from yelmo_gb300 import abi, gpu

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")

    cpu_base, tight, f_host = (None, None, None)
    if rank == 0 and not args.no_cpu:
        cpu_base, tight, f_host = cpu_baseline_leg(inst)
    if f_host is None:
        f_host = gpu.prepare(inst)
    nx, ny, nz = inst.nx, inst.ny, inst.nz
    kind = inst.par.kind

    dev = gpu.to_device(f_host, f"cuda:{local}")
    pristine = {k: dev[k].clone() for k in gpu.STATE_NAMES}
    fields = gpu.make_fields(dev, nx, ny, nz, inst.dx, inst.dx, inst.n_glen)
    solver = gpu.DeviceSolver(local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def reset():
        for k in gpu.STATE_NAMES:
            dev[k].copy_(pristine[k])
        for k in ("ux", "uy", "ux_i", "uy_i", "duxdz", "duydz"):
            dev[k].zero_()

    def run(par, steps, warmup):
        res = []
        for s in range(warmup + steps):
            reset()
            flush.zero_()             # L2 flush between timed solves
            torch.cuda.synchronize()
            st = solver.solve(kind, par, fields)
            if s >= warmup:
                res.append(st)
        return res

    results = {}
    for prec in ("fp64", "mixed"):
        par = inst.par.with_(precision=prec)
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        clk = ClockSampler(local)
        if prec == "mixed":
            clk.start()
        t0 = time.perf_counter()
        sts = run(par, args.steps, args.warmup)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        clocks = clk.stop() if prec == "mixed" else None
        ms = [s["device_ms"] for s in sts]
        u = {k: dev[k].cpu().numpy().reshape((nx, ny), order="F") for k in ("ux_bar", "uy_bar")}
        err = None
        if tight is not None:
            err = max(rel_l2(u["ux_bar"], tight["ux_bar"]), rel_l2(u["uy_bar"], tight["uy_bar"]))
        tot_ms = sum(ms)
        if dist is not None:
            t = torch.tensor([tot_ms], device=f"cuda:{local}")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            tot_ms = float(t.item())
        results[prec] = {"ms": ms, "tot_ms": tot_ms, "stats": sts[-1], "err": err, "clocks": clocks,
                         "wall": wall}

    # e2e: the C-ABI drop-in from host buffers (copies inside the timed region)
    e2e_times = []
    par_m = inst.par.with_(precision="mixed")
    for s in range(args.warmup + max(3, args.steps // 2)):
        f = {k: (v.copy(order="F") if isinstance(v, np.ndarray) else v) for k, v in f_host.items()}
        t = time.perf_counter()
        gpu.calc_velocity(f, inst.dx, inst.n_glen, par_m)
        dt = time.perf_counter() - t
        if s >= args.warmup:
            e2e_times.append(dt)
    h2d, d2h = gpu.host_io_bytes(kind, nx, ny, nz)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    mixed, fp64 = results["mixed"], results["fp64"]
    K = len(mixed["ms"])
    value = world * K / (mixed["tot_ms"] / 1e3)
    st = mixed["stats"]
    alg = gpu.algorithmic_bytes(st, kind, nx, ny, nz, mixed=True, energy=inst.par.ssa_solver == "energy")
    avg_ms = statistics.mean(mixed["ms"])
    achieved = alg / (avg_ms / 1e3) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    alg64 = gpu.algorithmic_bytes(fp64["stats"], kind, nx, ny, nz, mixed=False)
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": avg_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/f64 (FP32 Krylov, FP64 defect correction)",
        "data": "synthetic (seeded marine dome over a rough, seaward-deepening bed)",
        "config": {"workload": f"{inst.name} {nx}x{ny}x{nz} dx={inst.dx/1e3:g}km cold DIVA solve",
                   "picard_tol": inst.par.ssa_iter_conv, "lin": inst.par.lis_opt,
                   "l2": "flushed (256 MB write) between timed solves", "parallelism": f"replicas x{world}"},
        "latency_ms": {"p50": float(np.percentile(mixed["ms"], 50)), "p99": float(np.percentile(mixed["ms"], 99))},
        "fp64": {"value": world * len(fp64["ms"]) / (fp64["tot_ms"] / 1e3), "unit": "solves/s",
                 "ms_per_step": statistics.mean(fp64["ms"]),
                 "latency_ms": {"p50": float(np.percentile(fp64["ms"], 50)),
                                "p99": float(np.percentile(fp64["ms"], 99))},
                 "rel_err_vs_oracle": fp64["err"], "picard_iters": fp64["stats"]["ssa_iter_now"],
                 "lin_iters": fp64["stats"]["ssa_lin_iter"],
                 "achieved_gbs": alg64 / (statistics.mean(fp64["ms"]) / 1e3) / 1e9},
        "mixed_over_fp64": (statistics.mean(fp64["ms"]) / avg_ms),
        "rel_err_vs_oracle": mixed["err"],
        "picard_iters": st["ssa_iter_now"], "lin_iters": st["ssa_lin_iter"], "outer_iters": st["outer_iter"],
        "gpu_launches": K,
        "e2e": {"value": 1.0 / statistics.mean(e2e_times), "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "path": "ygpu_calc_velocity_diva (host buffers)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": "ygpu_solve_kernel (whole Picard solve, one launch)",
                     "note": "peak = measured copy bandwidth (MEASURED_PEAKS.json hbm_gbs)"},
        "clocks": mixed["clocks"],
        "cpu_baseline": cpu_base,
    }
    print(json.dumps(line))
    solver.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
