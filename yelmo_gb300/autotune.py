"""Launch autotuner: picks a context's tuning (team size, host-check interval,
chunk graphs, lockstep batch or queue) for a workload by timing a fixed number
of Picard iterations of its batched solve under each candidate (and, for the
batch-or-queue choice, full solves). In mixed precision it also picks the inner
FP32 solve's tolerance (``inner_tol`` of the parameters) from ``inner_tols`` by
full solves: the outer FP64 defect correction reaches the requested linear
tolerance whatever the inner one, so the choice trades inner iterations against
outer steps and changes the time, not the answer's tolerance.

    best = autotune(solver, kind, par, fields, reset)

``fields`` are the device fields of the batch (gpu.make_fields), ``reset()``
restores their state between trials (the solves update it in place). Every
trial runs exactly ``iters`` Picard iterations (no convergence exit), so the
trials do equal work. The chosen tuning is left set on the solver.
"""
from __future__ import annotations

import itertools
import time

DEFAULT_GRID = {
    "unknowns_per_cta": (256, 512, 1024, 2048),
    "check_every": (4, 8),
    "use_graphs": (True,),
}


DEFAULT_INNER_TOLS = (5e-4, 1e-3, 2e-3, 4e-3)


def autotune(solver, kind: int, par, fields: list, reset, iters: int = 8, grid: dict | None = None,
             reps: int = 1, inner_tols=DEFAULT_INNER_TOLS) -> dict:
    import torch
    grid = grid or DEFAULT_GRID
    trial_par = par.with_(ssa_iter_max=iters, ssa_iter_conv=0.0)
    results = []
    keys = list(grid)
    for values in itertools.product(*(grid[k] for k in keys)):
        cand = dict(zip(keys, values))
        solver.set_tuning(**cand)
        best = float("inf")
        for _ in range(reps + 1):          # the first run captures the chunk graph
            reset()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            solver.solve_batch(kind, trial_par, fields)
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        results.append((best, cand))
    results.sort(key=lambda r: r[0])
    best_t, best = results[0]
    # graphs on/off at the chosen shape
    for g in (False,):
        cand = dict(best, use_graphs=g)
        solver.set_tuning(**cand)
        t = float("inf")
        for _ in range(reps + 1):
            reset()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            solver.solve_batch(kind, trial_par, fields)
            torch.cuda.synchronize()
            t = min(t, time.perf_counter() - t0)
        if t < best_t:
            best_t, best = t, cand
    # lockstep batch or queue (continuous batching): full solves with the real
    # convergence test, since the queue's gain comes from instances that finish
    # at different iterations
    total_nu = sum(2 * f.nx * f.ny for f in fields)
    if len(fields) > 1 and total_nu > 1_500_000:
        full = []
        for U in (1_500_000, 4_000_000, 0):
            cand = dict(best, max_active_unknowns=U)
            solver.set_tuning(**cand)
            reset()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            solver.solve_batch(kind, par, fields)
            torch.cuda.synchronize()
            full.append((time.perf_counter() - t0, cand))
        full.sort(key=lambda r: r[0])
        best = full[0][1]
    solver.set_tuning(**best)
    # the inner tolerance of the mixed mode, by full solves at the chosen tuning
    inner = None
    if par.precision == "mixed" and inner_tols:
        timed = []
        for tol in inner_tols:
            p = par.with_(inner_tol=tol)
            t = float("inf")
            for _ in range(reps + 1):
                reset()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                solver.solve_batch(kind, p, fields)
                torch.cuda.synchronize()
                t = min(t, time.perf_counter() - t0)
            timed.append((t, tol))
        timed.sort(key=lambda r: r[0])
        inner = {"inner_tol": timed[0][1], "ms": {f"{tol:g}": t * 1e3 for t, tol in timed}}
    reset()
    return {"tuning": best, "trial_ms": best_t * 1e3, "iters": iters,
            "candidates": [{"ms": r[0] * 1e3, **r[1]} for r in results],
            "inner_tol": inner["inner_tol"] if inner else None, "inner_tol_ms": inner["ms"] if inner else None}
