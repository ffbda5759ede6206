"""One batched solve of a benchmark workload, for profilers.

    python -m yelmo_gb300.profile_case --workload marine_diva --batch 16 --precision mixed

Runs a single batched solve (no warm-up, no timing loop) so that a profiler can
select launches by kernel name and index. With --log every instance prints its
per-Picard-iteration line ("ssa: <iter> <resid> | lin <iterations> <status>"),
which gives the linear iterations of each step kernel launch.
"""
from __future__ import annotations

import argparse
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

TOL = dict(ssa_iter_max=300, ssa_iter_conv=1e-7,
           ssa_lis_opt_energy="-i cg -p jacobi -maxiter 5000 -tol 1.0e-9 -initx_zeros false",
           ssa_lis_opt_residual="-i bicgstab -p jacobi -maxiter 5000 -tol 1.0e-9 -initx_zeros false")


def instances(workload: str, batch: int, n: int = 0):
    from yelmo_gb300 import configs
    if workload == "marine_diva":
        return [configs.marine_diva(seed=2024 + b, **({"n": n} if n else {})) for b in range(batch)]
    if workload == "continent_diva":
        return [configs.continent_diva(seed=4242 + b, **({"n": n} if n else {})) for b in range(batch)]
    if workload == "dome_ssa":
        return [configs.dome_ssa(seed=1234 + b, **({"n": n} if n else {})) for b in range(batch)]
    if workload == "ensemble":
        return [configs.ensemble_member(i) for i in range(batch)]
    raise SystemExit(f"unknown workload {workload}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="marine_diva")
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--n", type=int, default=0, help="grid side (default: the workload's)")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--log", action="store_true")
    args = ap.parse_args()
    import torch
    from yelmo_gb300 import gpu
    insts = instances(args.workload, args.batch, args.n)
    for inst in insts:
        inst.par = inst.par.with_(**TOL).with_(precision=args.precision, ssa_write_log=args.log)
    devs = [gpu.to_device(gpu.prepare(i)) for i in insts]
    fields = [gpu.make_fields(d, i.nx, i.ny, i.nz, i.dx, i.dx, i.n_glen) for d, i in zip(devs, insts)]
    solver = gpu.DeviceSolver(0)
    torch.cuda.synchronize()
    sts = solver.solve_batch(insts[0].par.kind, insts[0].par, fields)
    torch.cuda.synchronize()
    print("picard", [s["ssa_iter_now"] for s in sts], "lin", [s["ssa_lin_iter"] for s in sts],
          "status", sorted(set(s["status"] for s in sts)))
    solver.close()


if __name__ == "__main__":
    main()
