"""Writes tests/golden/continent_diva_801_picard20.npz: the oracle's answer on the
continent-scale DIVA workload at its full size (801 x 801 cells, dx 4 km, 20 sigma
layers, power-law friction with q = 1/3).

    python tests/golden/make_continent_golden.py [threads]

That workload has no tightly converged answer: its Picard iteration settles into a
cycle whose relative change stays near 2e-3 (at 101 x 101 the same happens with
q = 0.5 and with beta_min = 0, so the floor on beta is not its cause). The comparison
is therefore a Picard-limit one. Both solvers stop after the namelist's 20 Picard
iterations (ssa_iter_max = 20) with every linear solve converged to a relative
residual of 1e-12, so the answer does not depend on the Krylov path: the oracle's
Jacobi-CG and ILU(0)-CG answers agree to 1e-10 there.

The fixture holds the 2D velocities (ux_bar, uy_bar, ux_b, uy_b) as float32, which
rounds them at 6e-8 relative, far inside the 1e-6 parity bar, and the SSA masks as
int8 so that a test can check that the inputs it rebuilds from the seeded builder
have the same discrete structure (flotation and ice masks) as the ones the oracle
solved. The oracle takes several minutes here on 8 threads; the GPU test reads the
fixture instead of running it.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NAME = "continent_diva_801_picard20"
PICARD_ITERS = 20
LIN_TOL = 1e-12
VEL_KEYS = ("ux_bar", "uy_bar", "ux_b", "uy_b")


def continent_case(n: int = 801, nz: int = 20):
    """The full-size continent workload with the Picard-limit settings."""
    from yelmo_gb300 import configs
    inst = configs.continent_diva(n=n, nz=nz)
    inst.par = inst.par.with_(
        ssa_iter_max=PICARD_ITERS, ssa_iter_conv=1e-12,
        ssa_lis_opt_energy=f"-i cg -p jacobi -maxiter 50000 -tol {LIN_TOL:.1e}")
    return inst


def main():
    import oracle
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else os.cpu_count()
    oracle.set_threads(threads)
    inst = continent_case()
    f = oracle.prepare(inst)
    t = time.time()
    out = oracle.calc_velocity(f, inst)
    print(NAME, out, f"{time.time() - t:.1f} s")
    assert out["status"] == 0 and out["ssa_iter_now"] == PICARD_ITERS, out
    data = {k: f[k].astype(np.float32) for k in VEL_KEYS}
    data["ssa_mask_acx"] = f["ssa_mask_acx"].astype(np.int8)
    data["ssa_mask_acy"] = f["ssa_mask_acy"].astype(np.int8)
    data["ssa_iter_now"] = np.array(out["ssa_iter_now"])
    np.savez_compressed(os.path.join(HERE, NAME + ".npz"), **data)


if __name__ == "__main__":
    main()
