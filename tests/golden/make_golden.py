"""Writes the golden fixtures of this directory: small seeded solves of the
oracle (the FP64 restatement of the reference path), converged tightly.

    python tests/golden/make_golden.py

Each fixture holds the solve's input state (after the calc_ydyn prologue and
the SSA masks) and its outputs. tests/test_golden.py checks that the oracle
still reproduces them (CPU) and that the GPU solver matches them (GPU), so the
GPU parity does not depend on building the oracle on the machine that runs it.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

OUT_KEYS = ("ux_b", "uy_b", "ux_bar", "uy_bar", "visc_eff", "visc_eff_int", "taub_acx", "taub_acy",
            "beta_acx", "beta_acy", "ssa_mask_acx", "ssa_mask_acy")


def golden_cases():
    from tests.cases import TIGHT
    from yelmo_gb300 import configs
    dome = configs.dome_ssa(n=25, nz=4)
    dome.par = dome.par.with_(**TIGHT)
    marine = configs.marine_diva(n=25, nz=4)
    marine.par = marine.par.with_(**TIGHT)
    return {"dome_ssa_residual_25": dome, "marine_diva_energy_25": marine}


def main():
    import oracle
    for name, inst in golden_cases().items():
        f0 = oracle.prepare(inst)
        f = {k: (v.copy(order="F") if isinstance(v, np.ndarray) else v) for k, v in f0.items()}
        out = oracle.calc_velocity(f, inst)
        data = {"in_" + k: v for k, v in f0.items() if isinstance(v, np.ndarray)}
        data.update({"out_" + k: f[k] for k in OUT_KEYS if k in f})
        data["ssa_iter_now"] = np.array(out["ssa_iter_now"])
        data["status"] = np.array(out["status"])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
        print(name, out)


if __name__ == "__main__":
    main()
