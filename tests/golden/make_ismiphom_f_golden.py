"""Writes tests/golden/ismiphom_f_steady.npz: the oracle's ISMIP-HOM experiment F
runs (F1 no slip, F2 slip ratio 1; 40 x 40 cells, dx 2.5 km, 10 sigma layers) through
the thickness time loop of yelmo_gb300.prognostic.

    python tests/golden/make_ismiphom_f_golden.py [threads]

Each experiment runs 2000 years in 1-year backward-Euler thickness steps with the
velocity solved after every step. Two linear-solve settings:

* "tight": CG with a relative residual of 1e-8 in every Picard iteration, so the
  state does not depend on the Krylov path; the GPU run must match it to 1e-6.
* "nml":   the namelist's own "-i cg -p jacobi -maxiter 200 -tol 1.0e-2"
  (par/yelmo_ISMIPHOM.nml). A warm-started solve then often stops after zero CG
  iterations, so the velocity follows the thickness in steps and which step
  triggers a new iteration depends on rounding; the GPU run is compared with it
  on the steady surface only, at a looser bound.

Stored per experiment and setting: z_srf and the surface speed on the aa-nodes
(us_aa) after 100 years and after 2000 years, float64 (40 x 40 each), and max
|dH/dt| of the last step. About 10 s per run on 4 threads.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NAME = "ismiphom_f_steady"
DT = 1.0
T_SHORT = 100.0
T_END = 2000.0
LIS_TIGHT = "-i cg -p jacobi -maxiter 1000 -tol 1.0e-8 -initx_zeros false"


def case(exp: int, setting: str):
    """ISMIP-HOM F of experiment exp with the linear-solve setting ("tight" or "nml")."""
    from yelmo_gb300 import configs
    inst = configs.ismiphom_f(exp)
    if setting == "tight":
        inst.par = inst.par.with_(ssa_lis_opt_energy=LIS_TIGHT)
    elif setting != "nml":
        raise ValueError(setting)
    return inst


class OracleBackend:
    """The oracle's restatement of the four calls of one time step."""

    def __init__(self):
        import oracle
        self.o = oracle

    def inputs(self, inst):
        return self.o.calc_dyn_inputs(inst)

    def masks(self, *a):
        return self.o.set_ssa_masks(*a)

    def velocity(self, fields, inst):
        return self.o.calc_velocity(fields, inst)

    def advect(self, H, ux, uy, smb, mask_ice, H_ref, dx, dt, boundaries):
        return self.o.calc_advec2D_impl_lis(H, ux, uy, smb, mask_ice, H_ref, dx, dx, dt, boundaries)


def main():
    import oracle
    from yelmo_gb300 import prognostic
    oracle.set_threads(int(sys.argv[1]) if len(sys.argv) > 1 else 4)
    data = {}
    for exp in (1, 2):
        for setting in ("tight", "nml"):
            key = f"f{exp}_{setting}"
            snap = {}

            def keep(k, t, f, dHdt):
                if abs(t - T_SHORT) < 1e-9:
                    snap["z_srf"] = f["z_srf"].copy()
                    snap["us_aa"] = prognostic.surface_speed_aa(f["ux"][:, :, -1], f["uy"][:, :, -1])

            t0 = time.time()
            r = prognostic.run(case(exp, setting), DT, T_END, backend=OracleBackend(), on_step=keep)
            print(key, r["steps"], "steps", f"{time.time() - t0:.1f} s",
                  "max|dH/dt|", r["history"]["dhdt_max"][-1])
            data[f"{key}_zs_100"] = snap["z_srf"]
            data[f"{key}_us_100"] = snap["us_aa"]
            data[f"{key}_zs"] = r["z_srf"]
            data[f"{key}_us"] = r["us_aa"]
            data[f"{key}_dhdt_last"] = np.float64(r["history"]["dhdt_max"][-1])
    np.savez_compressed(os.path.join(HERE, NAME + ".npz"), **data)


if __name__ == "__main__":
    main()
