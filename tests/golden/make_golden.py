"""Writes the golden fixtures of this directory: small seeded solves of the
oracle (the FP64 restatement of the reference path), converged tightly, and
the oracle's post-solve diagnostics, velocity Jacobian and vertical velocity
on seeded fields (post_solve_*.npz).

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


POST_BCS = ("zeros", "periodic")
POST_DX = (8e3, 6e3)


def post_solve_inputs(bc: str) -> dict:
    """Seeded fields, with ice margins, for the routines around the solve:
    post-solve diagnostics, velocity Jacobian, vertical velocity (12 x 10 cells,
    5 layers, 6 interfaces)."""
    nx, ny, nz = 12, 10, 5
    r = np.random.default_rng(2024 + POST_BCS.index(bc))
    F = lambda *s: np.asfortranarray(r.normal(size=s))
    f = r.choice([0.0, 0.4, 1.0, 1.0, 1.0, 1.0], size=(nx, ny))
    a = {"f_ice": np.asfortranarray(f),
         "H_ice": np.asfortranarray(np.where(f > 0, 500.0 + np.abs(F(nx, ny)) * 1000.0, 0.0)),
         "f_grnd": np.asfortranarray(r.choice([0.0, 0.3, 1.0, 1.0], size=(nx, ny)))}
    for n in ("ux", "uy", "ux_i", "uy_i"):
        a[n] = F(nx, ny, nz) * 100.0
    a["uz"] = F(nx, ny, nz + 1)
    for n in ("ux_bar", "uy_bar", "ux_b", "uy_b"):
        a[n] = F(nx, ny) * 50.0
    for n in ("taub_acx", "taub_acy", "taud_acx", "taud_acy"):
        a[n] = F(nx, ny) * 1e4
    for n in ("smb", "bmb", "dzbdt", "dzsdt", "dHidt_dyn"):
        a[n] = F(nx, ny) * 0.5
    for n in ("dzsdx", "dzsdy", "dzbdx", "dzbdy"):
        a[n] = F(nx, ny) * 1e-2
    a["mask_kin"] = np.asfortranarray(r.integers(0, 2, size=(nx, ny)).astype(np.int32))
    a["zeta_aa"] = np.linspace(0.0, 1.0, nz) ** 1.6
    a["zeta_ac"] = np.concatenate([[0.0], 0.5 * (a["zeta_aa"][1:] + a["zeta_aa"][:-1]), [1.0]])
    return a


def post_solve_outputs(impl, a: dict, bc: str) -> dict:
    """The routines around the solve on the fields of post_solve_inputs, through
    `impl` (the oracle module or yelmo_gb300.gpu): name -> array."""
    from yelmo_gb300 import abi, gpu
    dx, dy = POST_DX
    nz = a["ux"].shape[2]
    out = {}
    d = gpu.diagnostics_arrays(a, nz)
    impl.calc_dyn_diagnostics(d, dx, dy, bc)
    out.update({"diag_" + k: d[k] for k in abi.DIAG_OUTPUTS if k in d})
    j = impl.calc_jacobian_vel_3D(gpu.jacobian_arrays(a), dx, dy, bc, abi.JAC_UXY | abi.JAC_UZ)
    out.update({"jac_" + k: j[k] for k in abi.JAC_OUTPUTS})
    for name, method in (("uzaa", abi.UZ_AA), ("uzflux", abi.UZ_FLUX)):
        u = impl.calc_uz_3D(gpu.uz_arrays(a), dx, dy, bc, method)
        out.update({name + "_" + k: u[k] for k in abi.UZ_OUTPUTS})
    return out


def main():
    import oracle
    for bc in POST_BCS:
        a = post_solve_inputs(bc)
        out = post_solve_outputs(oracle, a, bc)
        data = {"in_" + k: v for k, v in a.items()}
        data.update({"out_" + k: v for k, v in out.items()})
        np.savez_compressed(os.path.join(HERE, f"post_solve_{bc}.npz"), **data)
        print("post_solve", bc, len(out), "outputs")
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
