"""Golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py):
small seeded solves of the oracle converged tightly.

CPU: the oracle built here reproduces them (the masks bit for bit, the fields
to 1e-10), which pins it across compilers and machines. GPU: the GPU solver,
started from the fixture's input state, matches the fixture's outputs within
the parity bar without running the oracle."""
import os

import numpy as np
import pytest

from tests.cases import rel_l2
from tests.golden.make_golden import OUT_KEYS, golden_cases

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = sorted(golden_cases())


def _load(name):
    d = np.load(os.path.join(HERE, name + ".npz"))
    inputs = {k[3:]: np.asfortranarray(d[k]) for k in d.files if k.startswith("in_")}
    outputs = {k[4:]: d[k] for k in d.files if k.startswith("out_")}
    return inputs, outputs, int(d["ssa_iter_now"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(name):
    import oracle
    inst = golden_cases()[name]
    inputs, outputs, iters = _load(name)
    f0 = oracle.prepare(inst)
    for k in ("ssa_mask_acx", "ssa_mask_acy", "mask_frnt", "f_ice", "f_grnd", "H_grnd"):
        np.testing.assert_array_equal(f0[k], inputs[k], err_msg=k)
    f = {k: (v.copy(order="F") if isinstance(v, np.ndarray) else v) for k, v in f0.items()}
    out = oracle.calc_velocity(f, inst)
    assert out["status"] == 0 and out["ssa_iter_now"] == iters
    for k in OUT_KEYS:
        if k in outputs:
            if outputs[k].dtype.kind == "i":
                np.testing.assert_array_equal(f[k], outputs[k], err_msg=k)
            else:
                assert rel_l2(f[k], outputs[k]) <= 1e-10, k


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_golden(name, precision):
    from yelmo_gb300 import gpu
    inst = golden_cases()[name]
    inputs, outputs, _ = _load(name)
    f = {k: v.copy(order="F") for k, v in inputs.items()}
    out = gpu.calc_velocity(f, inst.dx, inst.n_glen, inst.par.with_(precision=precision))
    assert out["status"] == 0
    vel = ("ux_b", "uy_b") if inst.par.solver == "ssa" else ("ux_bar", "uy_bar", "ux_b", "uy_b")
    for k in vel + ("visc_eff", "visc_eff_int", "taub_acx", "taub_acy"):
        assert rel_l2(f[k], outputs[k]) <= 1e-6, (k, rel_l2(f[k], outputs[k]))
