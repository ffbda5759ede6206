"""Golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py):
small seeded solves of the oracle converged tightly, and the oracle's post-solve
diagnostics, velocity Jacobian and vertical velocity on seeded fields.

CPU: the oracle built here reproduces them (the masks bit for bit, the fields
to 1e-10), which pins it across compilers and machines. GPU: the GPU solver,
started from the fixture's input state, matches the fixture's outputs within
the parity bar without running the oracle."""
import os

import numpy as np
import pytest

from tests.cases import rel_l2
from tests.golden.make_golden import OUT_KEYS, POST_BCS, golden_cases, post_solve_outputs

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


def _load_post(bc):
    d = np.load(os.path.join(HERE, f"post_solve_{bc}.npz"))
    inputs = {k[3:]: np.asfortranarray(d[k]) for k in d.files if k.startswith("in_")}
    outputs = {k[4:]: d[k] for k in d.files if k.startswith("out_")}
    return inputs, outputs


def _check_post(got, want, tol):
    assert set(got) == set(want)
    for k, v in want.items():
        scale = float(np.max(np.abs(v))) if v.size else 0.0
        np.testing.assert_allclose(got[k], v, rtol=0, atol=tol * scale + 1e-300, err_msg=k)


@pytest.mark.parametrize("bc", POST_BCS)
def test_oracle_reproduces_post_solve_golden(bc):
    import oracle
    inputs, outputs = _load_post(bc)
    _check_post(post_solve_outputs(oracle, inputs, bc), outputs, 1e-14)


# The diagnostics evaluate the reference expressions as written (bit-exact with
# the oracle on one machine); the Jacobian and vertical-velocity kernels keep
# divisions out of their layer loops and agree to rounding.
@pytest.mark.gpu
@pytest.mark.parametrize("bc", POST_BCS)
def test_gpu_matches_post_solve_golden(bc):
    from yelmo_gb300 import gpu
    inputs, outputs = _load_post(bc)
    got = post_solve_outputs(gpu, inputs, bc)
    _check_post({k: v for k, v in got.items() if k.startswith("diag_")},
                {k: v for k, v in outputs.items() if k.startswith("diag_")}, 1e-14)
    _check_post({k: v for k, v in got.items() if not k.startswith("diag_")},
                {k: v for k, v in outputs.items() if not k.startswith("diag_")}, 1e-12)


def test_continent_fixture_matches_its_builder():
    """The full-size continent fixture (make_continent_golden.py) was solved on the
    inputs the seeded builder makes: the oracle's prologue here gives its masks bit
    for bit, and it stopped at the Picard limit."""
    import oracle
    from tests.golden.make_continent_golden import NAME, PICARD_ITERS, VEL_KEYS, continent_case
    d = np.load(os.path.join(HERE, NAME + ".npz"))
    f0 = oracle.prepare(continent_case())
    for k in ("ssa_mask_acx", "ssa_mask_acy"):
        np.testing.assert_array_equal(f0[k], d[k].astype(np.int32), err_msg=k)
    assert int(d["ssa_iter_now"]) == PICARD_ITERS
    for k in VEL_KEYS:
        assert d[k].shape == f0["H_ice"].shape and np.all(np.isfinite(d[k])), k
