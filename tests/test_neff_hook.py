"""neff_hook of calc_velocity_diva (velocity_diva.f90:390-400): after every
Picard iteration a host hook recomputes c_bed from the basal velocity (a steady
hydrology's effective pressure), and the solve converges only when c_bed has
settled too. The hook here is a deterministic stand-in for K24: the bed
weakens with sliding speed, c_bed = c0 / (1 + |u_b| / 200 m/a)."""
import numpy as np
import pytest

import oracle
from tests.cases import case, rel_l2
from tests.test_gpu_parity import _copy, _prepare_shared


def _case():
    return case("continent_diva")        # power-law friction on c_bed (q = 0.5)


def _speed_hook(c0, calls):
    def hook(c_bed, ux_b, uy_b):
        calls.append(1)
        speed = np.sqrt(ux_b * ux_b + uy_b * uy_b)
        c_bed[...] = c0 / (1.0 + speed / 200.0)
    return hook


def test_oracle_noop_hook_changes_nothing():
    inst = _case()
    f0 = _prepare_shared(inst)
    fa, fb = _copy(f0), _copy(f0)
    outa = oracle.calc_velocity(fa, inst)
    calls = []
    outb = oracle.calc_velocity(fb, inst, neff_hook=lambda cb, ub, vb: calls.append(1))
    assert outa["ssa_iter_now"] == outb["ssa_iter_now"] == len(calls)
    for k in ("ux_bar", "uy_bar", "visc_eff"):
        np.testing.assert_array_equal(fa[k], fb[k])


def test_oracle_hook_couples_friction():
    inst = _case()
    f0 = _prepare_shared(inst)
    fa, fb = _copy(f0), _copy(f0)
    outa = oracle.calc_velocity(fa, inst)
    calls = []
    outb = oracle.calc_velocity(fb, inst, neff_hook=_speed_hook(f0["c_bed"].copy(), calls))
    assert outb["status"] == 0 and len(calls) == outb["ssa_iter_now"]
    assert rel_l2(fb["ux_bar"], fa["ux_bar"]) > 1e-3         # weaker bed, faster ice
    assert not np.array_equal(fb["c_bed"], f0["c_bed"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_hook_matches_oracle(precision):
    from yelmo_gb300 import gpu
    inst = _case()
    f0 = _prepare_shared(inst)
    fo, fg = _copy(f0), _copy(f0)
    calls_o, calls_g = [], []
    outo = oracle.calc_velocity(fo, inst, neff_hook=_speed_hook(f0["c_bed"].copy(), calls_o))
    # mixed precision: FP32 noise keeps the relative L1 change of c_bed near
    # 1e-8, so it runs to the bench's Picard tolerance (1e-7) instead of 1e-9
    par = inst.par.with_(precision=precision)
    if precision == "mixed":
        par = par.with_(ssa_iter_conv=1e-7)
    outg = gpu.calc_velocity(fg, inst.dx, inst.n_glen, par, neff_hook=_speed_hook(f0["c_bed"].copy(), calls_g))
    assert outg["status"] == 0
    assert len(calls_g) == outg["ssa_iter_now"] < par.ssa_iter_max
    if precision == "fp64":
        assert abs(outg["ssa_iter_now"] - outo["ssa_iter_now"]) <= 2
    for k in ("ux_bar", "uy_bar", "ux_b", "uy_b", "visc_eff", "c_bed"):
        assert rel_l2(fg[k], fo[k]) <= 1e-6, (k, rel_l2(fg[k], fo[k]))


@pytest.mark.gpu
def test_gpu_noop_hook_equals_plain_solve():
    from yelmo_gb300 import gpu
    inst = _case()
    f0 = _prepare_shared(inst)
    fa, fb = _copy(f0), _copy(f0)
    outa = gpu.calc_velocity(fa, inst.dx, inst.n_glen, inst.par)
    calls = []
    outb = gpu.calc_velocity(fb, inst.dx, inst.n_glen, inst.par, neff_hook=lambda cb, ub, vb: calls.append(1))
    assert outa["ssa_iter_now"] == outb["ssa_iter_now"] == len(calls)
    for k in ("ux_bar", "uy_bar", "visc_eff"):
        assert rel_l2(fb[k], fa[k]) <= 1e-12, k


@pytest.mark.gpu
def test_gpu_hook_through_batch_host_entry():
    """ygpu_solve_batch_host with one DIVA state and a hook: the same solve as the
    drop-in with the hook, and c_bed comes back with the hook's last update."""
    from yelmo_gb300 import gpu
    inst = _case()
    f0 = _prepare_shared(inst)
    fa, fb = _copy(f0), _copy(f0)
    calls_a, calls_b = [], []
    outa = gpu.calc_velocity(fa, inst.dx, inst.n_glen, inst.par, neff_hook=_speed_hook(f0["c_bed"].copy(), calls_a))
    stb = gpu.calc_velocity_batch([fb], [inst.dx], inst.n_glen, inst.par,
                                  neff_hook=_speed_hook(f0["c_bed"].copy(), calls_b))[0]
    assert stb["status"] == 0 and stb["ssa_iter_now"] == outa["ssa_iter_now"] == len(calls_b)
    assert not np.array_equal(fb["c_bed"], f0["c_bed"])
    for k in ("ux_bar", "uy_bar", "visc_eff", "c_bed"):
        assert rel_l2(fb[k], fa[k]) <= 1e-12, k
