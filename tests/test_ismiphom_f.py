"""ISMIP-HOM experiment F (tests/yelmo_ismiphom.f90:149-186, par/yelmo_ISMIPHOM.nml): a
slab on a 3 degree background slope over a Gaussian bed bump relaxing to steady state,
through the thickness time loop of yelmo_gb300.prognostic (advection, the prologue with
the background slope, the DIVA solve).

CPU: the background slope in the oracle's prologue, the unperturbed slab against its
analytic surface speed, and the first century of the oracle's loop against the
committed fixture (tests/golden/make_ismiphom_f_golden.py), with mass conserved.
GPU: the background-slope prologue bit-exact, the slab, and the full 2000-year runs
of F1 and F2 against the oracle's fixture."""
import os

import numpy as np
import pytest

import oracle
from tests.golden.make_ismiphom_f_golden import DT, LIS_TIGHT, T_END, T_SHORT, OracleBackend, case
from yelmo_gb300 import configs, prognostic

FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "ismiphom_f_steady.npz")


def _slab(exp, bump=0.0):
    inst = configs.ismiphom_f(exp, bump=bump)
    inst.par = inst.par.with_(ssa_lis_opt_energy=LIS_TIGHT)
    return inst


def _zs_err(a, b):
    """z_srf difference relative to the surface relief of b."""
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _us_err(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_background_slope_in_oracle_prologue():
    inst = configs.ismiphom_f(1)
    s = inst.slope_bg[0]
    flat = configs.ismiphom_f(1)
    flat.slope_bg = (0.0, 0.0)
    a = oracle.calc_dyn_inputs(inst)
    b = oracle.calc_dyn_inputs(flat)
    assert np.allclose(a["dzsdx"], b["dzsdx"] + s, rtol=0, atol=1e-15)
    assert np.array_equal(a["dzsdy"], b["dzsdy"])
    # on the unperturbed slab the driving stress is rho g H0 tan(alpha) down the slope
    d = oracle.calc_dyn_inputs(configs.ismiphom_f(1, bump=0.0))
    rhog = inst.par.rho_ice * inst.par.g
    assert np.allclose(d["taud_acx"], rhog * 1000.0 * s, rtol=1e-12)
    # the slope is added before the limit (yelmo_tools.f90:400-404)
    lim = configs.ismiphom_f(1)
    lim.par = lim.par.with_(grad_lim=0.04)
    c = oracle.calc_dyn_inputs(lim)
    assert np.all(c["dzsdx"] == -0.04)


@pytest.mark.parametrize("exp", [1, 2])
def test_slab_surface_speed_oracle(exp):
    inst = _slab(exp)
    r = prognostic.run(inst, DT, 1.0, backend=OracleBackend())
    u = inst.extra["u_s_slab"]
    assert np.max(np.abs(r["us_aa"] / u - 1.0)) < 1e-5
    ub = r["fields"]["ux_b"]
    if exp == 1:
        assert np.all(ub == 0.0)
    else:      # slip ratio 1: the basal speed is the deformation speed
        assert np.max(np.abs(ub / (0.5 * u) - 1.0)) < 1e-5


@pytest.mark.parametrize("exp", [1, 2])
def test_oracle_first_century_matches_fixture(exp):
    g = np.load(FIXTURE)
    inst = case(exp, "tight")
    r = prognostic.run(inst, DT, T_SHORT, backend=OracleBackend())
    assert r["steps"] == int(T_SHORT / DT)
    assert _zs_err(r["z_srf"], g[f"f{exp}_tight_zs_100"]) < 1e-9
    assert _us_err(r["us_aa"], g[f"f{exp}_tight_us_100"]) < 1e-9
    # zero mass balance on a periodic domain: the volume is conserved
    v0, v1 = inst.H_ice.sum(), r["H_ice"].sum()
    assert abs(v1 - v0) / v0 < 1e-12


def test_fixture_is_near_steady():
    g = np.load(FIXTURE)
    for exp in (1, 2):
        assert float(g[f"f{exp}_tight_dhdt_last"]) < 1e-4
        # the hump upstream of the bump and the trough downstream
        zs = g[f"f{exp}_tight_zs"][:, 20]
        x = configs.ismiphom_f(exp).extra["x"]
        assert -10e3 < x[np.argmax(zs)] < 0.0 < 10e3 < x[np.argmin(zs)] < 20e3


@pytest.mark.gpu
def test_prologue_background_slope_bit_exact():
    from yelmo_gb300 import gpu
    for exp, bc, lim in ((1, "periodic", 0.5), (2, "periodic", 0.04), (1, "infinite", 0.5), (1, "zeros", 0.5)):
        inst = configs.ismiphom_f(exp)
        inst.slope_bg = (inst.slope_bg[0], 0.013)
        inst.par = inst.par.with_(boundaries=bc, grad_lim=lim)
        a = oracle.calc_dyn_inputs(inst)
        b = gpu.calc_dyn_inputs(inst)
        for k in a:
            assert np.array_equal(a[k], b[k]), (exp, bc, k)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("exp", [1, 2])
def test_slab_surface_speed_gpu(exp, precision):
    inst = _slab(exp)
    inst.par = inst.par.with_(precision=precision)
    r = prognostic.run(inst, DT, 1.0)
    assert np.max(np.abs(r["us_aa"] / inst.extra["u_s_slab"] - 1.0)) < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("exp", [1, 2])
def test_steady_state_matches_oracle(exp, precision):
    """2000 years of F1 / F2 on the GPU against the oracle's run, linear solves at 1e-8."""
    g = np.load(FIXTURE)
    inst = case(exp, "tight")
    inst.par = inst.par.with_(precision=precision)
    r = prognostic.run(inst, DT, T_END)
    assert r["steps"] == int(T_END / DT)
    assert _zs_err(r["z_srf"], g[f"f{exp}_tight_zs"]) < 1e-6
    assert _us_err(r["us_aa"], g[f"f{exp}_tight_us"]) < 1e-6
    assert r["history"]["dhdt_max"][-1] < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("exp", [1, 2])
def test_steady_state_namelist_solver(exp):
    """The namelist's -tol 1e-2 linear solves in FP64: a warm-started solve often stops
    after zero CG iterations, so the velocity follows the thickness in steps whose
    timing could depend on rounding; the bound allows a fraction of a metre of the
    60 m relief (measured: the GPU follows the oracle's steps, 4e-7)."""
    g = np.load(FIXTURE)
    r = prognostic.run(case(exp, "nml"), DT, T_END)
    assert _zs_err(r["z_srf"], g[f"f{exp}_nml_zs"]) < 0.02
    assert _us_err(r["us_aa"], g[f"f{exp}_nml_us"]) < 0.01


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("exp", [1, 2])
def test_device_resident_loop_matches_oracle(exp, precision):
    """The same 2000 years with every field on the GPU (run_device: the device entry
    points on one stream) against the oracle's run."""
    g = np.load(FIXTURE)
    inst = case(exp, "tight")
    inst.par = inst.par.with_(precision=precision)
    r = prognostic.run_device(inst, DT, T_END)
    assert r["steps"] == int(T_END / DT)
    assert _zs_err(r["z_srf"], g[f"f{exp}_tight_zs"]) < 1e-6
    assert _us_err(r["us_aa"], g[f"f{exp}_tight_us"]) < 1e-6
    assert r["history"]["dhdt_max"][-1] < 1e-4
