"""Vertical velocity of calc_ydyn by uz_method (yelmo_dynamics.f90:259-290).

CPU: the oracle's restatements of calc_uz_3D_aa (uz_method 1,
velocity_general.f90:683-945) and calc_uz_3D_flux (uz_method 4, :947-1116)
against an independent restatement on seeded fields with margins, every boundary
code, with and without basal melt; and known answers: incompressible flow over a
flat bed (uz = -H zeta (du/dx + dv/dy)), the flux form's column mass balance
(uz_star at the surface = bmb - dH/dt + dHidt_dyn where the thickness step gives
the rate), the ice-free value and uz_srf_err. GPU: the kernel against the oracle
on a converged marine DIVA solve, through the host and the device entries."""
import ctypes as C

import numpy as np
import pytest

import oracle
from yelmo_gb300 import abi, configs, gpu

BCS = ["zeros", "infinite", "periodic", "periodic-x", "periodic-y", "MISMIP3D", "TROUGH"]
TOL_UNDERFLOW = 1e-15


def _nbr(i, j, nx, ny, bc):
    wx = bc in ("periodic", "periodic-x")
    wy = bc in ("periodic", "periodic-y", "MISMIP3D", "TROUGH")
    im1 = (i - 1) % nx if wx else max(i - 1, 0)
    ip1 = (i + 1) % nx if wx else min(i + 1, nx - 1)
    jm1 = (j - 1) % ny if wy else max(j - 1, 0)
    jp1 = (j + 1) % ny if wy else min(j + 1, ny - 1)
    return im1, ip1, jm1, jp1


def _flush(v):
    return 0.0 if abs(v) < TOL_UNDERFLOW else v


def _restated(a, dx, dy, bc, method, use_bmb):
    """Both routines per column, written from the equations: base value, layer
    divergence with the sigma correction (aa) or layer mass budget (flux), and the
    coordinate terms between uz and uz_star."""
    nx, ny = a["H_ice"].shape
    za, zc = a["zeta_aa"], a["zeta_ac"]
    nza, nzc = len(za), len(zc)
    fb = 1.0 if use_bmb else 0.0
    uz = np.zeros((nx, ny, nzc))
    us = np.zeros((nx, ny, nzc))
    ux, uy = a["ux"], a["uy"]
    for j in range(ny):
        for i in range(nx):
            im1, ip1, jm1, jp1 = _nbr(i, j, nx, ny, bc)
            if a["f_ice"][i, j] != 1.0:
                v = _flush(a["dzbdt"][i, j] - max(a["smb"][i, j], 0.0))
                uz[i, j, :] = v
                us[i, j, :] = v
                continue
            H = a["H_ice"][i, j]
            g = {n: 0.5 * (a[n][i, j] + a[n][im1, j]) for n in ("dzbdx", "dzsdx")}
            g.update({n: 0.5 * (a[n][i, j] + a[n][i, jm1]) for n in ("dzbdy", "dzsdy")})
            ua = 0.5 * (ux[i, j, :] + ux[im1, j, :])          # face means per layer
            va = 0.5 * (uy[i, j, :] + uy[i, jm1, :])
            lev_u = np.array([ua[0]] + [0.5 * (ua[k] + ua[k - 1]) for k in range(1, nza)] + [ua[-1]])
            lev_v = np.array([va[0]] + [0.5 * (va[k] + va[k - 1]) for k in range(1, nza)] + [va[-1]])
            slope_b = lambda z: (1 - z) * g["dzbdx"] + z * g["dzsdx"]
            slope_c = lambda z: (1 - z) * g["dzbdy"] + z * g["dzsdy"]
            rate = lambda z: (1 - z) * a["dzbdt"][i, j] + z * a["dzsdt"][i, j]
            coord = np.array([-lev_u[k] * slope_b(zc[k]) - lev_v[k] * slope_c(zc[k]) - rate(zc[k])
                              for k in range(nzc)])
            if method == abi.UZ_AA:
                col = np.zeros(nzc)
                col[0] = _flush(a["dzbdt"][i, j] + fb * a["bmb"][i, j] + ua[0] * g["dzbdx"] + va[0] * g["dzbdy"])
                for kc in range(1, nzc):
                    ka = kc - 1
                    hi, lo = (1, 0) if kc == 1 else (nza - 1, nza - 2) if kc == nzc - 1 else (kc, kc - 2)
                    cx = -(slope_b(zc[kc])) / H
                    cy = -(slope_c(zc[kc])) / H
                    div = ((ux[i, j, ka] - ux[im1, j, ka]) / dx + cx * (ua[hi] - ua[lo]) / (za[hi] - za[lo])
                           + (uy[i, j, ka] - uy[i, jm1, ka]) / dy + cy * (va[hi] - va[lo]) / (za[hi] - za[lo]))
                    col[kc] = _flush(col[kc - 1] - H * (zc[kc] - zc[kc - 1]) * div)
                uz[i, j, :] = col
                us[i, j, :] = [_flush(col[k] + coord[k]) for k in range(nzc)]
            else:
                H_ = a["H_ice"]
                Hw = H_[im1, j] if a["ux_bar"][im1, j] >= 0 else H_[i, j]
                He = H_[i, j] if a["ux_bar"][i, j] >= 0 else H_[ip1, j]
                Hs = H_[i, jm1] if a["uy_bar"][i, jm1] >= 0 else H_[i, j]
                Hn = H_[i, j] if a["uy_bar"][i, j] >= 0 else H_[i, jp1]
                dz = np.diff(zc)
                D = dz * ((He * ux[i, j, :] - Hw * ux[im1, j, :]) / dx + (Hn * uy[i, j, :] - Hs * uy[i, jm1, :]) / dy)
                if a["mask_kin"][i, j] == 1:
                    D = D + dz * (-a["dHidt_dyn"][i, j] - D.sum())
                col = np.zeros(nzc)
                col[0] = fb * a["bmb"][i, j]
                for k in range(nza):
                    col[k + 1] = col[k] - dz[k] * (a["dzsdt"][i, j] - a["dzbdt"][i, j]) - D[k]
                uz[i, j, :] = [_flush(col[k] - coord[k]) for k in range(nzc)]
                us[i, j, :] = [_flush(v) for v in col]
    err = np.where(a["f_ice"] == 1.0, us[:, :, -1] + a["smb"], 0.0)
    return {"uz": uz, "uz_star": us, "uz_srf_err": err}


def _random_fields(nx=9, ny=8, nz=5, seed=0):
    r = np.random.default_rng(seed)
    F = lambda *s: np.asfortranarray(r.normal(size=s))
    a = {"ux": F(nx, ny, nz) * 100.0, "uy": F(nx, ny, nz) * 100.0}
    f = r.choice([0.0, 0.4, 1.0, 1.0, 1.0, 1.0], size=(nx, ny))
    a["f_ice"] = np.asfortranarray(f)
    a["H_ice"] = np.asfortranarray(np.where(f > 0, 500.0 + np.abs(F(nx, ny)) * 1000.0, 0.0))
    for n in ("smb", "bmb", "dzbdt", "dzsdt", "dHidt_dyn"):
        a[n] = F(nx, ny) * 0.5
    for n in ("dzsdx", "dzsdy", "dzbdx", "dzbdy"):
        a[n] = F(nx, ny) * 1e-2
    a["ux_bar"], a["uy_bar"] = F(nx, ny) * 50.0, F(nx, ny) * 50.0
    a["mask_kin"] = np.asfortranarray(r.integers(0, 2, size=(nx, ny)).astype(np.int32))
    a["zeta_aa"] = np.linspace(0.0, 1.0, nz) ** 1.6
    a["zeta_ac"] = np.concatenate([[0.0], 0.5 * (a["zeta_aa"][1:] + a["zeta_aa"][:-1]), [1.0]])
    return a


@pytest.mark.parametrize("method", [abi.UZ_AA, abi.UZ_FLUX])
@pytest.mark.parametrize("bc", BCS)
def test_oracle_matches_restatement(bc, method):
    for use_bmb in (True, False):
        a = _random_fields(seed=3 * BCS.index(bc) + method)
        arr = oracle.calc_uz_3D(gpu.uz_arrays(a), 8e3, 6e3, bc, method, use_bmb)
        ref = _restated(a, 8e3, 6e3, bc, method, use_bmb)
        for n in abi.UZ_OUTPUTS:
            scale = float(np.max(np.abs(ref[n])))
            np.testing.assert_allclose(arr[n], ref[n], rtol=0, atol=1e-11 * scale, err_msg=f"{n} {use_bmb}")


def _flat_slab(nx=12, ny=10, nz=6, H=1500.0):
    a = {"H_ice": np.full((nx, ny), H, order="F"), "f_ice": np.ones((nx, ny), order="F")}
    for n in ("smb", "bmb", "dzbdt", "dzsdt", "dzsdx", "dzsdy", "dzbdx", "dzbdy", "dHidt_dyn"):
        a[n] = np.zeros((nx, ny), order="F")
    a["zeta_aa"] = np.linspace(0.0, 1.0, nz) ** 2
    a["zeta_ac"] = np.concatenate([[0.0], 0.5 * (a["zeta_aa"][1:] + a["zeta_aa"][:-1]), [1.0]])
    a["mask_kin"] = np.zeros((nx, ny), dtype=np.int32, order="F")
    return a


def test_uz_aa_incompressible_flat_slab():
    a = _flat_slab()
    nx, ny, nz, H = 12, 10, 6, 1500.0
    dx = 5e3
    xf = (np.arange(nx) + 0.5) * dx
    yf = (np.arange(ny) + 0.5) * dx
    a["ux"] = np.asfortranarray(np.repeat((0.002 * xf)[:, None, None], ny, 1).repeat(nz, 2))
    a["uy"] = np.asfortranarray(np.repeat((-0.0005 * yf)[None, :, None], nx, 0).repeat(nz, 2))
    out = oracle.calc_uz_3D(gpu.uz_arrays(a), dx, dx, "zeros", abi.UZ_AA)
    want = -H * a["zeta_ac"] * (0.002 - 0.0005)
    inner = out["uz"][1:-1, 1:-1, :]
    np.testing.assert_allclose(inner, np.broadcast_to(want, inner.shape), rtol=1e-12, atol=1e-12)
    np.testing.assert_array_equal(out["uz_star"], out["uz"])      # no coordinate terms on a flat slab


def test_uz_flux_column_mass_balance():
    """Where the thickness step gives the column rate, the surface uz_star closes the
    column budget whatever the velocities: bmb - (dzsdt - dzbdt) + dHidt_dyn."""
    a = _random_fields(nx=10, ny=9, nz=7, seed=21)
    a["mask_kin"][:] = 1
    for use_bmb in (True, False):
        out = oracle.calc_uz_3D(gpu.uz_arrays(a), 8e3, 8e3, "periodic", abi.UZ_FLUX, use_bmb)
        ice = a["f_ice"] == 1.0
        want = (1.0 if use_bmb else 0.0) * a["bmb"] - (a["dzsdt"] - a["dzbdt"]) + a["dHidt_dyn"]
        np.testing.assert_allclose(out["uz_star"][:, :, -1][ice], want[ice], rtol=0, atol=1e-9)
        np.testing.assert_allclose(out["uz_srf_err"][ice], (want + a["smb"])[ice], rtol=0, atol=1e-9)
        assert not np.any(out["uz_srf_err"][~ice])


def test_ice_free_cells_take_bed_rate_minus_accumulation():
    a = _random_fields(seed=4)
    for method in (abi.UZ_AA, abi.UZ_FLUX):
        out = oracle.calc_uz_3D(gpu.uz_arrays(a), 8e3, 8e3, "zeros", method)
        free = a["f_ice"] != 1.0
        want = a["dzbdt"] - np.maximum(a["smb"], 0.0)
        for k in range(out["uz"].shape[2]):
            np.testing.assert_array_equal(out["uz"][:, :, k][free], want[free])
            np.testing.assert_array_equal(out["uz_star"][:, :, k][free], want[free])


def test_uz_rejects_bad_arguments():
    """Argument checks of the C ABI (they return before any device work)."""
    L = gpu.lib()
    a = gpu.uz_arrays(_random_fields())
    U = abi.uz3d(a, 8e3, 8e3)
    for method in (0, 5):
        assert L.ygpu_calc_uz_3D(C.byref(U), 0, method) == abi.ERR_BAD_ARG
    assert L.ygpu_calc_uz_3D(C.byref(U), 0, abi.UZ_JAC) == abi.ERR_BAD_ARG    # no Jacobian given
    U.nz_ac = U.nz_aa
    assert L.ygpu_calc_uz_3D(C.byref(U), 0, abi.UZ_AA) == abi.ERR_BAD_ARG
    U = abi.uz3d(a, 8e3, 8e3)
    U.mask_kin = None
    assert L.ygpu_calc_uz_3D(C.byref(U), 0, abi.UZ_FLUX) == abi.ERR_BAD_ARG


def _solved_inputs(bc):
    inst = configs.marine_diva(n=33, nz=6)
    inst.par = inst.par.with_(boundaries=bc, ssa_iter_max=30)
    inputs = oracle.calc_dyn_inputs(inst)
    f = oracle.prepare(inst)
    oracle.calc_velocity(f, inst)
    nx, ny = f["H_ice"].shape
    r = np.random.default_rng(9)
    ocn = (f["z_bed"] < f["z_sl"]).astype(np.int32)
    zb = f["z_bed"]
    bx = np.asfortranarray((np.roll(zb, -1, 0) - zb) / inst.dx)
    by = np.asfortranarray((np.roll(zb, -1, 1) - zb) / inst.dx)
    a = {"ux": f["ux"], "uy": f["uy"], "H_ice": f["H_ice"], "f_ice": f["f_ice"], "zeta_aa": f["zeta_aa"],
         "ux_bar": f["ux_bar"], "uy_bar": f["uy_bar"]}
    a["dzsdx"], a["dzsdy"] = oracle.calc_gradient_column_ac(inputs["dzsdx"], inputs["dzsdy"], f["f_ice"], ocn, bc)
    a["dzbdx"], a["dzbdy"] = oracle.calc_gradient_column_ac(bx, by, f["f_ice"], ocn, bc)
    za = f["zeta_aa"]
    a["zeta_ac"] = np.concatenate([[0.0], 0.5 * (za[1:] + za[:-1]), [1.0]])
    for n, s in (("smb", 0.3), ("bmb", 0.2), ("dzbdt", 0.01), ("dzsdt", 0.1), ("dHidt_dyn", 0.1)):
        a[n] = np.asfortranarray(r.normal(size=(nx, ny)) * s)
    a["mask_kin"] = np.asfortranarray(r.integers(0, 2, size=(nx, ny)).astype(np.int32))
    return inst, a


# The kernel keeps divisions out of its level loops (reciprocal spacings, 1/H per
# column) and regroups the level means, so it agrees with the oracle to rounding:
# to 1e-12 of each output's largest magnitude.
UZ_TOL = 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("bc", BCS)
def test_gpu_uz_matches_oracle(bc):
    inst, a = _solved_inputs(bc)
    for method in (abi.UZ_AA, abi.UZ_FLUX):
        for use_bmb in (True, False):
            g = gpu.calc_uz_3D(gpu.uz_arrays(a), inst.dx, inst.dx, bc, method, use_bmb)
            o = oracle.calc_uz_3D(gpu.uz_arrays(a), inst.dx, inst.dx, bc, method, use_bmb)
            for n in abi.UZ_OUTPUTS:
                scale = float(np.max(np.abs(o[n])))
                np.testing.assert_allclose(g[n], o[n], rtol=0, atol=UZ_TOL * scale,
                                           err_msg=f"{n} method={method} bmb={use_bmb}")
            assert np.count_nonzero(o["uz"])


@pytest.mark.gpu
def test_gpu_uz_device_entry_on_a_stream():
    import torch
    inst, a = _solved_inputs("zeros")
    ref = gpu.calc_uz_3D(gpu.uz_arrays(a), inst.dx, inst.dx, "zeros", abi.UZ_FLUX)
    dev = {n: torch.from_numpy(np.asarray(v).ravel(order="F")).cuda() for n, v in a.items()}
    outs = {n: torch.zeros(ref[n].size, dtype=torch.float64, device="cuda") for n in abi.UZ_OUTPUTS}
    nx, ny = a["H_ice"].shape
    U = abi.Uz3D()
    U.nx, U.ny, U.nz_aa, U.nz_ac, U.dx, U.dy, U.use_bmb = nx, ny, len(a["zeta_aa"]), len(a["zeta_ac"]), \
        inst.dx, inst.dx, 1
    for n, t in list(dev.items()) + list(outs.items()):
        setattr(U, n, t.data_ptr())
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    st = gpu.lib().ygpu_calc_uz_3D_device(C.c_void_p(s.cuda_stream), C.byref(U), 0, abi.UZ_FLUX)
    assert st == 0, gpu.last_error()
    s.synchronize()
    for n in abi.UZ_OUTPUTS:
        np.testing.assert_array_equal(outs[n].cpu().numpy(), ref[n].ravel(order="F"), err_msg=n)
