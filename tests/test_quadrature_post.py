"""The routines of calc_ydyn that take fields to quadrature nodes: the vertical
velocity by uz_method 2 (calc_uz_3D, velocity_general.f90:346-681) and 3 (the
default, calc_uz_3D_jac, :41-344), and the strain-rate tensor
(calc_strain_rate_tensor_jac_quad3D, deformation.f90:963-1183).

Both rest on fesm-utils' gq2D / gq3D, which the reference does not vendor. The
oracle restates them (corner means, Gauss nodes at +-1/sqrt(3), equal weights):
"restated, unpinned". CPU: the oracle against an independent restatement written
from the corner means directly (the equal-weight mean of the Gauss nodes of a
bilinear or trilinear interpolant is the mean of its corners), on seeded fields
with margins and every boundary code; and known answers: linear velocity fields
give constant strain rates and, when divergence-free, a vertical velocity equal to
its base value; the eigenvalues of known 2D tensors. GPU: the kernels against the
oracle to 1e-12 of each output's largest magnitude, through the host and the
device entries."""
import ctypes as C

import numpy as np
import pytest

import oracle
from yelmo_gb300 import abi, gpu

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


def _active(f_ice, bc):
    nx, ny = f_ice.shape
    ax = np.zeros((nx, ny), bool)
    ay = np.zeros((nx, ny), bool)
    for j in range(ny):
        for i in range(nx):
            im1, ip1, jm1, jp1 = _nbr(i, j, nx, ny, bc)
            ax[i, j] = f_ice[i, j] == 1.0 or f_ice[ip1, j] == 1.0
            ay[i, j] = f_ice[i, j] == 1.0 or f_ice[i, jp1] == 1.0
    return ax, ay


def _amean(vals, acts):
    n = sum(bool(a) for a in acts)
    return sum(v for v, a in zip(vals, acts) if a) / n if n else 0.0


def _acx_corners(v2, ax, i, j, im1, jm1, jp1):
    """Corner values (SW, SE, NE, NW) of an acx field: active mean of the two faces."""
    faces = [((im1, jm1), (im1, j)), ((i, jm1), (i, j)), ((i, j), (i, jp1)), ((im1, j), (im1, jp1))]
    return [_amean([v2[a], v2[b]], [ax[a], ax[b]]) for a, b in faces]


def _acy_corners(v2, ay, i, j, im1, ip1, jm1):
    faces = [((im1, jm1), (i, jm1)), ((i, jm1), (ip1, jm1)), ((i, j), (ip1, j)), ((im1, j), (i, j))]
    return [_amean([v2[a], v2[b]], [ay[a], ay[b]]) for a, b in faces]


def _aa_corners(v2, i, j, im1, ip1, jm1, jp1):
    cells = [((im1, jm1), (i, jm1), (im1, j), (i, j)), ((i, jm1), (ip1, jm1), (i, j), (ip1, j)),
             ((i, j), (ip1, j), (i, jp1), (ip1, jp1)), ((im1, j), (i, j), (im1, jp1), (i, jp1))]
    return [0.25 * sum(v2[c] for c in cc) for cc in cells]


def _q2(v2, act, kind, i, j, nb):
    im1, ip1, jm1, jp1 = nb
    cs = _acx_corners(v2, act, i, j, im1, jm1, jp1) if kind == "x" else _acy_corners(v2, act, i, j, im1, ip1, jm1)
    return float(np.mean(cs))


def _q3(v3, act, kind, i, j, k, nb):
    """3D quadrature value of an acx/acy field on layer k: the mean of the 8 corners,
    each the mean of its 2D corner value on the two layers meeting there."""
    nza = v3.shape[2]
    km1, kp1 = max(k - 1, 0), min(k + 1, nza - 1)
    lo = [0.5 * (a + b) for a, b in zip(_corners(v3[:, :, km1], act, kind, i, j, nb),
                                        _corners(v3[:, :, k], act, kind, i, j, nb))]
    hi = [0.5 * (a + b) for a, b in zip(_corners(v3[:, :, k], act, kind, i, j, nb),
                                        _corners(v3[:, :, kp1], act, kind, i, j, nb))]
    return float(np.mean(lo + hi))


def _corners(v2, act, kind, i, j, nb):
    im1, ip1, jm1, jp1 = nb
    return _acx_corners(v2, act, i, j, im1, jm1, jp1) if kind == "x" else _acy_corners(v2, act, i, j, im1, ip1, jm1)


def _q3z(vac, i, j, klo, khi, nb):
    im1, ip1, jm1, jp1 = nb
    return float(np.mean(_aa_corners(vac[:, :, klo], i, j, im1, ip1, jm1, jp1) +
                         _aa_corners(vac[:, :, khi], i, j, im1, ip1, jm1, jp1)))


def _strain_2d(ux, uy, f_ice, ax, ay, dx, dy, bc):
    """dudx (acx) and dvdy (acy) of calc_strain_rate_horizontal_2D (deformation.f90:1393-1507)."""
    nx, ny = ux.shape
    dudx = np.zeros((nx, ny))
    dvdy = np.zeros((nx, ny))
    for j in range(ny):
        for i in range(nx):
            im1, ip1, jm1, jp1 = _nbr(i, j, nx, ny, bc)
            dudx[i, j] = (ux[ip1, j] - ux[im1, j]) / (2 * dx)
            dvdy[i, j] = (uy[i, jp1] - uy[i, jm1]) / (2 * dy)
            if f_ice[i, j] == 1.0 and f_ice[ip1, j] < 1.0:
                im2 = _nbr(im1, j, nx, ny, bc)[0]
                dudx[i, j] = ((ux[im2, j] - 4 * ux[im1, j] + 3 * ux[i, j]) / (2 * dx)
                              if f_ice[im1, j] == 1.0 and im2 != im1 else (ux[i, j] - ux[im1, j]) / dx)
            elif f_ice[i, j] < 1.0 and f_ice[ip1, j] == 1.0:
                ip2 = _nbr(ip1, j, nx, ny, bc)[1]
                dudx[i, j] = (-(ux[ip2, j] - 4 * ux[ip1, j] + 3 * ux[i, j]) / (2 * dx)
                              if ip2 != ip1 and f_ice[ip2, j] == 1.0 else (ux[ip1, j] - ux[i, j]) / dx)
            if f_ice[i, j] == 1.0 and f_ice[i, jp1] < 1.0:
                jm2 = _nbr(i, jm1, nx, ny, bc)[2]
                dvdy[i, j] = ((uy[i, jm2] - 4 * uy[i, jm1] + 3 * uy[i, j]) / (2 * dy)
                              if f_ice[i, jm1] == 1.0 and jm2 != jm1 else (uy[i, j] - uy[i, jm1]) / dy)
            elif f_ice[i, j] < 1.0 and f_ice[i, jp1] == 1.0:
                jp2 = _nbr(i, jp1, nx, ny, bc)[3]
                dvdy[i, j] = (-(uy[i, jp2] - 4 * uy[i, jp1] + 3 * uy[i, j]) / (2 * dy)
                              if jp2 != jp1 and f_ice[i, jp2] == 1.0 else (uy[i, jp1] - uy[i, j]) / dy)
    return dudx, dvdy


def _uz_restated(a, dx, dy, bc, method, use_bmb):
    nx, ny = a["H_ice"].shape
    za, zc = a["zeta_aa"], a["zeta_ac"]
    nza, nzc = len(za), len(zc)
    fb = 1.0 if use_bmb else 0.0
    ax, ay = _active(a["f_ice"], bc)
    ux, uy = a["ux"], a["uy"]
    if method == abi.UZ_NODES:
        sr = [_strain_2d(ux[:, :, k], uy[:, :, k], a["f_ice"], ax, ay, dx, dy, bc) for k in range(nza)]
    uz = np.zeros((nx, ny, nzc))
    us = np.zeros((nx, ny, nzc))
    for j in range(ny):
        for i in range(nx):
            nb = _nbr(i, j, nx, ny, bc)
            if a["f_ice"][i, j] != 1.0:
                v = _flush(a["dzbdt"][i, j] - max(a["smb"][i, j], 0.0))
                uz[i, j, :] = v
                us[i, j, :] = v
                continue
            H = a["H_ice"][i, j]
            bx, sx = _q2(a["dzbdx"], ax, "x", i, j, nb), _q2(a["dzsdx"], ax, "x", i, j, nb)
            by, sy = _q2(a["dzbdy"], ay, "y", i, j, nb), _q2(a["dzsdy"], ay, "y", i, j, nb)
            uxl = [_q2(ux[:, :, k], ax, "x", i, j, nb) for k in range(nza)]
            uyl = [_q2(uy[:, :, k], ay, "y", i, j, nb) for k in range(nza)]
            col = np.zeros(nzc)
            col[0] = _flush(a["dzbdt"][i, j] + fb * a["bmb"][i, j] + uxl[0] * bx + uyl[0] * by)
            for kc in range(1, nzc):
                if method == abi.UZ_JAC:
                    div = _q3(a["jac_dxx"], ax, "x", i, j, kc - 1, nb) + _q3(a["jac_dyy"], ay, "y", i, j, kc - 1, nb)
                else:
                    z = za[kc - 1]
                    cx = -((1 - z) * bx + z * sx) / H
                    cy = -((1 - z) * by + z * sy) / H
                    kup, kdn = (1, 0) if kc == 1 else (kc - 1, kc - 2) if kc == nzc - 1 else (kc, kc - 2)
                    dudz = (uxl[kup] - uxl[kdn]) / (za[kup] - za[kdn])
                    dvdz = (uyl[kup] - uyl[kdn]) / (za[kup] - za[kdn])
                    div = (_q2(sr[kc - 1][0], ax, "x", i, j, nb) + cx * dudz +
                           _q2(sr[kc - 1][1], ay, "y", i, j, nb) + cy * dvdz)
                col[kc] = _flush(col[kc - 1] - H * (zc[kc] - zc[kc - 1]) * div)
            uz[i, j, :] = col
            for kc in range(nzc):
                kup, kdn = (0, 0) if kc == 0 else (kc - 1, kc - 1) if kc == nzc - 1 else (kc, kc - 1)
                uxa = 0.5 * (uxl[kup] + uxl[kdn])
                uya = 0.5 * (uyl[kup] + uyl[kdn])
                z = zc[kc]
                us[i, j, kc] = _flush(col[kc] - uxa * ((1 - z) * bx + z * sx) - uya * ((1 - z) * by + z * sy)
                                      - ((1 - z) * a["dzbdt"][i, j] + z * a["dzsdt"][i, j]))
    err = np.where(a["f_ice"] == 1.0, us[:, :, -1] + a["smb"], 0.0)
    return {"uz": uz, "uz_star": us, "uz_srf_err": err}


def _random_fields(nx=9, ny=8, nz=5, seed=0):
    r = np.random.default_rng(seed)
    F = lambda *s: np.asfortranarray(r.normal(size=s))
    a = {"ux": F(nx, ny, nz) * 100.0, "uy": F(nx, ny, nz) * 100.0}
    f = r.choice([0.0, 0.4, 1.0, 1.0, 1.0, 1.0], size=(nx, ny))
    a["f_ice"] = np.asfortranarray(f)
    a["f_grnd"] = np.asfortranarray(r.choice([0.0, 0.5, 1.0, 1.0], size=(nx, ny)))
    a["H_ice"] = np.asfortranarray(np.where(f > 0, 500.0 + np.abs(F(nx, ny)) * 1000.0, 0.0))
    for n in ("smb", "bmb", "dzbdt", "dzsdt", "dHidt_dyn"):
        a[n] = F(nx, ny) * 0.5
    for n in ("dzsdx", "dzsdy", "dzbdx", "dzbdy"):
        a[n] = F(nx, ny) * 1e-2
    a["ux_bar"], a["uy_bar"] = F(nx, ny) * 50.0, F(nx, ny) * 50.0
    a["mask_kin"] = np.asfortranarray(r.integers(0, 2, size=(nx, ny)).astype(np.int32))
    a["zeta_aa"] = np.linspace(0.0, 1.0, nz) ** 1.6
    a["zeta_ac"] = np.concatenate([[0.0], 0.5 * (a["zeta_aa"][1:] + a["zeta_aa"][:-1]), [1.0]])
    for n in ("dxx", "dxy", "dxz", "dyx", "dyy", "dyz"):
        a[n] = F(nx, ny, nz) * 1e-3
    for n in ("dzx", "dzy"):
        a[n] = F(nx, ny, nz + 1) * 1e-3
    a["jac_dxx"], a["jac_dyy"] = a["dxx"], a["dyy"]
    return a


@pytest.mark.parametrize("method", [abi.UZ_NODES, abi.UZ_JAC])
@pytest.mark.parametrize("bc", BCS)
def test_oracle_uz_quadrature_matches_restatement(bc, method):
    for use_bmb in (True, False):
        a = _random_fields(seed=5 * BCS.index(bc) + method)
        arr = oracle.calc_uz_3D(gpu.uz_arrays(a), 8e3, 6e3, bc, method, use_bmb)
        ref = _uz_restated(a, 8e3, 6e3, bc, method, use_bmb)
        for n in abi.UZ_OUTPUTS:
            scale = float(np.max(np.abs(ref[n])))
            np.testing.assert_allclose(arr[n], ref[n], rtol=0, atol=1e-11 * scale, err_msg=f"{n} {use_bmb}")


def _trapz(v, z):
    return sum(0.5 * (v[k] + v[k - 1]) * (z[k] - z[k - 1]) for k in range(1, len(z)))


def _strain_restated(a, bc, de_max):
    nx, ny = a["H_ice"].shape
    nza = len(a["zeta_aa"])
    ax, ay = _active(a["f_ice"], bc)
    out = {k: np.zeros((nx, ny, nza)) for k in abi.STRAIN_OUTPUTS_3D}
    for j in range(ny):
        for i in range(nx):
            if a["f_ice"][i, j] != 1.0:
                continue
            nb = _nbr(i, j, nx, ny, bc)
            for k in range(nza):
                dxx = _q3(a["dxx"], ax, "x", i, j, k, nb)
                dyy = _q3(a["dyy"], ay, "y", i, j, k, nb)
                dxy = 0.5 * (_q3(a["dxy"], ax, "x", i, j, k, nb) + _q3(a["dyx"], ay, "y", i, j, k, nb))
                dxz = 0.5 * (_q3(a["dxz"], ax, "x", i, j, k, nb) + _q3z(a["dzx"], i, j, k, k + 1, nb))
                dyz = 0.5 * (_q3(a["dyz"], ay, "y", i, j, k, nb) + _q3z(a["dzy"], i, j, k, k + 1, nb))
                de = min(np.sqrt(dxx * dxx + dyy * dyy + dxx * dyy + dxy * dxy + dxz * dxz + dyz * dyz), de_max)
                fs = np.sqrt(dxz * dxz + dyz * dyz) / de if de > 0 else 1.0
                fs = 0.0 if a["f_grnd"][i, j] == 0.0 else min(max(fs, 0.0), 1.0)
                for n, v in (("s_dxx", dxx), ("s_dyy", dyy), ("s_dxy", dxy), ("s_dxz", dxz), ("s_dyz", dyz),
                             ("s_de", de), ("s_div", dxx + dyy), ("s_f_shear", fs)):
                    out[n][i, j, k] = v
    for n3, n2 in zip(abi.STRAIN_OUTPUTS_3D, abi.STRAIN_OUTPUTS_2D):
        out[n2] = np.array([[_trapz(out[n3][i, j, :], a["zeta_aa"]) for j in range(ny)] for i in range(nx)])
    e1, e2 = np.zeros((nx, ny)), np.zeros((nx, ny))
    for j in range(ny):
        for i in range(nx):
            txx, tyy, txy = out["a_dxx"][i, j], out["a_dyy"][i, j], out["a_dxy"][i, j]
            disc = (txx + tyy) ** 2 - 4 * (txx * tyy - txy * txy)
            if disc > 0:
                r = np.sqrt(disc)
                e1[i, j], e2[i, j] = 0.5 * (txx + tyy + r), 0.5 * (txx + tyy - r)
    out["eps_eig_1"], out["eps_eig_2"] = e1, e2
    return out


@pytest.mark.parametrize("bc", BCS)
def test_oracle_strain_tensor_matches_restatement(bc):
    a = _random_fields(seed=40 + BCS.index(bc))
    de_max = 9e-4            # caps some cells of the seeded fields
    arr = oracle.calc_strain_rate_tensor(gpu.strain_arrays(a, a), 8e3, 6e3, bc, de_max)
    ref = _strain_restated(a, bc, de_max)
    assert np.any(arr["s_de"] == de_max) and np.any((arr["s_de"] > 0) & (arr["s_de"] < de_max))
    for n in abi.STRAIN_OUTPUTS_3D + abi.STRAIN_OUTPUTS_2D:
        scale = float(np.max(np.abs(ref[n]))) or 1.0
        np.testing.assert_allclose(arr[n], ref[n], rtol=0, atol=1e-11 * scale, err_msg=n)


def _linear_slab(nx=12, ny=10, nz=6, H=1200.0, dx=5e3, a_=2e-3, b_=3e-4, c_=-4e-4, d_=-2e-3, shear=1e-4):
    """A fully iced flat slab with ux = a x + b y + shear z-profile, uy = c x + d y at
    their faces, and the Jacobian of that field (constant horizontal gradients)."""
    za = np.linspace(0.0, 1.0, nz) ** 2
    zc = np.concatenate([[0.0], 0.5 * (za[1:] + za[:-1]), [1.0]])
    xf, yc = (np.arange(nx) + 0.5) * dx, np.arange(ny) * dx
    xc, yf = np.arange(nx) * dx, (np.arange(ny) + 0.5) * dx
    ux = a_ * xf[:, None, None] + b_ * yc[None, :, None] + shear * H * za[None, None, :]
    uy = c_ * xc[:, None, None] + d_ * yf[None, :, None] + 0.0 * za[None, None, :]
    a = {"H_ice": np.full((nx, ny), H), "f_ice": np.ones((nx, ny)), "f_grnd": np.ones((nx, ny)),
         "zeta_aa": za, "zeta_ac": zc, "ux": np.asfortranarray(ux), "uy": np.asfortranarray(uy)}
    for n in ("smb", "bmb", "dzbdt", "dzsdt", "dzsdx", "dzsdy", "dzbdx", "dzbdy", "dHidt_dyn"):
        a[n] = np.zeros((nx, ny))
    full = lambda v, nzz: np.full((nx, ny, nzz), v)
    a.update(dxx=full(a_, nz), dxy=full(b_, nz), dyx=full(c_, nz), dyy=full(d_, nz), dxz=full(shear, nz),
             dyz=full(0.0, nz), dzx=full(0.0, nz + 1), dzy=full(0.0, nz + 1))
    a["jac_dxx"], a["jac_dyy"] = a["dxx"], a["dyy"]
    return {k: (np.asfortranarray(v) if isinstance(v, np.ndarray) and v.ndim > 1 else v) for k, v in a.items()}


def test_divergence_free_slab_keeps_the_base_velocity():
    """ux = a x + b y, uy = c x - a y: every level of uz equals the base value (0 on
    a flat bed without melt), by both quadrature methods, away from the edges."""
    a = _linear_slab(d_=-2e-3, a_=2e-3, shear=0.0)
    for method in (abi.UZ_NODES, abi.UZ_JAC):
        out = oracle.calc_uz_3D(gpu.uz_arrays(a), 5e3, 5e3, "zeros", method)
        inner = out["uz"][2:-2, 2:-2, :]
        np.testing.assert_allclose(inner, 0.0, atol=1e-12)


def test_compressive_slab_integrates_the_divergence():
    """du/dx + dv/dy = a + d: uz = -H zeta_ac (a + d) on a flat bed (method 3)."""
    a = _linear_slab(a_=2e-3, d_=-5e-4, shear=0.0)
    out = oracle.calc_uz_3D(gpu.uz_arrays(a), 5e3, 5e3, "zeros", abi.UZ_JAC)
    want = -1200.0 * a["zeta_ac"] * (2e-3 - 5e-4)
    inner = out["uz"][2:-2, 2:-2, :]
    np.testing.assert_allclose(inner, np.broadcast_to(want, inner.shape), rtol=1e-12, atol=1e-12)


def test_constant_gradients_give_the_analytic_tensor():
    a = _linear_slab()
    out = oracle.calc_strain_rate_tensor(gpu.strain_arrays(a, a), 5e3, 5e3, "zeros", de_max=1.0)
    dxx, dyy, dxy, dxz = 2e-3, -2e-3, 0.5 * (3e-4 - 4e-4), 0.5 * 1e-4
    de = np.sqrt(dxx ** 2 + dyy ** 2 + dxx * dyy + dxy ** 2 + dxz ** 2)
    want = {"s_dxx": dxx, "s_dyy": dyy, "s_dxy": dxy, "s_dxz": dxz, "s_dyz": 0.0, "s_de": de,
            "s_div": 0.0, "s_f_shear": dxz / de, "a_dxx": dxx, "a_dyy": dyy, "a_dxy": dxy}
    for n, v in want.items():
        got = out[n][2:-2, 2:-2]
        np.testing.assert_allclose(got, v, rtol=1e-12, atol=1e-15, err_msg=n)
    # eigenvalues of [[dxx, dxy], [dxy, dyy]]
    lam = np.linalg.eigvalsh(np.array([[dxx, dxy], [dxy, dyy]]))
    np.testing.assert_allclose(out["eps_eig_1"][2:-2, 2:-2], lam[1], rtol=1e-12)
    np.testing.assert_allclose(out["eps_eig_2"][2:-2, 2:-2], lam[0], rtol=1e-12)


def test_uz_jac_rejects_missing_jacobian():
    L = gpu.lib()
    a = gpu.uz_arrays(_random_fields())
    U = abi.uz3d(a, 8e3, 8e3)
    U.jac_dxx = None
    assert L.ygpu_calc_uz_3D(C.byref(U), 0, abi.UZ_JAC) == abi.ERR_BAD_ARG


# ---------------------------------------------------------------------------- GPU

def _solved_fields(bc):
    """A converged marine DIVA solve with its Jacobian: the inputs calc_ydyn hands
    to the vertical velocity and the strain-rate tensor."""
    from tests.test_vertical_velocity import _solved_inputs
    inst, a = _solved_inputs(bc)
    nx, ny = a["H_ice"].shape
    # the Jacobian of the solved velocity, with the vertical velocity of uz_method 1
    a["uz"] = oracle.calc_uz_3D(gpu.uz_arrays(a), inst.dx, inst.dx, bc, abi.UZ_AA)["uz"]
    j = oracle.calc_jacobian_vel_3D(gpu.jacobian_arrays({k: a[k] for k in abi.JAC_INPUTS}), inst.dx, inst.dx, bc,
                                    abi.JAC_UXY | abi.JAC_UZ)
    a.update({k: j[k] for k in abi.JAC_OUTPUTS})
    a["jac_dxx"], a["jac_dyy"] = j["dxx"], j["dyy"]
    a["f_grnd"] = np.asfortranarray(np.where(a["H_ice"] > 0, 1.0, 0.0))
    return inst, a


QUAD_TOL = 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("bc", BCS)
def test_gpu_uz_quadrature_matches_oracle(bc):
    inst, a = _solved_fields(bc)
    for method in (abi.UZ_NODES, abi.UZ_JAC):
        for use_bmb in (True, False):
            g = gpu.calc_uz_3D(gpu.uz_arrays(a), inst.dx, inst.dx, bc, method, use_bmb)
            o = oracle.calc_uz_3D(gpu.uz_arrays(a), inst.dx, inst.dx, bc, method, use_bmb)
            for n in abi.UZ_OUTPUTS:
                scale = float(np.max(np.abs(o[n])))
                np.testing.assert_allclose(g[n], o[n], rtol=0, atol=QUAD_TOL * scale,
                                           err_msg=f"{n} method={method} bmb={use_bmb}")


@pytest.mark.gpu
@pytest.mark.parametrize("bc", BCS)
def test_gpu_strain_tensor_matches_oracle(bc):
    inst, a = _solved_fields(bc)
    for de_max in (0.5, 2e-3):
        g = gpu.calc_strain_rate_tensor(gpu.strain_arrays(a, a), inst.dx, inst.dx, bc, de_max)
        o = oracle.calc_strain_rate_tensor(gpu.strain_arrays(a, a), inst.dx, inst.dx, bc, de_max)
        for n in abi.STRAIN_OUTPUTS_3D + abi.STRAIN_OUTPUTS_2D:
            scale = float(np.max(np.abs(o[n]))) or 1.0
            np.testing.assert_allclose(g[n], o[n], rtol=0, atol=QUAD_TOL * scale, err_msg=f"{n} {de_max}")
        assert np.count_nonzero(o["s_de"])


@pytest.mark.gpu
def test_gpu_strain_tensor_device_entry_on_a_stream():
    import torch
    inst, a = _solved_fields("zeros")
    arr = gpu.strain_arrays(a, a)
    ref = gpu.calc_strain_rate_tensor({k: (v.copy(order="F") if isinstance(v, np.ndarray) else v)
                                       for k, v in arr.items()}, inst.dx, inst.dx, "zeros", 0.5)
    dev = {n: torch.from_numpy(np.asarray(v).ravel(order="F").copy()).cuda() for n, v in arr.items()}
    S = abi.Strain3D()
    nx, ny = a["H_ice"].shape
    S.nx, S.ny, S.nz_aa, S.nz_ac = nx, ny, len(a["zeta_aa"]), len(a["zeta_ac"])
    S.dx, S.dy, S.de_max = inst.dx, inst.dx, 0.5
    for n, t in dev.items():
        setattr(S, n, t.data_ptr())
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    assert gpu.lib().ygpu_calc_strain_rate_tensor_device(C.c_void_p(s.cuda_stream), C.byref(S), 0) == 0, \
        gpu.last_error()
    s.synchronize()
    for n in abi.STRAIN_OUTPUTS_3D + abi.STRAIN_OUTPUTS_2D:
        np.testing.assert_array_equal(dev[n].cpu().numpy(), ref[n].ravel(order="F"), err_msg=n)
