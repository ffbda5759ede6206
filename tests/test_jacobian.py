"""Velocity Jacobian and column gradients of calc_ydyn (yelmo_dynamics.f90:243-296).

CPU: the oracle's restatement of calc_gradient_column_ac (yelmo_tools.f90:479-571)
and of calc_jacobian_vel_3D_uxyterms / _uzterms (deformation.f90:397-961) against
an independent restatement (vertical derivatives from the derivative of the
Lagrange interpolant through three layers instead of the reference's closed
forms), on seeded fields with ice margins, every boundary code; and analytic
known answers: the three-point formulas are exact for a velocity quadratic in z,
centred and one-sided differences exact for one linear in x or y.
GPU: the kernel against the oracle, bit-exact, on a converged marine DIVA solve,
through the host and the device entries."""
import ctypes as C

import numpy as np
import pytest

import oracle
from yelmo_gb300 import abi, configs, gpu

BCS = ["zeros", "infinite", "periodic", "periodic-x", "periodic-y", "MISMIP3D", "TROUGH"]
BOTH = abi.JAC_UXY | abi.JAC_UZ


def _nbr(i, j, nx, ny, bc):
    """get_neighbor_indices_bc_codes (yelmo_tools.f90:118-201), 0-based."""
    wx = bc in ("periodic", "periodic-x")
    wy = bc in ("periodic", "periodic-y", "MISMIP3D", "TROUGH")
    im1 = (i - 1) % nx if wx else max(i - 1, 0)
    ip1 = (i + 1) % nx if wx else min(i + 1, nx - 1)
    jm1 = (j - 1) % ny if wy else max(j - 1, 0)
    jp1 = (j + 1) % ny if wy else min(j + 1, ny - 1)
    return im1, ip1, jm1, jp1


def _column_gradient(g, f, ocn, bc, axis):
    nx, ny = f.shape
    out = np.zeros((nx, ny))
    for j in range(ny):
        for i in range(nx):
            im1, ip1, jm1, jp1 = _nbr(i, j, nx, ny, bc)
            if axis == 0:
                nb, prev, nxt = (ip1, j), (im1, j), None
                _, ip2, _, _ = _nbr(ip1, j, nx, ny, bc)
                nxt = (ip2, j)
                has_prev, has_next = im1 != i, ip2 != ip1
            else:
                nb, prev = (i, jp1), (i, jm1)
                _, _, _, jp2 = _nbr(i, jp1, nx, ny, bc)
                nxt = (i, jp2)
                has_prev, has_next = jm1 != j, jp2 != jp1
            a, b = f[i, j] == 1.0, f[nb] == 1.0
            if a and b:
                out[i, j] = g[i, j]
            elif (a and not ocn[nb]) or (b and not ocn[i, j]):
                out[i, j] = g[i, j]
            elif a:
                out[i, j] = g[prev] if has_prev and f[prev] == 1.0 else 0.0
            elif b:
                out[i, j] = g[nb] if has_next and f[nxt] == 1.0 else 0.0
    return out


def _lagrange_d1(xs, us, xe):
    """Derivative at xe of the quadratic through (xs[m], us[m])."""
    d = 0.0
    for m in range(3):
        o = [q for q in range(3) if q != m]
        num = (xe - xs[o[0]]) + (xe - xs[o[1]])
        den = (xs[m] - xs[o[0]]) * (xs[m] - xs[o[1]])
        d += us[m] * num / den
    return d


def _vderiv(u, z, k, top3=True):
    nz = len(z)
    if k == 0:
        return _lagrange_d1(z[0:3], u[0:3], z[0])
    if k < nz - 1:
        return _lagrange_d1(z[k - 1:k + 2], u[k - 1:k + 2], z[k])
    if not top3:
        return (u[k] - u[k - 1]) / (z[k] - z[k - 1])
    return _lagrange_d1(z[k - 2:k + 1], u[k - 2:k + 1], z[k])


def _one_sided(u, f, i, j, bc, axis, h, check_self):
    """Margin derivative along `axis` at (i, j); None where the centred one stays."""
    nx, ny = f.shape
    im1, ip1, jm1, jp1 = _nbr(i, j, nx, ny, bc)
    if axis == 0:
        p, m, last = (ip1, j), (im1, j), ip1 < nx - 1
        m2, p2 = (im1 - 1, j), (ip1 + 1, j)
        first = im1 > 0
    else:
        p, m = (i, jp1), (i, jm1)
        last, first = jp1 < ny - 1, jm1 > 0
        m2, p2 = (i, jm1 - 1), (i, jp1 + 1)
    c = (i, j)
    if check_self:      # ux/uy terms: the cell and its forward neighbour decide
        back = f[c] == 1.0 and f[p] < 1.0
        fwd = f[c] < 1.0 and f[p] == 1.0
        back3 = first and f[m] == 1.0
    else:               # uz terms: the two neighbours decide
        if f[p] < 1.0 and f[m] < 1.0:
            return 0.0
        back = f[p] < 1.0 and f[m] == 1.0
        fwd = f[p] == 1.0 and f[m] < 1.0
        back3 = first and f[m2] == 1.0 if back else False
    if back:
        if back3:
            return (u[m2] - 4.0 * u[m] + 3.0 * u[c]) / (2.0 * h)
        return (u[c] - u[m]) / h
    if fwd:
        if last and f[p2] == 1.0:
            return -(u[p2] - 4.0 * u[p] + 3.0 * u[c]) / (2.0 * h)
        return (u[p] - u[c]) / h
    return None


def _numpy_jacobian(a, dx, dy, bc):
    f, H = a["f_ice"], a["H_ice"]
    nx, ny = f.shape
    za, zc = a["zeta_aa"], a["zeta_ac"]
    nza, nzc = len(za), len(zc)
    ax = np.zeros((nx, ny), bool)
    ay = np.zeros((nx, ny), bool)
    for j in range(ny):
        for i in range(nx):
            im1, ip1, jm1, jp1 = _nbr(i, j, nx, ny, bc)
            ax[i, j] = f[i, j] == 1.0 or f[ip1, j] == 1.0
            ay[i, j] = f[i, j] == 1.0 or f[i, jp1] == 1.0

    def mean_act(vals, acts):
        n = sum(acts)
        return sum(v for v, t in zip(vals, acts) if t) / n if n else 0.0

    def dact(vm, v0, vp, am, ap, h):
        if am and ap:
            return (vp - vm) / (2.0 * h)
        if ap:
            return (vp - v0) / h
        if am:
            return (v0 - vm) / h
        return 0.0

    out = {n: np.zeros((nx, ny, nza)) for n in abi.JAC_OUTPUTS[:6]}
    out.update({n: np.zeros((nx, ny, nzc)) for n in abi.JAC_OUTPUTS[6:]})
    bx, by, sx, sy = a["dzbdx"], a["dzbdy"], a["dzsdx"], a["dzsdy"]
    for j in range(ny):
        for i in range(nx):
            im1, ip1, jm1, jp1 = _nbr(i, j, nx, ny, bc)
            Hf = []
            for nb in ((ip1, j), (i, jp1)):
                if f[i, j] == 1.0 and f[nb] < 1.0:
                    Hf.append(H[i, j])
                elif f[i, j] < 1.0 and f[nb] == 1.0:
                    Hf.append(H[nb])
                else:
                    Hf.append(0.5 * (H[i, j] + H[nb]))
            bx_acy = mean_act([bx[i, j], bx[i, jp1], bx[im1, j], bx[im1, jp1]],
                              [ax[i, j], ax[i, jp1], ax[im1, j], ax[im1, jp1]])
            sx_acy = mean_act([sx[i, j], sx[i, jp1], sx[im1, j], sx[im1, jp1]],
                              [ax[i, j], ax[i, jp1], ax[im1, j], ax[im1, jp1]])
            by_acx = mean_act([by[i, j], by[ip1, j], by[i, jm1], by[ip1, jm1]],
                              [ay[i, j], ay[ip1, j], ay[i, jm1], ay[ip1, jm1]])
            sy_acx = mean_act([sy[i, j], sy[ip1, j], sy[i, jm1], sy[ip1, jm1]],
                              [ay[i, j], ay[ip1, j], ay[i, jm1], ay[ip1, jm1]])
            for k in range(nza):
                ux, uy = a["ux"][:, :, k], a["uy"][:, :, k]
                dxz = _vderiv(a["ux"][i, j, :], Hf[0] * za, k) if Hf[0] > 0 else 0.0
                dyz = _vderiv(a["uy"][i, j, :], Hf[1] * za, k) if Hf[1] > 0 else 0.0
                dxx = _one_sided(ux, f, i, j, bc, 0, dx, True)
                dxx = (ux[ip1, j] - ux[im1, j]) / (2.0 * dx) if dxx is None else dxx
                dyy = _one_sided(uy, f, i, j, bc, 1, dy, True)
                dyy = (uy[i, jp1] - uy[i, jm1]) / (2.0 * dy) if dyy is None else dyy
                dxy = dact(ux[i, jm1], ux[i, j], ux[i, jp1], ax[i, jm1], ax[i, jp1], dy)
                dyx = dact(uy[im1, j], uy[i, j], uy[ip1, j], ay[im1, j], ay[ip1, j], dx)
                z = za[k]
                out["dxx"][i, j, k] = dxx - ((1 - z) * bx[i, j] + z * sx[i, j]) * dxz
                out["dyy"][i, j, k] = dyy - ((1 - z) * by[i, j] + z * sy[i, j]) * dyz
                out["dxy"][i, j, k] = dxy - ((1 - z) * by_acx + z * sy_acx) * dxz
                out["dyx"][i, j, k] = dyx - ((1 - z) * bx_acy + z * sx_acy) * dyz
                out["dxz"][i, j, k], out["dyz"][i, j, k] = dxz, dyz
            if f[i, j] != 1.0:
                continue
            bxa, bya = 0.5 * (bx[i, j] + bx[im1, j]), 0.5 * (by[i, j] + by[i, jm1])
            sxa, sya = 0.5 * (sx[i, j] + sx[im1, j]), 0.5 * (sy[i, j] + sy[i, jm1])
            for k in range(nzc):
                uz = a["uz"][:, :, k]
                dzz = _vderiv(a["uz"][i, j, :], H[i, j] * zc, k, top3=False)
                dzx = _one_sided(uz, f, i, j, bc, 0, dx, False)
                dzx = (uz[ip1, j] - uz[im1, j]) / (2.0 * dx) if dzx is None else dzx
                dzy = _one_sided(uz, f, i, j, bc, 1, dy, False)
                dzy = (uz[i, jp1] - uz[i, jm1]) / (2.0 * dy) if dzy is None else dzy
                z = zc[k]
                out["dzx"][i, j, k] = dzx - ((1 - z) * bxa + z * sxa) * dzz
                out["dzy"][i, j, k] = dzy - ((1 - z) * bya + z * sya) * dzz
                out["dzz"][i, j, k] = dzz
    return out


def _random_fields(nx=9, ny=8, nz=5, seed=0):
    r = np.random.default_rng(seed)
    F = lambda *s: np.asfortranarray(r.normal(size=s))
    a = {"ux": F(nx, ny, nz) * 100.0, "uy": F(nx, ny, nz) * 100.0, "uz": F(nx, ny, nz + 1)}
    a["H_ice"] = np.asfortranarray(500.0 + np.abs(F(nx, ny)) * 1000.0)
    f = r.choice([0.0, 0.4, 1.0, 1.0, 1.0, 1.0], size=(nx, ny))
    a["H_ice"][f == 0.0] = 0.0
    a["f_ice"] = np.asfortranarray(f)
    for n in ("dzsdx", "dzsdy", "dzbdx", "dzbdy"):
        a[n] = F(nx, ny) * 1e-2
    a["zeta_aa"] = np.linspace(0.0, 1.0, nz) ** 1.7
    a["zeta_ac"] = np.concatenate([[0.0], 0.5 * (a["zeta_aa"][1:] + a["zeta_aa"][:-1]), [1.0]])
    return a


@pytest.mark.parametrize("bc", BCS)
def test_gradient_column_oracle_matches_restatement(bc):
    r = np.random.default_rng(BCS.index(bc))
    nx, ny = 10, 9
    f = np.asfortranarray(r.choice([0.0, 0.5, 1.0, 1.0], size=(nx, ny)))
    ocn = np.asfortranarray(r.integers(0, 2, size=(nx, ny)).astype(np.int32))
    gx, gy = np.asfortranarray(r.normal(size=(nx, ny))), np.asfortranarray(r.normal(size=(nx, ny)))
    cx, cy = oracle.calc_gradient_column_ac(gx, gy, f, ocn, bc)
    np.testing.assert_array_equal(cx, _column_gradient(gx, f, ocn, bc, 0))
    np.testing.assert_array_equal(cy, _column_gradient(gy, f, ocn, bc, 1))
    # every branch was taken: kept, ice-side copy, zero
    assert np.any(cx == gx) and np.any(cx == 0.0) and np.any((cx != gx) & (cx != 0.0))


@pytest.mark.parametrize("bc", BCS)
def test_jacobian_oracle_matches_restatement(bc):
    a = _random_fields(seed=10 + BCS.index(bc))
    arr = gpu.jacobian_arrays(a)
    oracle.calc_jacobian_vel_3D(arr, 8e3, 6e3, bc)
    ref = _numpy_jacobian(a, 8e3, 6e3, bc)
    for n in abi.JAC_OUTPUTS:
        scale = np.max(np.abs(ref[n])) + 1e-300
        np.testing.assert_allclose(arr[n], ref[n], rtol=1e-11, atol=1e-12 * scale, err_msg=n)
    assert np.count_nonzero(arr["dzz"]) and np.count_nonzero(arr["dxz"])


def test_jacobian_uxy_only_zeroes_uz_terms():
    a = _random_fields(seed=3)
    arr = gpu.jacobian_arrays(a)
    for n in abi.JAC_OUTPUTS[6:]:
        arr[n][:] = 7.0
    oracle.calc_jacobian_vel_3D(arr, 8e3, 6e3, "zeros", abi.JAC_UXY)
    for n in abi.JAC_OUTPUTS[6:]:
        assert not np.any(arr[n]), n
    both = gpu.jacobian_arrays(a)
    oracle.calc_jacobian_vel_3D(both, 8e3, 6e3, "zeros", BOTH)
    for n in abi.JAC_OUTPUTS[:6]:
        np.testing.assert_array_equal(arr[n], both[n])


def _flat_slab(nx=12, ny=10, nz=6, H=1500.0):
    a = {"H_ice": np.full((nx, ny), H, order="F"), "f_ice": np.ones((nx, ny), order="F")}
    for n in ("dzsdx", "dzsdy", "dzbdx", "dzbdy"):
        a[n] = np.zeros((nx, ny), order="F")
    a["zeta_aa"] = np.linspace(0.0, 1.0, nz) ** 2
    a["zeta_ac"] = np.linspace(0.0, 1.0, nz + 1) ** 1.5
    return a


def test_jacobian_exact_for_quadratic_in_z():
    a = _flat_slab()
    nx, ny, H = 12, 10, 1500.0
    z = H * a["zeta_aa"]
    zc = H * a["zeta_ac"]
    p = lambda z: 3.0 + 0.02 * z - 1.5e-5 * z ** 2
    dp = lambda z: 0.02 - 3.0e-5 * z
    a["ux"] = np.asfortranarray(np.broadcast_to(p(z), (nx, ny, len(z))))
    a["uy"] = np.asfortranarray(np.broadcast_to(-2.0 * p(z), (nx, ny, len(z))))
    a["uz"] = np.asfortranarray(np.broadcast_to(0.5 * p(zc), (nx, ny, len(zc))))
    arr = oracle.calc_jacobian_vel_3D(gpu.jacobian_arrays(a), 5e3, 5e3, "periodic")
    np.testing.assert_allclose(arr["dxz"], np.broadcast_to(dp(z), arr["dxz"].shape), rtol=1e-10)
    np.testing.assert_allclose(arr["dyz"], np.broadcast_to(-2.0 * dp(z), arr["dyz"].shape), rtol=1e-10)
    # uz: three-point inside and at the base, first order at the top
    want = np.broadcast_to(0.5 * dp(zc), arr["dzz"].shape)
    np.testing.assert_allclose(arr["dzz"][:, :, :-1], want[:, :, :-1], rtol=1e-10)
    top = 0.5 * (p(zc[-1]) - p(zc[-2])) / (zc[-1] - zc[-2])
    np.testing.assert_allclose(arr["dzz"][:, :, -1], top, rtol=1e-12)
    for n in ("dxx", "dxy", "dyx", "dyy", "dzx", "dzy"):
        assert np.max(np.abs(arr[n])) < 1e-15, n


def test_jacobian_exact_for_linear_in_x_and_y_with_a_margin():
    a = _flat_slab()
    nx, ny, nz = 12, 10, 6
    xf = (np.arange(nx) + 0.5) * 5e3          # ux on the right faces
    yc = np.arange(ny) * 5e3
    m = 8                                      # ice up to cell m, then ice free
    a["f_ice"][m + 1:, :] = 0.0
    a["H_ice"][m + 1:, :] = 0.0
    ux = 0.01 * xf[:, None] + 0.003 * yc[None, :]
    a["ux"] = np.asfortranarray(np.repeat(ux[:, :, None], nz, axis=2))
    a["uy"] = np.zeros((nx, ny, nz), order="F")
    a["uz"] = np.asfortranarray(np.repeat((0.02 * np.arange(nx) * 5e3)[:, None, None], ny, 1).repeat(nz + 1, 2))
    arr = oracle.calc_jacobian_vel_3D(gpu.jacobian_arrays(a), 5e3, 5e3, "zeros")
    inner = (slice(1, m + 1), slice(1, ny - 1))
    np.testing.assert_allclose(arr["dxx"][inner], 0.01, rtol=1e-12)       # one-sided 3-point at i = m
    np.testing.assert_allclose(arr["dxy"][inner], 0.003, rtol=1e-10)
    np.testing.assert_allclose(arr["dzx"][2:m - 1, 1:ny - 1], 0.02, rtol=1e-12)
    np.testing.assert_allclose(arr["dzx"][m, 1:ny - 1], 0.02, rtol=1e-12)  # backward 3-point at the margin
    assert not np.any(arr["dzx"][m + 1:])                                  # ice free


def test_jacobian_rejects_bad_arguments():
    """Argument checks of the C ABI (they return before any device work)."""
    L = gpu.lib()
    a = _random_fields(nz=2)
    J = abi.jvel(gpu.jacobian_arrays(a), 8e3, 8e3)
    assert L.ygpu_calc_jacobian_vel_3D(C.byref(J), 0, abi.JAC_UXY) == abi.ERR_BAD_ARG
    a = _random_fields()
    J = abi.jvel(gpu.jacobian_arrays(a), 8e3, 8e3)
    assert L.ygpu_calc_jacobian_vel_3D(C.byref(J), 0, 0) == abi.ERR_BAD_ARG
    assert L.ygpu_calc_jacobian_vel_3D(C.byref(J), 9, BOTH) == abi.ERR_BAD_ARG
    J.uz = None
    assert L.ygpu_calc_jacobian_vel_3D(C.byref(J), 0, abi.JAC_UZ) == abi.ERR_BAD_ARG
    assert L.ygpu_calc_gradient_column_ac(None, None, None, None, None, None, 0, 4, 4) == abi.ERR_BAD_ARG


def _solved_state(bc):
    inst = configs.marine_diva(n=33, nz=6)
    inst.par = inst.par.with_(boundaries=bc, ssa_iter_max=30)
    inputs = oracle.calc_dyn_inputs(inst)
    f = oracle.prepare(inst)
    oracle.calc_velocity(f, inst)
    f["dzsdx"], f["dzsdy"] = inputs["dzsdx"], inputs["dzsdy"]
    nx, ny = f["H_ice"].shape
    r = np.random.default_rng(5)
    zb = f["z_bed"]
    bx = np.asfortranarray((np.roll(zb, -1, 0) - zb) / inst.dx)
    by = np.asfortranarray((np.roll(zb, -1, 1) - zb) / inst.dx)
    ocn = (f["z_bed"] < f["z_sl"]).astype(np.int32)
    a = {"ux": f["ux"], "uy": f["uy"], "H_ice": f["H_ice"], "f_ice": f["f_ice"], "zeta_aa": f["zeta_aa"]}
    a["dzsdx"], a["dzsdy"] = oracle.calc_gradient_column_ac(f["dzsdx"], f["dzsdy"], f["f_ice"], ocn, bc)
    a["dzbdx"], a["dzbdy"] = oracle.calc_gradient_column_ac(bx, by, f["f_ice"], ocn, bc)
    za = f["zeta_aa"]
    a["zeta_ac"] = np.concatenate([[0.0], 0.5 * (za[1:] + za[:-1]), [1.0]])
    a["uz"] = np.asfortranarray(r.normal(size=(nx, ny, len(za) + 1)) * 0.3)
    return inst, a, (f["dzsdx"], f["dzsdy"], bx, by, ocn)


# The kernel evaluates the reference's derivatives without divisions in its layer
# loops (difference form with per-layer weights, reciprocals of dx, dy and H), so
# it agrees with the oracle to rounding: per component, to 1e-12 of its largest
# magnitude. A wrong stencil, weight or branch is an O(1) error.
JAC_TOL = 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("bc", BCS)
def test_gpu_jacobian_matches_oracle(bc):
    inst, a, (sx, sy, bx, by, ocn) = _solved_state(bc)
    for g, h in (((sx, sy), ("dzsdx", "dzsdy")), ((bx, by), ("dzbdx", "dzbdy"))):
        gx, gy = gpu.calc_gradient_column_ac(g[0], g[1], a["f_ice"], ocn, bc)
        np.testing.assert_array_equal(gx, a[h[0]])       # selects only: bit-exact
        np.testing.assert_array_equal(gy, a[h[1]])
    for terms in (abi.JAC_UXY, abi.JAC_UZ, BOTH):
        ga = gpu.calc_jacobian_vel_3D(gpu.jacobian_arrays(a, terms), inst.dx, inst.dx, bc, terms)
        oa = oracle.calc_jacobian_vel_3D(gpu.jacobian_arrays(a, terms), inst.dx, inst.dx, bc, terms)
        for n in abi.JAC_OUTPUTS:
            if n in oa:
                scale = float(np.max(np.abs(oa[n])))
                np.testing.assert_allclose(ga[n], oa[n], rtol=0, atol=JAC_TOL * scale + 1e-300,
                                           err_msg=f"{n} terms={terms}")
    assert np.count_nonzero(oa["dxx"]) and np.count_nonzero(oa["dzz"])


@pytest.mark.gpu
def test_gpu_jacobian_analytic_known_answers():
    """The known answers of the CPU tests, through the GPU kernel."""
    a = _flat_slab()
    nx, ny, H = 12, 10, 1500.0
    z, zc = H * a["zeta_aa"], H * a["zeta_ac"]
    p = lambda z: 3.0 + 0.02 * z - 1.5e-5 * z ** 2
    dp = lambda z: 0.02 - 3.0e-5 * z
    a["ux"] = np.asfortranarray(np.broadcast_to(p(z), (nx, ny, len(z))))
    a["uy"] = np.asfortranarray(np.broadcast_to(-2.0 * p(z), (nx, ny, len(z))))
    a["uz"] = np.asfortranarray(np.broadcast_to(0.5 * p(zc), (nx, ny, len(zc))))
    g = gpu.calc_jacobian_vel_3D(gpu.jacobian_arrays(a), 5e3, 5e3, "periodic")
    np.testing.assert_allclose(g["dxz"], np.broadcast_to(dp(z), g["dxz"].shape), rtol=1e-10)
    np.testing.assert_allclose(g["dyz"], np.broadcast_to(-2.0 * dp(z), g["dyz"].shape), rtol=1e-10)
    np.testing.assert_allclose(g["dzz"][:, :, :-1], np.broadcast_to(0.5 * dp(zc), g["dzz"].shape)[:, :, :-1],
                               rtol=1e-10)


@pytest.mark.gpu
def test_gpu_jacobian_device_entry_on_a_stream():
    import torch
    inst, a, _ = _solved_state("zeros")
    ref = gpu.calc_jacobian_vel_3D(gpu.jacobian_arrays(a), inst.dx, inst.dx, "zeros")
    dev = {n: torch.from_numpy(np.asarray(v).ravel(order="F")).cuda() for n, v in a.items()}
    outs = {n: torch.zeros(ref[n].size, dtype=torch.float64, device="cuda") for n in abi.JAC_OUTPUTS}
    J = abi.JVel()
    nx, ny = a["H_ice"].shape
    J.nx, J.ny, J.nz_aa, J.nz_ac, J.dx, J.dy = nx, ny, len(a["zeta_aa"]), len(a["zeta_ac"]), inst.dx, inst.dx
    for n, t in list(dev.items()) + list(outs.items()):
        setattr(J, n, t.data_ptr())
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    st = gpu.lib().ygpu_calc_jacobian_vel_3D_device(C.c_void_p(s.cuda_stream), C.byref(J), 0, BOTH)
    assert st == 0, gpu.last_error()
    s.synchronize()
    for n in abi.JAC_OUTPUTS:
        np.testing.assert_array_equal(outs[n].cpu().numpy(), ref[n].ravel(order="F"), err_msg=n)
