"""Implicit upwind advection, calc_advec2D(solver = "impl-lis")
(solver_advection.f90:20-145).

CPU: the oracle against an independent restatement built here with scipy: the
same system (linear_solver_matrix_advection_csr_2D, :171-487; border kinds of
define_advection_bcs, :548-622; limit_border_inflow, :646-668;
calc_upwind_faces, :670-755) solved directly, then calc_fixed_cell_transport
(:489-546), every boundary kind. GPU: the device assembly and BiCGSTAB against
the oracle on a marine geometry with prescribed and ice-free cells."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle
from yelmo_gb300 import configs, gpu

BCS = ["zeros", "infinite", "mask", "periodic", "periodic-x", "periodic-y", "MISMIP3D", "TROUGH"]
KINDS = {  # right, upper, left, lower
    "MISMIP3D": ("zero", "periodic", "infinite", "periodic"), "TROUGH": ("zero", "periodic", "infinite", "periodic"),
    "infinite": ("outflow",) * 4, "mask": ("infinite",) * 4, "zeros": ("zero",) * 4, "periodic": ("periodic",) * 4,
    "periodic-x": ("periodic", "outflow", "periodic", "outflow"),
    "periodic-y": ("outflow", "periodic", "outflow", "periodic"),
}


def _nbr(i, j, nx, ny, bc):
    wx = bc in ("periodic", "periodic-x")
    wy = bc in ("periodic", "periodic-y", "MISMIP3D", "TROUGH")
    im1 = (i - 1) % nx if wx else max(i - 1, 0)
    ip1 = (i + 1) % nx if wx else min(i + 1, nx - 1)
    jm1 = (j - 1) % ny if wy else max(j - 1, 0)
    jp1 = (j + 1) % ny if wy else min(j + 1, ny - 1)
    return im1, ip1, jm1, jp1


def _faces(H, ux, uy, bc):
    k = KINDS[bc]
    nx, ny = H.shape
    ux, uy = ux.copy(), uy.copy()
    if k[2] == "outflow":
        ux[0, :] = np.where(ux[0, :] > 0, 0.0, ux[0, :])
    if k[0] == "outflow":
        ux[nx - 2, :] = np.where(ux[nx - 2, :] < 0, 0.0, ux[nx - 2, :])
    if k[3] == "outflow":
        uy[:, 0] = np.where(uy[:, 0] > 0, 0.0, uy[:, 0])
    if k[1] == "outflow":
        uy[:, ny - 2] = np.where(uy[:, ny - 2] < 0, 0.0, uy[:, ny - 2])
    out = {}
    for j in range(ny):
        for i in range(nx):
            im1, ip1, jm1, jp1 = _nbr(i, j, nx, ny, "infinite" if bc == "mask" else bc)
            u1, u2, v1, v2 = ux[im1, j], ux[i, j], uy[i, jm1], uy[i, j]
            if i == 0 and k[2] != "periodic":
                u1 = 0.0
            if i == nx - 1 and k[0] != "periodic":
                u2 = 0.0
            if j == 0 and k[3] != "periodic":
                v1 = 0.0
            if j == ny - 1 and k[1] != "periodic":
                v2 = 0.0
            hx1 = H[im1, j] if u1 >= 0 else H[i, j]
            hx2 = H[i, j] if u2 >= 0 else H[ip1, j]
            hy1 = H[i, jm1] if v1 >= 0 else H[i, j]
            hy2 = H[i, j] if v2 >= 0 else H[i, jp1]
            out[i, j] = (u1, u2, v1, v2, hx1, hx2, hy1, hy2)
    return out


def _scipy_advec(H, ux, uy, F, mask, Href, dx, dy, dt, bc):
    nx, ny = H.shape
    k = KINDS[bc]
    row_bc = [x in ("zero", "infinite") for x in k]
    f = _faces(H, ux, uy, bc)
    dtda = dt / (dx * dy)
    A = sp.lil_matrix((nx * ny, nx * ny))
    b = np.zeros(nx * ny)
    idx = lambda i, j: (i % nx) + nx * (j % ny)
    for j in range(ny):
        for i in range(nx):
            r = idx(i, j)
            border = mask[i, j] != 0
            if mask[i, j] == 1:
                A[r, r] = 1.0
                b[r] = Href[i, j]
            elif border and row_bc[0] and i == nx - 1:
                A[r, r] = 1.0
                if k[0] == "infinite":
                    A[r, idx(i - 1, j)] = -1.0
            elif border and row_bc[1] and j == ny - 1:
                A[r, r] = 1.0
                if k[1] == "infinite":
                    A[r, idx(i, j - 1)] = -1.0
            elif border and row_bc[2] and i == 0:
                A[r, r] = 1.0
                if k[2] == "infinite":
                    A[r, idx(i + 1, j)] = -1.0
            elif border and row_bc[3] and j == 0:
                A[r, r] = 1.0
                if k[3] == "infinite":
                    A[r, idx(i, j + 1)] = -1.0
            else:
                u1, u2, v1, v2 = f[i, j][:4]
                A[r, idx(i, j - 1)] += -dtda * v1 * dx if v1 > 0 else 0.0
                A[r, idx(i - 1, j)] += -dtda * u1 * dy if u1 > 0 else 0.0
                c = 1.0
                c -= dtda * v1 * dx if v1 < 0 else 0.0
                c -= dtda * u1 * dy if u1 < 0 else 0.0
                c += dtda * u2 * dy if u2 > 0 else 0.0
                c += dtda * v2 * dx if v2 > 0 else 0.0
                A[r, r] += c
                A[r, idx(i + 1, j)] += dtda * u2 * dy if u2 < 0 else 0.0
                A[r, idx(i, j + 1)] += dtda * v2 * dx if v2 < 0 else 0.0
                b[r] = H[i, j] + dt * F[i, j]
    x = spla.spsolve(A.tocsc(), b).reshape((nx, ny), order="F")
    if np.any(mask == 1):
        g = _faces(x, ux, uy, bc)
        xn = x.copy()
        for (i, j), (u1, u2, v1, v2, hx1, hx2, hy1, hy2) in g.items():
            if mask[i, j] == 1:
                xn[i, j] = H[i, j] + dt * F[i, j] - dtda * ((u2 * hx2 - u1 * hx1) * dy + (v2 * hy2 - v1 * hy1) * dx)
        x = xn
    return (x - H) / dt


def _fields(nx=14, ny=11, seed=0):
    r = np.random.default_rng(seed)
    Fm = lambda s=1.0: np.asfortranarray(r.normal(size=(nx, ny)) * s)
    H = np.asfortranarray(np.abs(Fm(300.0)))
    mask = np.asfortranarray(np.full((nx, ny), 2, dtype=np.int32))
    mask[4, 5] = 1
    mask[7, 2] = 1
    mask[0, 6] = 0
    mask[nx - 1, 3] = 0
    return H, Fm(100.0), Fm(100.0), Fm(0.5), mask, np.asfortranarray(H * 1.2)


@pytest.mark.parametrize("bc", BCS)
def test_oracle_matches_scipy_restatement(bc):
    H, ux, uy, F, mask, Href = _fields(seed=BCS.index(bc))
    d_o, it, st = oracle.calc_advec2D_impl_lis(H, ux, uy, F, mask, Href, 8e3, 6e3, 5.0, bc)
    assert st == 0 and it > 0
    d_s = _scipy_advec(H, ux, uy, F, mask, Href, 8e3, 6e3, 5.0, bc)
    np.testing.assert_allclose(d_o, d_s, rtol=1e-9, atol=1e-9 * np.abs(d_s).max())


def test_oracle_homogeneous_system():
    """b == 0 (no thickness, no source, ice-free borders): dvdt = 0 without iterating."""
    H, ux, uy, F, mask, Href = _fields()
    z = np.zeros_like(H, order="F")
    d_o, it, st = oracle.calc_advec2D_impl_lis(z, ux, uy, z, np.asfortranarray(np.full_like(mask, 2)), z, 8e3, 8e3,
                                               1.0, "zeros")
    assert it == 0 and st == 0 and np.all(d_o == 0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("bc", ["zeros", "infinite", "mask", "periodic", "MISMIP3D"])
def test_gpu_matches_oracle(bc):
    inst = configs.marine_diva(n=65, nz=4)
    f = oracle.prepare(inst)
    H = np.asfortranarray(inst.H_ice)
    r = np.random.default_rng(3)
    ux = np.asfortranarray(r.normal(size=H.shape) * 200.0)
    uy = np.asfortranarray(r.normal(size=H.shape) * 200.0)
    F = np.asfortranarray(r.normal(size=H.shape) * 0.3)
    mask = np.asfortranarray(np.where(f["f_ice"] > 0, 2, 0).astype(np.int32))
    mask[20:23, 30:33] = 1
    Href = np.asfortranarray(H + 50.0)
    d_o, it_o, st_o = oracle.calc_advec2D_impl_lis(H, ux, uy, F, mask, Href, inst.dx, inst.dx, 2.0, bc)
    d_g, it_g, st_g = gpu.calc_advec2D_impl_lis(H, ux, uy, F, mask, Href, inst.dx, inst.dx, 2.0, bc)
    assert st_o == 0 and st_g == 0, (st_o, st_g)
    err = np.linalg.norm(d_g - d_o) / np.linalg.norm(d_o)
    assert err <= 1e-9, err
    assert abs(it_g - it_o) <= max(2, it_o // 5), (it_g, it_o)


@pytest.mark.gpu
def test_gpu_device_entry_equals_host_entry():
    torch = pytest.importorskip("torch")
    import ctypes as C
    H, ux, uy, F, mask, Href = _fields(nx=40, ny=33, seed=9)
    d_h, it_h, st_h = gpu.calc_advec2D_impl_lis(H, ux, uy, F, mask, Href, 8e3, 8e3, 3.0, "periodic-x")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a.ravel(order="F"))).cuda()
    dH, dux, duy, dF, dm, dR = t(H), t(ux), t(uy), t(F), t(mask), t(Href)
    out = torch.zeros_like(dH)
    solver = gpu.DeviceSolver(0)
    it, st = C.c_int(0), C.c_int(0)
    try:
        torch.cuda.synchronize()
        rc = gpu.lib().ygpu_advec2D_impl_lis_device(solver.ctx, out.data_ptr(), dH.data_ptr(), dux.data_ptr(),
                                                    duy.data_ptr(), dF.data_ptr(), dm.data_ptr(), dR.data_ptr(),
                                                    8e3, 8e3, 3.0, 5, 40, 33, C.byref(it), C.byref(st))
    finally:
        solver.close()
    assert rc == 0 and st.value == st_h == 0 and it.value == it_h
    np.testing.assert_array_equal(out.cpu().numpy().reshape((40, 33), order="F"), d_h)
