"""Post-solve diagnostics (calc_ydyn, yelmo_dynamics.f90:304-336 and :642-644).

CPU: the oracle's restatement against an independent numpy restatement of the
reference routines (calc_ice_flux, calc_grounding_line_flux,
calc_magnitude_from_staggered, calc_vel_ratio, integrate_trapezoid1D_pt) on
seeded fields, every boundary code. GPU: the kernels against the oracle,
bit-exact, on the fields of a converged marine DIVA solve."""
import numpy as np
import pytest

import oracle
from yelmo_gb300 import abi, configs, gpu

BCS = ["zeros", "infinite", "periodic", "periodic-x", "periodic-y", "MISMIP3D", "TROUGH"]
TOL_UNDERFLOW = 1e-15


def _nbr(i, j, nx, ny, bc):
    """get_neighbor_indices_bc_codes (yelmo_tools.f90:118-201), 0-based."""
    wx = bc in ("periodic", "periodic-x")
    wy = bc in ("periodic", "periodic-y", "MISMIP3D", "TROUGH")
    im1 = (i - 1) % nx if wx else max(i - 1, 0)
    ip1 = (i + 1) % nx if wx else min(i + 1, nx - 1)
    jm1 = (j - 1) % ny if wy else max(j - 1, 0)
    jp1 = (j + 1) % ny if wy else min(j + 1, ny - 1)
    return im1, ip1, jm1, jp1


def _mag(u, v, f, bc):
    nx, ny = f.shape
    m = np.zeros((nx, ny))
    for j in range(ny):
        for i in range(nx):
            im1, ip1, jm1, jp1 = _nbr(i, j, nx, ny, bc)
            un = vn = 0.0
            if f[i, j] == 1.0:
                un = 0.5 * (u[im1, j] + u[i, j])
                vn = 0.5 * (v[i, jm1] + v[i, j])
                un = 0.0 if abs(un) < TOL_UNDERFLOW else un
                vn = 0.0 if abs(vn) < TOL_UNDERFLOW else vn
            x = np.sqrt(un * un + vn * vn)
            m[i, j] = 0.0 if abs(x) < TOL_UNDERFLOW else x
    return m


def _numpy_diag(a, dx, dy, bc):
    nx, ny = a["H_ice"].shape
    per_x = bc in ("periodic", "periodic-x")
    per_y = bc in ("periodic", "periodic-y", "MISMIP3D", "TROUGH")
    z = a["zeta_aa"]
    out = {}
    out["ux_i_bar"] = sum(0.5 * (a["ux_i"][:, :, k] + a["ux_i"][:, :, k - 1]) * (z[k] - z[k - 1]) for k in range(1, len(z)))
    out["uy_i_bar"] = sum(0.5 * (a["uy_i"][:, :, k] + a["uy_i"][:, :, k - 1]) * (z[k] - z[k - 1]) for k in range(1, len(z)))
    qx, qy = np.zeros((nx, ny)), np.zeros((nx, ny))
    H = a["H_ice"]
    for j in range(ny):
        for i in range(nx):
            im1, ip1, jm1, jp1 = _nbr(i, j, nx, ny, bc)
            if i < nx - 1 or per_x:
                area = H[i, j] * dy if a["ux_bar"][i, j] >= 0.0 else H[ip1, j] * dy
                qx[i, j] = area * a["ux_bar"][i, j]
            if j < ny - 1 or per_y:
                area = H[i, j] * dx if a["uy_bar"][i, j] >= 0.0 else H[i, jp1] * dx
                qy[i, j] = area * a["uy_bar"][i, j]
    out["qq_acx"], out["qq_acy"] = qx, qy
    fg, fi = a["f_grnd"], a["f_ice"]
    gl = lambda g0, g1, f0, f1: (g0 > 0 and g1 == 0 and f1 > 0) or (g1 > 0 and g0 == 0 and f0 > 0)
    glx, gly = np.zeros((nx, ny)), np.zeros((nx, ny))
    for j in range(ny):
        for i in range(nx):
            im1, ip1, jm1, jp1 = _nbr(i, j, nx, ny, bc)
            if gl(fg[i, j], fg[ip1, j], fi[i, j], fi[ip1, j]):
                glx[i, j] = qx[i, j]
            if gl(fg[i, j], fg[i, jp1], fi[i, j], fi[i, jp1]):
                gly[i, j] = qy[i, j]
    out["qq_gl_acx"], out["qq_gl_acy"] = glx, gly
    out["qq"] = _mag(qx, qy, fi, bc)
    out["taub"] = _mag(a["taub_acx"], a["taub_acy"], fi, bc)
    out["taud"] = _mag(a["taud_acx"], a["taud_acy"], fi, bc)
    out["uxy_b"] = _mag(a["ux_b"], a["uy_b"], fi, bc)
    out["uxy_i_bar"] = _mag(out["ux_i_bar"], out["uy_i_bar"], fi, bc)
    out["uxy_bar"] = _mag(a["ux_bar"], a["uy_bar"], fi, bc)
    nz = a["ux"].shape[2]
    out["uxy"] = np.stack([_mag(a["ux"][:, :, k], a["uy"][:, :, k], fi, bc) for k in range(nz)], axis=2)
    out["ux_s"], out["uy_s"], out["uxy_s"] = a["ux"][:, :, -1], a["uy"][:, :, -1], out["uxy"][:, :, -1]
    us = out["uxy_s"]
    out["f_vbvs"] = np.where(us > 0.0, np.minimum(1.0, out["uxy_b"] / np.where(us > 0.0, us, 1.0)), 1.0)
    return out


def _random_fields(nx=9, ny=7, nz=4, seed=0):
    r = np.random.default_rng(seed)
    F = lambda *s: np.asfortranarray(r.normal(size=s) * 100.0)
    f = {k: F(nx, ny) for k in ("ux_bar", "uy_bar", "ux_b", "uy_b", "taub_acx", "taub_acy", "taud_acx", "taud_acy")}
    f["H_ice"] = np.asfortranarray(np.abs(F(nx, ny)) * 10.0)
    f["f_ice"] = np.asfortranarray(r.choice([0.0, 0.5, 1.0, 1.0, 1.0], size=(nx, ny)))
    f["f_grnd"] = np.asfortranarray(r.choice([0.0, 0.0, 0.3, 1.0], size=(nx, ny)))
    f["ux_i"], f["uy_i"], f["ux"], f["uy"] = F(nx, ny, nz), F(nx, ny, nz), F(nx, ny, nz), F(nx, ny, nz)
    f["ux_b"][0, 0] = 1e-17          # underflow flush
    f["zeta_aa"] = np.linspace(0.0, 1.0, nz) ** 1.5
    return f


@pytest.mark.parametrize("bc", BCS)
def test_oracle_matches_numpy_restatement(bc):
    f = _random_fields(seed=BCS.index(bc))
    arr = gpu.diagnostics_arrays(f, f["ux"].shape[2])
    oracle.calc_dyn_diagnostics(arr, 8e3, 6e3, bc)
    ref = _numpy_diag(f, 8e3, 6e3, bc)
    for k, v in ref.items():
        np.testing.assert_allclose(arr[k], v, rtol=1e-14, atol=1e-300, err_msg=k)


@pytest.mark.gpu
@pytest.mark.parametrize("bc", ["zeros", "periodic", "MISMIP3D", "infinite"])
def test_gpu_diagnostics_bit_exact(bc):
    inst = configs.marine_diva(n=33, nz=6)
    inst.par = inst.par.with_(boundaries=bc, ssa_iter_max=30)
    f = oracle.prepare(inst)
    oracle.calc_velocity(f, inst)
    nz = inst.nz
    for groups in ((True, True), (False, False)):
        ga = gpu.diagnostics_arrays(f, nz, *groups)
        oa = gpu.diagnostics_arrays(f, nz, *groups)
        gpu.calc_dyn_diagnostics(ga, inst.dx, inst.dx, bc)
        oracle.calc_dyn_diagnostics(oa, inst.dx, inst.dx, bc)
        for k in abi.DIAG_OUTPUTS:
            if k in oa:
                np.testing.assert_array_equal(ga[k], oa[k], err_msg=f"{k} {groups}")
    assert np.any(oa["qq"] > 0.0)
