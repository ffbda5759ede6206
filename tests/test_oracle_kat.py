"""The oracle against the known-answer tests of the reference's own suite.

 - tests/test_ssa_energy.f90: K_inner = -A_residual * dx*dy, b_inner = -taud*dx*dy
   on an 8x8 periodic grid; front rows carry +-taul_int*dy.
 - tests/test_ssa_energy_sym.f90: K = K^T (periodic, zeros, front strip,
   free-slip edges).
 - tests/test_ssa_energy_lr_sym.f90: reflection equivariance of K and b.
The reference runs these in single precision with rtol 1e-5; the oracle is
FP64, so the same identities must hold to ~1e-12.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from tests.kat_fields import energy_identity_fields, uniform_fields

DX = DY = 5000.0


def _mat(energy, f, bc):
    ptr, idx, val, b, x, cf = oracle.assemble_csr(energy, f, DX, DY, bc)
    n = len(b)
    A = sp.csr_matrix((val, idx, ptr), shape=(n, n))
    A.sum_duplicates()
    return A, b, cf


def test_energy_equals_minus_residual_times_area():
    f = energy_identity_fields()
    Ar, br, _ = _mat(False, f, "periodic")
    Ae, be, _ = _mat(True, f, "periodic")
    expect = -Ar * (DX * DY)
    diff = (Ae - expect).toarray()
    scale = np.abs(expect.toarray()).max()
    assert np.abs(diff).max() <= 1e-12 * scale
    assert np.allclose(be, -br * DX * DY, rtol=1e-12, atol=1e-6)


@pytest.mark.parametrize("idir", [1, 2])
def test_front_rhs_sign(idir):
    """test_ssa_energy.f90:148-211: b = +taul*dy (ice on the low side), -taul*dy (high side)."""
    f = energy_identity_fields()
    nx, ny = f["f_ice"].shape
    f["f_ice"][:] = 0.0
    if idir == 1:
        f["f_ice"][2:5, :] = 1.0
        f["ssa_mask_acx"][1, :] = 3; f["taul_int_acx"][1, :] = 4.0e7
        f["ssa_mask_acx"][4, :] = 3; f["taul_int_acx"][4, :] = 6.0e7
    else:
        f["f_ice"][:, 2:5] = 1.0
        f["ssa_mask_acy"][:, 1] = 3; f["taul_int_acy"][:, 1] = 4.0e7
        f["ssa_mask_acy"][:, 4] = 3; f["taul_int_acy"][:, 4] = 6.0e7
    _, b, _ = _mat(True, f, "periodic")
    for i in range(nx):
        for j in range(ny):
            if idir == 1 and f["ssa_mask_acx"][i, j] == 3:
                nr = 2 * (i * ny + j)
                exp = f["taul_int_acx"][i, j] * DY * (-1 if i == 1 else 1)
            elif idir == 2 and f["ssa_mask_acy"][i, j] == 3:
                nr = 2 * (i * ny + j) + 1
                exp = f["taul_int_acy"][i, j] * DX * (-1 if j == 1 else 1)
            else:
                continue
            assert abs(b[nr] - exp) <= 1e-12 * abs(exp)


def _sym_cases():
    f = uniform_fields()
    yield "periodic", f, "periodic"
    yield "zeros", uniform_fields(), "zeros"
    g = uniform_fields()
    g["ssa_mask_acx"][:, 9 // 2 - 1] = 3
    g["ssa_mask_acy"][:, 9 // 2 - 1] = 3
    yield "front_strip", g, "periodic"
    I = np.arange(1, 10)[:, None] * np.ones((1, 9))
    J = np.arange(1, 10)[None, :] * np.ones((9, 1))
    for bc in ("infinite", "periodic-x", "periodic-y"):
        h = uniform_fields()
        h["N_aa"] = np.asfortranarray(1.0e10 * (1.0 + 0.3 * np.sin(I) * np.cos(0.7 * J)))
        yield f"tied_{bc}", h, bc


@pytest.mark.parametrize("name,f,bc", list(_sym_cases()), ids=[c[0] for c in _sym_cases()])
def test_energy_matrix_symmetric(name, f, bc):
    A, _, _ = _mat(True, f, bc)
    d = (A - A.T).toarray()
    assert np.abs(d).max() <= 1e-12 * np.abs(A.toarray()).max()


@pytest.mark.parametrize("axis", ["x", "y"])
def test_energy_reflection_equivariant(axis):
    """test_ssa_energy_lr_sym.f90: P K P^T = K, P b = b under the C-grid mirror."""
    n = 11
    f = uniform_fields(n, n)
    f["f_ice"][:] = 0.0
    f["beta_acx"][:] = 0.0
    f["beta_acy"][:] = 0.0
    f["taud_acx"][:] = 0.0
    f["taud_acy"][:] = 0.0
    if axis == "x":
        f["f_ice"][3:8, :] = 1.0
        f["ssa_mask_acx"][:] = 0
        f["ssa_mask_acx"][3:7, :] = 1
        f["ssa_mask_acx"][2, :] = 3; f["ssa_mask_acx"][7, :] = 3
        f["taul_int_acx"][2, :] = 5.0e7; f["taul_int_acx"][7, :] = 5.0e7
        f["ssa_mask_acy"][:] = 0
        f["ssa_mask_acy"][3:8, :] = 1
    else:
        f["f_ice"][:, 3:8] = 1.0
        f["ssa_mask_acy"][:] = 0
        f["ssa_mask_acy"][:, 3:7] = 1
        f["ssa_mask_acy"][:, 2] = 3; f["ssa_mask_acy"][:, 7] = 3
        f["taul_int_acy"][:, 2] = 5.0e7; f["taul_int_acy"][:, 7] = 5.0e7
        f["ssa_mask_acx"][:] = 0
        f["ssa_mask_acx"][:, 3:8] = 1
    A, b, _ = _mat(True, f, "periodic")
    N = 2 * n * n
    perm = np.zeros(N, dtype=int)
    sgn = np.zeros(N)
    for i in range(n):
        for j in range(n):
            q = i * n + j
            if axis == "x":
                # ux(i) -> -ux(n-2-i) (faces), uy(i) -> uy(n-1-i)  (0-based, periodic)
                perm[2 * q] = 2 * (((n - 2 - i) % n) * n + j); sgn[2 * q] = -1
                perm[2 * q + 1] = 2 * ((n - 1 - i) * n + j) + 1; sgn[2 * q + 1] = 1
            else:
                perm[2 * q + 1] = 2 * (i * n + (n - 2 - j) % n) + 1; sgn[2 * q + 1] = -1
                perm[2 * q] = 2 * (i * n + (n - 1 - j)); sgn[2 * q] = 1
    P = sp.csr_matrix((sgn, (perm, np.arange(N))), shape=(N, N))
    K = A.toarray()
    KP = (P @ A @ P.T).toarray()
    assert np.abs(KP - K).max() <= 1e-12 * np.abs(K).max()
    assert np.abs(P @ b - b).max() <= 1e-12 * np.abs(b).max()
