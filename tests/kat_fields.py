"""Synthetic assembler inputs of the reference's own unit tests.

tests/test_ssa_energy.f90:58-78 (8x8 periodic, spatially varying fields),
tests/test_ssa_energy_sym.f90:52-67 (9x9 uniform fields) and
tests/test_ssa_energy_lr_sym.f90 (11x11 ice strip with calving fronts),
restated here as numpy arrays (i, j are the Fortran 1-based indices).
"""
import numpy as np


def _F(a, dtype=np.float64):
    return np.asfortranarray(a, dtype=dtype)


def energy_identity_fields(nx=8, ny=8):
    """tests/test_ssa_energy.f90:58-78."""
    I = np.arange(1, nx + 1, dtype=np.float64)[:, None] + np.zeros((1, ny))
    J = np.arange(1, ny + 1, dtype=np.float64)[None, :] + np.zeros((nx, 1))
    f = {
        "z_bed": _F(np.full((nx, ny), -1000.0)),
        "z_sl": _F(np.zeros((nx, ny))),
        "H_ice": _F(1000.0 + 50.0 * np.sin(I) + 30.0 * np.cos(J)),
        "f_ice": _F(np.ones((nx, ny))),
        "N_aa": _F(1.0e10 * (1.0 + 0.2 * np.sin(0.5 * I) * np.cos(0.5 * J))),
        "beta_acx": _F(1.0e3 * (1.0 + 0.1 * I)),
        "beta_acy": _F(1.0e3 * (1.0 + 0.1 * J)),
        "taud_acx": _F(-5.0e4 + 1.0e3 * (I + J)),
        "taud_acy": _F(-3.0e4 + 5.0e2 * (I - J)),
        "ux": _F(10.0 + 0.5 * I),
        "uy": _F(5.0 + 0.3 * J),
        "taul_int_acx": _F(np.zeros((nx, ny))),
        "taul_int_acy": _F(np.zeros((nx, ny))),
        "ssa_mask_acx": _F(np.ones((nx, ny)), np.int32),
        "ssa_mask_acy": _F(np.ones((nx, ny)), np.int32),
    }
    return f


def uniform_fields(nx=9, ny=9):
    """tests/test_ssa_energy_sym.f90:52-67."""
    s = (nx, ny)
    return {
        "H_ice": _F(np.full(s, 1000.0)), "f_ice": _F(np.ones(s)),
        "z_bed": _F(np.full(s, -1000.0)), "z_sl": _F(np.zeros(s)),
        "N_aa": _F(np.full(s, 1.0e10)), "beta_acx": _F(np.full(s, 1.0e3)),
        "beta_acy": _F(np.full(s, 1.0e3)), "taud_acx": _F(np.full(s, -5.0e4)),
        "taud_acy": _F(np.full(s, -5.0e4)), "ux": _F(np.full(s, 10.0)), "uy": _F(np.full(s, 10.0)),
        "taul_int_acx": _F(np.zeros(s)), "taul_int_acy": _F(np.zeros(s)),
        "ssa_mask_acx": _F(np.ones(s), np.int32), "ssa_mask_acy": _F(np.ones(s), np.int32),
    }
