"""The algorithmic byte model behind the bench's roofline (yelmo_gb300.gpu.algorithmic_bytes):
per-cell counts of each step, the FP32 / FP64 word size of the Krylov step, and the
least-traffic form of each Krylov method. Host logic only: no GPU."""
import pytest

from yelmo_gb300 import abi, gpu

STATS = {"ssa_iter_now": 10, "ssa_lin_iter": 100, "active_cells": 500, "outer_iter": 30}


def _krylov(**kw):
    return gpu.algorithmic_bytes(STATS, abi.KIND_DIVA, 40, 30, 10, by_step=True, **kw)["krylov"]


def test_pipelined_cg_bytes_per_active_cell_and_iteration():
    # FP64: 42w + 8 with w = 8; no defect-correction term
    assert _krylov(mixed=False, cg=True) == 500 * 100 * (42 * 8 + 8)
    # mixed: FP32 words, plus 186 B per active cell and outer step
    assert _krylov(mixed=True, cg=True) == 500 * 100 * (42 * 4 + 8) + 500 * 30 * 186


def test_bicgstab_and_fp64_krylov_in_mixed_mode():
    assert _krylov(mixed=False, cg=False) == 500 * 100 * (62 * 8 + 16)
    # the residual form's BiCGSTAB with ILU(0) runs in FP64 in the mixed mode too
    assert _krylov(mixed=True, cg=False, krylov64=True) == 500 * 100 * (62 * 8 + 16) + 500 * 30 * 186


@pytest.mark.parametrize("cg,words", [(True, 23), (False, 36)])
def test_least_traffic_form(cg, words):
    full = _krylov(mixed=False, cg=cg)
    least = _krylov(mixed=False, cg=cg, minimal=True)
    assert least == 500 * 100 * words * 8
    assert least < full


def test_pre_and_post_steps_count_every_cell():
    st = gpu.algorithmic_bytes(STATS, abi.KIND_DIVA, 40, 30, 10, mixed=False, by_step=True)
    w, n2, it = 8, 40 * 30, 10
    pre = 7 * w + (3 * 10 + 14) * w + (20 * w + 8) + (16 * w + 8)
    assert st["pre"] == n2 * it * pre
    assert st["post"] == n2 * it * (16 * w + 8)
    # the mixed mode adds the FP32 coefficient copies to the pre step
    stm = gpu.algorithmic_bytes(STATS, abi.KIND_DIVA, 40, 30, 10, mixed=True, by_step=True)
    assert stm["pre"] == n2 * it * (pre + 72)
