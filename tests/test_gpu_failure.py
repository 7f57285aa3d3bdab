"""Failure path of the apply kernels, made to fire without a GPU fault.

Every mbarrier wait in the apply kernels is bounded.  When one runs out, the
kernel records an error word, stops computing, waits (bounded) for the
partner-tile copies it did issue, and returns; ``qr_check`` reports
QR_EKERNEL and the context stays usable.  The tests reach that path with the
operator's test hooks: CTA 0 never issues the copy of one ring step (a
barrier phase that nothing completes) and the wait bound is 50 ms.  Nothing
is left in flight: the withheld copy was never issued.  After the hooks are
cleared, the same operator must return the normal result bit for bit.
Reference error model: QrustyErr (qrusty/src/lib.rs:34-52), an error value
rather than an abort.
"""
import numpy as np
import pytest

from qrusty_gb300 import PauliOperator, QrError, _lib
from qrusty_gb300 import workloads as W

pytestmark = pytest.mark.gpu

WAIT_NS = 50_000_000  # 50 ms: the withheld step's wait runs out after this


def _expect_kernel_error_then_recover(cuda, op, psi, withhold):
    import torch
    y_ref = op.apply(psi)
    op.sync_check()
    op.set_test_hooks(wait_ns=WAIT_NS, withhold_step=withhold)
    y_bad = op.apply(psi)
    with pytest.raises(QrError) as ei:
        op.sync_check()
    assert ei.value.code == _lib.QR_EKERNEL
    assert "bounded mbarrier wait expired" in str(ei.value)
    del y_bad
    # the error word was cleared when reported; hooks off: normal results
    op.set_test_hooks()
    y = op.apply(psi)
    op.sync_check()
    assert torch.equal(y, y_ref)
    # and a second apply on the same operator is clean as well
    y2 = op.apply(psi)
    op.sync_check()
    assert torch.equal(y2, y_ref)


def _state(cuda, n, dtype, seed=5):
    import torch
    psi = W.random_state(np.random.default_rng(seed), 1 << n)
    return torch.from_numpy(psi).to(cuda).to(dtype)


def test_pair_kernel_withheld_copy(cuda):
    """apply_c64c_pair: partner tiles two per ring slot; step 2 is the first
    refill (steps 0 and 1 are the prologue)."""
    import torch
    t = W.cfg2(n=16, npair=600, nz=200)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    info = op.info()
    assert info["tile_bits"] == 12 and info["nsub"] <= 512 and info["nblocks"] >= 6
    psi = _state(cuda, t.n, torch.complex64)
    for step in (0, 2, 3):
        _expect_kernel_error_then_recover(cuda, op, psi, step)


def test_chunked_table_kernel_withheld_copy(cuda):
    """apply_c64c_tab with several table chunks (more than 512 sub-groups)."""
    import torch
    rng = np.random.default_rng(77)
    t = W.random_letters_op(rng, 14, 1500)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    info = op.info()
    # 4 partner tiles, split into 5 blocks of <= 512 sub-groups; steps 0-3 are
    # the prologue, step 4 the first refill
    assert info["nsub"] > 512 and info["nblocks"] >= 5
    psi = _state(cuda, t.n, torch.complex64)
    for step in (1, 4):
        _expect_kernel_error_then_recover(cuda, op, psi, step)


def test_single_tile_table_kernel_withheld_copy(cuda):
    """apply_c64c_tab with one partner tile (n = 11: 512 threads x 4
    amplitudes, one output tile): the withheld copy is the prologue's."""
    import torch
    rng = np.random.default_rng(78)
    t = W.random_letters_op(rng, 11, 200)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    psi = _state(cuda, t.n, torch.complex64)
    _expect_kernel_error_then_recover(cuda, op, psi, 0)


def test_complex128_kernel_withheld_copy(cuda):
    """apply_c128 (decoupled warps, per-stage release counters): the abort
    flag, then the drain of the copies issued into each stage."""
    import torch
    t = W.cfg2(n=16, npair=600, nz=200)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    psi = _state(cuda, t.n, torch.complex128)
    for step in (0, 3):
        _expect_kernel_error_then_recover(cuda, op, psi, step)


def test_hooks_validate_arguments(cuda):
    t = W.cfg2(n=12, npair=50, nz=10)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    with pytest.raises(QrError, match="below 1 ms"):
        op.set_test_hooks(wait_ns=1000)
    with pytest.raises(QrError, match="withhold_step"):
        op.set_test_hooks(withhold_step=-2)
    op.set_test_hooks()
