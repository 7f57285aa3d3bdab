"""Grouping of the terms on the device (qr_group.cu), checked against numpy.

At creation the terms are sorted stably by x with an LSD radix sort (8-bit
digits, so n = 63 takes 8 passes and T > 2,048 spans several tiles), cut into
groups of equal x in ascending order (make_row's sort,
qrusty/src/accel.rs:188-208), and terms with equal (x, z) are merged into
strings numbered by first occurrence.  qr_op_get_groups reads the result
back; it must equal numpy's stable argsort and a first-occurrence dictionary.
The CSR tables built from it on the device (position trie, spans, sign-class
folds) are checked bit for bit against the oracle, and after a device
coefficient update the CSR coefficient tables follow without a host copy.
"""
import numpy as np
import pytest

from qrusty_gb300 import PauliOperator
from qrusty_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def _expected(x, z):
    order = np.argsort(x, kind="stable")
    gx, counts = np.unique(x, return_counts=True)
    goff = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
    first = {}
    mmap = np.empty(len(x), dtype=np.uint32)
    for k, key in enumerate(zip(x.tolist(), z.tolist())):
        mmap[k] = first.setdefault(key, len(first))
    return gx, goff, order.astype(np.uint32), mmap, len(first)


def _case(rng, n, T, xbits, zbits):
    x = rng.integers(0, 1 << min(xbits, 62), T, dtype=np.uint64)
    z = rng.integers(0, 1 << min(zbits, 62), T, dtype=np.uint64)
    if n == 63:  # masks with the top bit set: the eighth radix pass
        top = rng.random(T) < 0.5
        x[top] |= np.uint64(1 << 62)
        z[rng.random(T) < 0.5] |= np.uint64(1 << 62)
    ph = rng.integers(0, 4, T).astype(np.uint8)
    c = (rng.standard_normal(T) + 1j * rng.standard_normal(T)).astype(np.complex128)
    return W.Terms(n, x, z, ph, c)


CASES = [
    # n, T, x bits, z bits
    (1, 1, 1, 1),
    (2, 7, 2, 2),
    (10, 300, 3, 2),        # heavy duplicates: long merged runs
    (12, 5000, 4, 3),       # several radix tiles, every x-group spans tiles
    (20, 6000, 20, 20),     # nearly all distinct
    (40, 4097, 40, 6),      # five radix passes, one past a tile boundary
    (63, 3000, 63, 63),     # eight radix passes, top bit set
]


@pytest.mark.parametrize("n,T,xb,zb", CASES)
def test_device_grouping_matches_numpy(cuda, n, T, xb, zb):
    rng = np.random.default_rng(1000 + n * 7 + T)
    t = _case(rng, n, T, min(xb, n), min(zb, n))
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    got = op.groups()
    gx, goff, order, mmap, M = _expected(t.x, t.z)
    assert np.array_equal(got["gx"], gx)
    assert np.array_equal(got["goff"], goff)
    assert np.array_equal(got["order"], order)
    assert np.array_equal(got["mmap"], mmap)
    if n <= 20:  # info builds the apply plans (a 2^n diagonal among them)
        inf = op.info()
        assert inf["ngroups"] == len(gx) and inf["nmerged"] == M


def test_device_grouping_millions_of_terms(cuda):
    """4.5 million terms: the scans run several top-level chunks and the
    radix sort thousands of tiles; checked with vectorised numpy."""
    rng = np.random.default_rng(4242)
    T, n = 4_500_000, 40
    x = rng.integers(0, 1 << 14, T, dtype=np.uint64) << np.uint64(20)
    z = rng.integers(0, 1 << 6, T, dtype=np.uint64) | (x >> np.uint64(3))
    ph = rng.integers(0, 4, T).astype(np.uint8)
    c = rng.standard_normal(T).astype(np.complex128)
    op = PauliOperator(n, x, z, ph, c)
    got = op.groups()
    assert np.array_equal(got["order"], np.argsort(x, kind="stable").astype(np.uint32))
    gx, counts = np.unique(x, return_counts=True)
    assert np.array_equal(got["gx"], gx)
    assert np.array_equal(got["goff"], np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32))
    # merged strings numbered by first occurrence
    keys = np.stack([x, z], axis=1)
    _, first, inv = np.unique(keys, axis=0, return_index=True, return_inverse=True)
    rank = np.empty(len(first), dtype=np.int64)
    rank[np.argsort(first, kind="stable")] = np.arange(len(first))
    assert np.array_equal(got["mmap"], rank[inv.reshape(-1)].astype(np.uint32))


def _check_csr(oracle, op, t, c):
    ip, ij, d = op.csr_host()
    oi, oj, od = oracle.csr_build(t.n, t.x, t.z, oracle.make_params(t.phase, c), step=1024)
    assert np.array_equal(ip, oi)
    assert np.array_equal(ij, oj)
    assert np.array_equal(_bits(d), _bits(od))


def _diag_heavy(rng, n, T):
    """x in a handful of masks, z spread: groups of span rank > 10 (fold mode
    with a prefix table), rank 5..10, and rank <= 4; duplicates included."""
    xs = np.array([0, 1, 0b110, 1 << (n - 1)], dtype=np.uint64)
    x = xs[rng.integers(0, len(xs), T)]
    z = rng.integers(0, 1 << n, T).astype(np.uint64)
    z[x == xs[2]] &= np.uint64(0b11111)        # rank <= 5
    z[x == xs[1]] &= np.uint64(0b11)           # rank <= 2
    z[:T // 10] = z[T // 10:2 * (T // 10)]     # repeated (x, z) strings
    x[:T // 10] = x[T // 10:2 * (T // 10)]
    ph = rng.integers(0, 4, T).astype(np.uint8)
    c = (rng.standard_normal(T) + 1j * rng.standard_normal(T)).astype(np.complex128)
    c[rng.random(T) < 0.1] = 0.0               # explicit zeros (signed-zero folds)
    return W.Terms(n, x, z, ph, c)


@pytest.mark.parametrize("n,T", [(9, 40), (11, 3000), (12, 700)])
def test_csr_tables_from_device_grouping(cuda, oracle, n, T):
    rng = np.random.default_rng(n * 31 + T)
    t = _diag_heavy(rng, n, T)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    _check_csr(oracle, op, t, t.coeff)


def test_csr_follows_device_coefficient_update(cuda, oracle):
    """CSR built, coefficients changed on the device (no host copy), CSR
    built again: both bit-exact against the oracle, and the diagonal too."""
    import torch
    rng = np.random.default_rng(5)
    t = _diag_heavy(rng, 10, 900)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    _check_csr(oracle, op, t, t.coeff)
    c1 = (rng.standard_normal(t.T) + 1j * rng.standard_normal(t.T)).astype(np.complex128)
    c1[::7] = 0.0
    c1d = torch.from_numpy(c1).to(cuda)
    torch.cuda.synchronize()
    torch.cuda.set_sync_debug_mode("error")
    try:
        op.set_coeffs_device(c1d)
    finally:
        torch.cuda.set_sync_debug_mode("default")
    _check_csr(oracle, op, t, c1)
    fresh = PauliOperator(t.n, t.x, t.z, t.phase, c1)
    assert torch.equal(op.diagonal(), fresh.diagonal())
    # and a host update after it
    op.set_coeffs(t.coeff)
    _check_csr(oracle, op, t, t.coeff)


def test_merged_strings_drive_apply_and_grad(cuda, oracle):
    """Many repeated strings: the merged coefficients (FP64 fold in input
    order) feed the apply plans and the term gradients."""
    import torch
    rng = np.random.default_rng(9)
    t = _diag_heavy(rng, 11, 2500)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    psi = W.random_state(rng, 1 << t.n)
    y = op.apply(torch.from_numpy(psi).to(cuda)).cpu().numpy()
    yo = oracle.apply(t.n, t.x, t.z, oracle.make_params(t.phase, t.coeff), psi)
    assert np.linalg.norm(y - yo) <= 1e-12 * np.linalg.norm(yo)
    g = W.random_state(rng, 1 << t.n)
    R = op.term_grad(torch.from_numpy(psi).to(cuda), torch.from_numpy(g).to(cuda)).cpu().numpy()
    Ro = oracle.term_grad(t.n, t.x, t.z, t.phase, psi, g)
    assert np.abs(R - Ro).max() <= 1e-12 * np.abs(Ro).max()
