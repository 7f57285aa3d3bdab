"""Matrix-free H psi on the GPU vs the oracle (CSR-build + SpMV restated).

Tolerances: complex128 kernel rel. err <= 1e-12 (||y - y_ref|| / ||y_ref||);
compensated complex64 kernel rel. err <= 1e-6 against the FP64 oracle.
"""
import numpy as np
import pytest
import scipy.sparse as sps

from qrusty_gb300 import PauliOperator, Pauli, SparsePauliOp, spmat_dot_densevec, csr_matrix
from qrusty_gb300 import workloads as W
from tests.helpers import terms_of_labels

pytestmark = pytest.mark.gpu

TOL_C128 = 1e-12
TOL_C64C = 1e-6


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def oracle_y(oracle, n, x, z, ph, c, psi):
    return oracle.apply(n, x, z, oracle.make_params(ph, c), psi)


def run_both(cuda, op, psi):
    import torch
    p128 = torch.from_numpy(psi).to(cuda)
    y128 = op.apply(p128)
    y64 = op.apply(p128.to(torch.complex64))
    op.sync_check()
    return y128.cpu().numpy(), y64.cpu().numpy().astype(np.complex128)


def check(cuda, oracle, n, x, z, ph, c, psi=None, seed=0):
    if psi is None:
        psi = W.random_state(np.random.default_rng(seed), 1 << n)
    op = PauliOperator(n, x, z, ph, c)
    y_ref = oracle_y(oracle, n, x, z, ph, c, psi)
    y128, y64 = run_both(cuda, op, psi)
    e128, e64 = rel(y128, y_ref), rel(y64, y_ref)
    assert e128 <= TOL_C128, e128
    assert e64 <= TOL_C64C, e64
    return op, e128, e64


@pytest.mark.parametrize("name", ["H2", "H4", "H6"])
def test_fixtures(cuda, oracle, golden, name):
    check(cuda, oracle, *terms_of_labels(*golden[name]))


def test_cfg0(cuda, oracle):
    t, psi = W.cfg0()
    op, e128, e64 = check(cuda, oracle, t.n, t.x, t.z, t.phase, t.coeff, psi)
    info = op.info()
    assert info["ngroups"] == 176 and info["nterms"] == 200


@pytest.mark.parametrize("n", [10, 16])
def test_chain(cuda, oracle, n):
    t, psi = W.cfg1(n=n)
    op, _, _ = check(cuda, oracle, t.n, t.x, t.z, t.phase, t.coeff, psi)
    assert op.info()["has_diag"] == 1  # ZZ chain: z span rank n-1 > table limit


def test_chain_full_n22(cuda, oracle):
    t, psi = W.cfg1()
    check(cuda, oracle, t.n, t.x, t.z, t.phase, t.coeff, psi)


@pytest.mark.parametrize("n,npair,nz", [(14, 2000, 500), (16, 4000, 1000)])
def test_jw(cuda, oracle, n, npair, nz):
    t = W.cfg2(n=n, npair=npair, nz=nz)
    check(cuda, oracle, t.n, t.x, t.z, t.phase, t.coeff, seed=n)


def test_fat_groups(cuda, oracle):
    # x = 0b1 with seven independent z strings: rank 7 > 4 -> term-by-term group
    rng = np.random.default_rng(5)
    n = 9
    zs = rng.integers(0, 1 << n, 12).astype(np.uint64)
    x = np.concatenate([np.full(12, 1, np.uint64), np.full(12, 6, np.uint64)])
    z = np.concatenate([zs, zs[::-1]])
    ph = rng.integers(0, 4, 24).astype(np.uint8)
    c = rng.standard_normal(24) + 1j * rng.standard_normal(24)
    op, _, _ = check(cuda, oracle, n, x, z, ph, c)
    assert op.info()["nfat"] >= 1


@pytest.mark.parametrize("n,T", [(12, 2000), (14, 3000), (17, 1500)])
def test_many_sub_groups(cuda, oracle, n, T):
    """Random-letter operators with thousands of x groups: the compensated
    kernel's factor table is rebuilt per chunk of <= 512 sub-groups; at n = 12
    every group shares one partner tile, which is visited as several blocks."""
    rng = np.random.default_rng(n * 1000 + T)
    t = W.random_letters_op(rng, n, T)
    c = t.coeff * (1 - 0.4j)
    psi = W.random_state(rng, 1 << n)
    op, _, _ = check(cuda, oracle, t.n, t.x, t.z, t.phase, c, psi)
    assert op.info()["nsub"] > 512


def test_small_diag_group_in_table(cuda, oracle):
    # x = 0 group of rank <= 4 stays a regular table group (no diagonal vector)
    n = 13
    x = np.array([0, 0, 0, 3, 1 << 12], np.uint64)
    z = np.array([1, 6, 7, 0, 5], np.uint64)
    op, _, _ = check(cuda, oracle, n, x, z, np.zeros(5, np.uint8), np.array([1, .5, -.25, .3, .7]))
    assert op.info()["has_diag"] == 0


@pytest.mark.parametrize("n", [1, 2, 5, 9, 12, 13, 14])
def test_sizes(cuda, oracle, n):
    rng = np.random.default_rng(n)
    t = W.random_letters_op(rng, n, 40)
    c = t.coeff * (1 + 0.3j)  # non-Hermitian
    check(cuda, oracle, t.n, t.x, t.z, t.phase, c, seed=n)


def test_adjoint(cuda, oracle):
    import torch
    rng = np.random.default_rng(11)
    n = 11
    t = W.random_letters_op(rng, n, 120)
    c = t.coeff + 1j * rng.standard_normal(t.T)
    cp = oracle.make_params(t.phase, c)
    ip, ij, d = oracle.csr_build(n, t.x, t.z, cp)
    A = sps.csr_matrix((d, ij.astype(np.int64), ip.astype(np.int64)), shape=(1 << n, 1 << n))
    psi = W.random_state(rng, 1 << n)
    want = A.conj().T @ psi
    op = PauliOperator(n, t.x, t.z, t.phase, c)
    p = torch.from_numpy(psi).to(cuda)
    y128 = op.apply(p, adjoint=True).cpu().numpy()
    y64 = op.apply(p.to(torch.complex64), adjoint=True).cpu().numpy()
    assert rel(y128, want) <= TOL_C128
    assert rel(y64.astype(np.complex128), want) <= TOL_C64C


def register_split_op(rng, n, ngroups):
    """x groups whose terms' z differ in register bits of the compensated
    kernel's layout (bits 9-11 of a 4,096-amplitude tile; thread t holds
    amplitudes t + 512 m, m < 8).  Variant by group index g: the split bit
    cycles through 9, 10, 11; the sign pattern z & 0xe00 is zero or not; z on
    the thread bits (0-8) is zero or not; the group has rank 0, 1 (a tile
    bit) or 2 (a thread bit too) inside each half; every fifth group is split
    on two register bits (four sub-groups)."""
    xs, zs, ph = [], [], []
    seen = set()
    for g in range(ngroups):
        while True:
            hi = int(rng.integers(0, 1 << (n - 12)))
            reg = int(rng.integers(0, 8)) if g % 2 else 0
            x = (hi << 12) | (reg << 9) | int(rng.integers(0, 1 << 9))
            if x and x not in seen:
                seen.add(x)
                break
        z0 = int(rng.integers(0, 1 << n))
        if g % 3 == 0:
            z0 &= ~0x1ff          # factor constant over the thread index
        if g % 4 == 1:
            z0 &= ~0xe00          # no register-bit sign pattern
        bb = 1 << (9 + g % 3)
        zg = [z0, z0 ^ bb]
        if g % 5 == 4:
            b2 = 1 << (9 + (g + 1) % 3)
            zg += [z0 ^ b2, z0 ^ bb ^ b2]
        if g % 4 >= 2:            # rank 1 on a tile bit
            t1 = 1 << int(rng.integers(12, n))
            zg += [z ^ t1 for z in zg]
        if g % 4 == 3:            # rank 2: a thread bit too
            t2 = 1 << int(rng.integers(0, 9))
            zg += [z ^ t2 for z in zg]
        for z in zg:
            xs.append(x)
            zs.append(z)
            ph.append(int(rng.integers(0, 4)))
    T = len(xs)
    c = rng.standard_normal(T) + 1j * rng.standard_normal(T)
    return (np.array(xs, np.uint64), np.array(zs, np.uint64), np.array(ph, np.uint8), c)


@pytest.mark.parametrize("n,ngroups", [(13, 40), (15, 90)])
def test_register_bit_split_groups(cuda, oracle, n, ngroups):
    """Sub-groups of one x group that differ in one register bit of z share
    their partner loads in the compensated kernel (fused pairs): every key
    variant, forward and adjoint, against the oracle."""
    import torch
    rng = np.random.default_rng(31 * n + ngroups)
    x, z, ph, c = register_split_op(rng, n, ngroups)
    psi = W.random_state(rng, 1 << n)
    op, _, _ = check(cuda, oracle, n, x, z, ph, c, psi)
    assert ngroups < op.info()["nsub"] <= 512
    cp = oracle.make_params(ph, c)
    ip, ij, d = oracle.csr_build(n, x, z, cp)
    A = sps.csr_matrix((d, ij.astype(np.int64), ip.astype(np.int64)), shape=(1 << n, 1 << n))
    want = A.conj().T @ psi
    p = torch.from_numpy(psi).to(cuda)
    y128 = op.apply(p, adjoint=True).cpu().numpy()
    y64 = op.apply(p.to(torch.complex64), adjoint=True).cpu().numpy()
    assert rel(y128, want) <= TOL_C128
    assert rel(y64.astype(np.complex128), want) <= TOL_C64C


def test_multi_state(cuda, oracle):
    import torch
    t, _ = W.cfg1(with_state=False, n=14)
    rng = np.random.default_rng(9)
    psi = W.random_state(rng, 1 << 14, nstates=3)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    y = op.apply(torch.from_numpy(psi).to(cuda)).cpu().numpy()
    for s in range(3):
        ref = oracle_y(oracle, t.n, t.x, t.z, t.phase, t.coeff, psi[s])
        assert rel(y[s], ref) <= TOL_C128


def test_host_entry_matches_device(cuda):
    import torch
    t, psi = W.cfg0()
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    yh = op.apply(psi)  # numpy -> qr_apply_host
    yd = op.apply(torch.from_numpy(psi).to(cuda)).cpu().numpy()
    assert np.array_equal(yh, yd)
    yh64 = op.apply(psi.astype(np.complex64))
    yd64 = op.apply(torch.from_numpy(psi).to(cuda).to(torch.complex64)).cpu().numpy()
    assert np.array_equal(yh64, yd64)
    # three pageable states: per-state copies overlapped with the kernels
    psi3 = W.random_state(np.random.default_rng(4), 1 << t.n, nstates=3).reshape(-1)
    for dt in (np.complex128, np.complex64):
        p = psi3.astype(dt)
        yh3 = op.apply(p)
        yd3 = op.apply(torch.from_numpy(p).to(cuda)).cpu().numpy()
        assert np.array_equal(yh3, yd3)


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_host_entry_pinned_output(cuda, dtype):
    """Page-locked y: the kernel writes the result straight into host memory
    (no staging copy); same bits as the device entry, two states, both the
    operator and its adjoint, and psi and y the same buffer."""
    import torch
    t = W.cfg2(n=14)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    rng = np.random.default_rng(9)
    psi = W.random_state(rng, 1 << t.n, nstates=2).astype(dtype).reshape(-1)
    tdt = torch.complex128 if dtype == np.complex128 else torch.complex64
    h_in = torch.from_numpy(psi.copy()).pin_memory()
    h_out = torch.empty_like(h_in).pin_memory()
    for adj in (False, True):
        yd = op.apply(torch.from_numpy(psi).to(cuda), adjoint=adj).cpu().numpy()
        h_out.fill_(float("nan"))
        op.apply(h_in.numpy(), out=h_out.numpy(), adjoint=adj)
        assert h_out.dtype == tdt and np.array_equal(h_out.numpy(), yd)
    inplace = h_in.clone().pin_memory()
    op.apply(inplace.numpy(), out=inplace.numpy())
    assert np.array_equal(inplace.numpy(), op.apply(torch.from_numpy(psi).to(cuda)).cpu().numpy())


def test_spmat_dot_densevec(cuda, oracle, golden):  # test_it.py:218-230
    m = Pauli("IX").to_matrix()
    x = np.array([1.0 + 2j, 2.0 + 3j, 3.0 + 4j, 4.0 + 5j])
    assert np.allclose(spmat_dot_densevec(m, x), csr_matrix(Pauli("IX").to_matrix()).dot(x))
    labels, coeffs = golden["H6"]
    H6 = SparsePauliOp([Pauli(l) for l in labels], list(coeffs))
    m = H6.to_matrix_mode("RowwiseUnsafeChunked/1000")
    rng = np.random.default_rng(1)
    v = rng.random(4096) + 1j * rng.random(4096)
    y = spmat_dot_densevec(m, v)
    ip, ij, d = m._it[3], m._it[2], m._it[1]
    y_or = oracle.spmv(ip, ij, d, v)
    assert rel(y, y_or) <= TOL_C128
    assert np.allclose(y, csr_matrix(m).dot(v))


def test_full_size_jw_properties(cuda, oracle):
    """26-qubit, 10k-term workload: sampled rows vs the oracle, c64c vs c128,
    linearity and Hermiticity (real coefficients)."""
    import torch
    t = W.cfg2()
    n, N = t.n, 1 << t.n
    op = PauliOperator(n, t.x, t.z, t.phase, t.coeff)
    g = torch.Generator(device=cuda).manual_seed(1234)
    psi = torch.complex(torch.randn(N, device=cuda, dtype=torch.float64, generator=g),
                        torch.randn(N, device=cuda, dtype=torch.float64, generator=g))
    psi /= torch.linalg.vector_norm(psi)
    y = op.apply(psi)
    y64 = op.apply(psi.to(torch.complex64))
    op.sync_check()
    e = float(torch.linalg.vector_norm(y64.to(torch.complex128) - y) / torch.linalg.vector_norm(y))
    assert e <= TOL_C64C, e
    # sampled rows vs oracle
    rng = np.random.default_rng(2)
    rows = np.unique(np.concatenate([[0, N - 1], rng.integers(0, N, 62)]))
    psi_h = psi.cpu().numpy()
    cp = oracle.make_params(t.phase, t.coeff)
    y_h = y.cpu().numpy()
    for r in rows[:16]:
        ref = oracle.apply_rows(t.x, t.z, cp, psi_h, int(r), int(r) + 1)[0]
        assert abs(y_h[r] - ref) <= 1e-12 * max(1e-300, float(np.abs(y_h).max())) * 10, r
    blk = oracle.apply_rows(t.x, t.z, cp, psi_h, 4096, 4096 + 512)
    assert rel(y_h[4096:4608], blk) <= TOL_C128
    # a 65,536-row block (16 output tiles, unaligned start) against the FP64
    # oracle: complex128 at 1e-12; compensated complex64 at 1e-6, both on
    # the complex64-rounded state it was given (the kernel's own error) and
    # on the FP64 state before rounding (what a caller converting sees)
    lo = (0x2A5B << 12) + 777
    hi = lo + 65536
    ref = oracle.apply_rows(t.x, t.z, cp, psi_h, lo, hi)
    assert rel(y_h[lo:hi], ref) <= TOL_C128
    y64_h = y64.cpu().numpy()[lo:hi].astype(np.complex128)
    assert rel(y64_h, ref) <= TOL_C64C
    psi64_h = psi.to(torch.complex64).cpu().numpy().astype(np.complex128)
    ref64 = oracle.apply_rows(t.x, t.z, cp, psi64_h, lo, hi)
    assert rel(y64_h, ref64) <= TOL_C64C
    del psi_h, y_h, psi64_h
    # linearity and Hermiticity
    phi = torch.complex(torch.randn(N, device=cuda, dtype=torch.float64, generator=g),
                        torch.randn(N, device=cuda, dtype=torch.float64, generator=g))
    a, b = 0.3 - 0.7j, -1.1 + 0.2j
    lhs = op.apply(a * psi + b * phi)
    hphi = op.apply(phi)
    rhs = a * y + b * hphi
    assert float(torch.linalg.vector_norm(lhs - rhs) / torch.linalg.vector_norm(rhs)) <= 1e-12
    s1 = torch.vdot(phi, y)
    s2 = torch.vdot(hphi, psi)
    assert abs(complex(s1) - complex(s2)) <= 1e-10 * abs(complex(s1))
