"""GPU CSR construction vs the oracle (qrusty's rowwise builder restated):
indptr / indices bit-exact, values bit-exact (same term-order FP64 fold)."""
import numpy as np
import pytest

from qrusty_gb300 import PauliOperator, Pauli, SparsePauliOp, csr_matrix
from qrusty_gb300 import workloads as W
from tests.helpers import kron_dense, terms_of_labels

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def check_csr(oracle, n, x, z, ph, c, sample_rows=None):
    op = PauliOperator(n, x, z, ph, c)
    indptr, indices, data = op.csr_host()
    cp = oracle.make_params(ph, c)
    G = len(np.unique(x))
    N = 1 << n
    assert len(indices) == N * G
    if sample_rows is None:
        oi, oj, od = oracle.csr_build(n, x, z, cp, step=1024)
        assert np.array_equal(indptr, oi)
        assert np.array_equal(indices, oj)
        assert np.array_equal(_bits(data), _bits(od))
    else:
        assert np.array_equal(indptr, np.arange(N + 1, dtype=np.uint64) * np.uint64(G))
        for r in sample_rows:
            cols, vals = oracle.make_row(x, z, cp, r)
            lo = r * G
            assert np.array_equal(indices[lo:lo + G], cols)
            assert np.array_equal(_bits(data[lo:lo + G]), _bits(vals))
    return op, (indptr, indices, data)


@pytest.mark.parametrize("name", ["H2", "H4", "H6"])
def test_fixtures(cuda, oracle, golden, name):
    labels, coeffs = golden[name]
    check_csr(oracle, *terms_of_labels(labels, coeffs))


def test_fixture_H8_rows(cuda, oracle, golden):
    labels, coeffs = golden["H8"]
    n, x, z, ph, c = terms_of_labels(labels, coeffs)
    rng = np.random.default_rng(3)
    rows = [0, 1, (1 << n) - 1] + [int(v) for v in rng.integers(0, 1 << n, 40)]
    check_csr(oracle, n, x, z, ph, c, sample_rows=rows)


def test_cfg0(cuda, oracle):
    t, _ = W.cfg0(with_state=False)
    check_csr(oracle, t.n, t.x, t.z, t.phase, t.coeff)


def test_cfg1_small(cuda, oracle):
    t, _ = W.cfg1(with_state=False, n=12)
    check_csr(oracle, t.n, t.x, t.z, t.phase, t.coeff)


def test_jw_small(cuda, oracle):
    t = W.cfg2(n=12, npair=600, nz=150)
    check_csr(oracle, t.n, t.x, t.z, t.phase, t.coeff)


@pytest.mark.parametrize("seed", range(6))
def test_random_edge_cases(cuda, oracle, seed):
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(1, 11))
    T = int(rng.integers(1, 60))
    # few distinct strings so that duplicates and cancellations occur
    pool = rng.integers(0, 1 << n, size=(max(1, T // 3), 2)).astype(np.uint64)
    pick = rng.integers(0, len(pool), T)
    x, z = pool[pick, 0], pool[pick, 1]
    ph = rng.integers(0, 4, T).astype(np.uint8)
    c = (rng.integers(-2, 3, T) + 1j * rng.integers(-2, 3, T)).astype(np.complex128)
    check_csr(oracle, n, x, z, ph, c)


def test_single_term_and_n1(cuda, oracle):
    check_csr(oracle, 1, np.array([1], np.uint64), np.array([1], np.uint64),
              np.array([1], np.uint8), np.array([0.5 - 2j]))
    check_csr(oracle, 5, np.array([0], np.uint64), np.array([0], np.uint64),
              np.array([0], np.uint8), np.array([3.0]))


def test_cancellation_zero_kept(cuda, oracle):
    x = np.array([1, 1, 2], np.uint64)
    z = np.array([0, 0, 2], np.uint64)
    op, (ip, ij, d) = check_csr(oracle, 2, x, z, np.zeros(3, np.uint8),
                                np.array([1.0, -1.0, 0.5]))
    assert np.count_nonzero(d == 0) == 4


@pytest.mark.parametrize("kind", ["real", "imag", "neg_zero", "mixed"])
def test_fold_group_signed_zero_parts(cuda, oracle, kind):
    """A group whose z span exceeds the class-table rank is folded per row;
    a part whose coefficients are all +-0 is formed without FP64 additions
    and must carry the same zero sign as the term-order fold."""
    rng = np.random.default_rng(7)
    n, T = 9, 24
    x = np.zeros(T, np.uint64)
    z = rng.integers(1, 1 << n, T).astype(np.uint64)
    z[3:9] = 1 << np.arange(6, dtype=np.uint64)  # GF(2) rank >= 6: fold mode
    ph = rng.choice(np.array([0, 2], np.uint8), T)  # phase 2 flips the zero's sign
    v = rng.uniform(-1, 1, T)
    if kind == "real":
        c = v + 0j
    elif kind == "imag":
        c = 1j * v
    elif kind == "neg_zero":
        c = np.array([complex(a, -0.0) for a in v])
        ph[:] = 0
    else:
        c = np.array([complex(a, -0.0 if i % 3 else 0.0) for i, a in enumerate(v)])
    check_csr(oracle, n, x, z, ph, c)


@pytest.mark.parametrize("kind", ["complex", "real", "imag"])
def test_fold_group_prefix_and_tail(cuda, oracle, kind):
    """A fold group of z-span rank 14: its first terms (rank <= 10) come from
    a per-class prefix table, the later ones are added per row; both parts
    must reproduce the term-order fold bit for bit."""
    rng = np.random.default_rng(11)
    n, T = 14, 48
    x = np.zeros(T, np.uint64)
    z = rng.integers(1, 1 << n, T).astype(np.uint64)
    ph = rng.integers(0, 4, T).astype(np.uint8)
    v = rng.normal(size=T)
    c = {"complex": v + 1j * rng.normal(size=T), "real": v + 0j, "imag": 1j * v}[kind]
    # a second group (x = 1) keeps the fill kernel's class-table path in play
    x = np.concatenate([x, np.ones(4, np.uint64)])
    z = np.concatenate([z, np.array([0, 1, 2, 3], np.uint64)])
    ph = np.concatenate([ph, np.zeros(4, np.uint8)])
    c = np.concatenate([c, np.ones(4)])
    check_csr(oracle, n, x, z, ph, c)


def test_more_than_256_groups(cuda, oracle):
    """G > 256: the direct-store fill and the in-place fold of the x = 0
    group (z span of rank 11, so a prefix table and a per-row tail)."""
    rng = np.random.default_rng(21)
    n = 11
    x = rng.integers(1, 1 << n, 700).astype(np.uint64)
    z = rng.integers(0, 1 << n, 700).astype(np.uint64)
    x = np.concatenate([x, np.zeros(30, np.uint64)])
    z = np.concatenate([z, rng.integers(1, 1 << n, 30).astype(np.uint64)])
    T = len(x)
    ph = rng.integers(0, 4, T).astype(np.uint8)
    c = rng.normal(size=T) + 1j * rng.normal(size=T)
    assert len(np.unique(x)) > 256
    check_csr(oracle, n, x, z, ph, c)


def test_many_fold_groups(cuda, oracle):
    """Forty fold-mode groups (16 terms each, z span up to rank 14): more
    fold entries per stage than threads, so they are placed by the strided
    loop; each group has a prefix table and a per-row tail."""
    rng = np.random.default_rng(22)
    n, ng, per = 14, 40, 16
    xs = rng.choice(np.arange(1, 1 << n), ng, replace=False).astype(np.uint64)
    x = np.repeat(xs, per)
    z = rng.integers(1, 1 << n, ng * per).astype(np.uint64)
    T = len(x)
    ph = rng.integers(0, 4, T).astype(np.uint8)
    c = rng.normal(size=T) + 0j  # real: the zero-imaginary rule too
    check_csr(oracle, n, x, z, ph, c)


@pytest.mark.parametrize("name", ["H2", "H4"])
def test_reference_test_H(cuda, golden, name):
    """pyqrusty/tests/test_H.py:32-48 on the GPU build: kron path
    (to_matrix) == RowwiseUnsafeChunked/100, dense, exactly."""
    labels, coeffs = golden[name]
    H = SparsePauliOp([Pauli(l) for l in labels], list(coeffs))
    m1 = csr_matrix(H.to_matrix()).todense()
    assert np.array_equal(m1, csr_matrix(H.to_matrix_mode(mode="")).todense())
    m2 = csr_matrix(H.to_matrix_mode(mode="RowwiseUnsafeChunked/100")).todense()
    assert np.array_equal(m1, m2)
    assert np.array_equal(m1, kron_dense(labels, coeffs))


def test_reference_test_H6_and_shape(cuda, golden):
    labels, coeffs = golden["H6"]
    H = SparsePauliOp([Pauli(l) for l in labels], list(coeffs))
    m = H.to_matrix()
    assert m.shape() == (1 << 12, 1 << 12)
    m1 = csr_matrix(m).todense()
    m2 = csr_matrix(H.to_matrix_mode(mode="RowwiseUnsafeChunked/100")).todense()
    assert np.array_equal(m1, m2)


@pytest.mark.parametrize("label,mat", [
    ("I", [[1, 0], [0, 1]]), ("X", [[0, 1], [1, 0]]), ("Z", [[1, 0], [0, -1]]),
    ("Y", [[0, -1j], [1j, 0]])])
def test_reference_pauli_matrices(cuda, label, mat):  # test_it.py:60-83
    spmat = csr_matrix(Pauli(label).to_matrix())
    assert np.array_equal(np.array(mat, dtype=complex), spmat.todense())


def test_i_plus_2x_all_modes(cuda):  # qrusty/src/lib.rs:775-813
    spop = SparsePauliOp([Pauli("I"), Pauli("X")], [1.0, 2.0])
    want = np.array([[1, 2], [2, 1]], dtype=complex)
    for mode in ["", "Binary", "Accel", "Rowwise", "RowwiseUnsafe", "RowwiseUnsafeChunked/500",
                 "Reduce", "Rayon", "RayonChunked/1"]:
        assert np.array_equal(csr_matrix(spop.to_matrix_mode(mode)).todense(), want)
    # the named builders of pyqrusty's SparsePauliOp (pyqrusty/src/lib.rs:382-404)
    for m in (spop.to_matrix(), spop.to_matrix_binary(), spop.to_matrix_accel(),
              spop.to_matrix_reduce(), spop.to_matrix_rayon(), spop.to_matrix_rayon_chunked(1)):
        assert np.array_equal(csr_matrix(m).todense(), want)


def test_export_moves(cuda):  # pyqrusty/src/lib.rs:190-214
    m = Pauli("XY").to_matrix()
    assert m.nnz() == 4
    assert repr(m).startswith("<4x4 sparse matrix of type Complex64")
    shape, data, indices, indptr = m.export()
    assert shape == (4, 4) and data.dtype == np.complex128 and indices.dtype == np.uint64
    with pytest.raises(Exception, match="already-exported"):
        m.export()
    assert repr(m) == "<already-dropped sparse matrix of type Complex64>"


def test_device_build_matches_host(cuda):
    import torch
    t, _ = W.cfg0(with_state=False)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    hi, hj, hd = op.csr_host()
    di, dj, dd = op.csr_device()
    torch.cuda.synchronize()
    assert np.array_equal(di.cpu().numpy().view(np.uint64), hi)
    assert np.array_equal(dj.cpu().numpy().view(np.uint64), hj)
    assert np.array_equal(_bits(dd.cpu().numpy()), _bits(hd))


def test_host_build_in_chunks_matches_device(cuda):
    """Chain n = 21 (2.1 GB of CSR): the host-memory build runs in two
    ~1 GiB row chunks (each with its own fold-value buffer and row offset)
    and must equal the one-shot device build bit for bit."""
    import torch
    t, _ = W.cfg1(with_state=False, n=21)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    nr, nz = op.csr_size()
    assert nz * 24 > 2 ** 30  # more than one chunk
    hi, hj, hd = op.csr_host()
    di, dj, dd = op.csr_device()
    torch.cuda.synchronize()
    assert np.array_equal(di.cpu().numpy().view(np.uint64), hi)
    step = 1 << 24
    for lo in range(0, nz, step):
        assert np.array_equal(dj[lo:lo + step].cpu().numpy().view(np.uint64), hj[lo:lo + step])
        assert np.array_equal(_bits(dd[lo:lo + step].cpu().numpy()), _bits(hd[lo:lo + step]))


def test_spmv_skips_out_of_range_columns(cuda):
    """qr_csr_spmv skips entries whose column is >= ncols (even when their
    value is not finite), for rows shorter and longer than the unrolled step."""
    import scipy.sparse as sps
    import torch
    from qrusty_gb300 import _lib
    rng = np.random.default_rng(2)
    nrows, ncols = 37, 50
    lens = rng.integers(0, 90, nrows)
    indptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    nnz = int(indptr[-1])
    indices = rng.integers(0, ncols + 20, nnz).astype(np.int64)
    data = rng.standard_normal(nnz) + 1j * rng.standard_normal(nnz)
    data[indices >= ncols] = np.inf
    v = rng.standard_normal(ncols) + 1j * rng.standard_normal(ncols)
    keep = indices < ncols
    A = sps.csr_matrix((np.where(keep, data, 0), np.where(keep, indices, 0), indptr),
                       shape=(nrows, ncols))
    want = A @ v
    d = lambda a: torch.from_numpy(a).to(cuda)
    ip, ij, dd, vd = d(indptr), d(indices), d(data), d(v)
    y = torch.empty(nrows, dtype=torch.complex128, device=cuda)
    _lib.check(_lib.load().qr_csr_spmv(nrows, ncols, ip.data_ptr(), ij.data_ptr(), dd.data_ptr(),
                                       vd.data_ptr(), y.data_ptr(), None))
    got = y.cpu().numpy()
    assert np.all(np.isfinite(got))
    assert np.allclose(got, want, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("first_len", [0, 1, 7, 44, 64, 65, 300])
def test_spmv_ragged_rows(cuda, first_len):
    """The step depth of qr_csr_spmv follows the first row's length; every
    other row length (empty, shorter, longer, many steps) must come out the
    same as scipy's product, with several rows per warp in flight."""
    import scipy.sparse as sps
    import torch
    from qrusty_gb300 import _lib
    rng = np.random.default_rng(first_len + 11)
    nrows, ncols = 1000, 700
    lens = rng.integers(0, 200, nrows)
    lens[rng.random(nrows) < 0.1] = 0
    lens[0] = first_len
    indptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    nnz = int(indptr[-1])
    indices = rng.integers(0, ncols, nnz).astype(np.int64)
    data = rng.standard_normal(nnz) + 1j * rng.standard_normal(nnz)
    v = rng.standard_normal(ncols) + 1j * rng.standard_normal(ncols)
    want = sps.csr_matrix((data, indices, indptr), shape=(nrows, ncols)) @ v
    d = lambda a: torch.from_numpy(a).to(cuda)
    ip, ij, dd, vd = d(indptr), d(indices), d(data), d(v)
    y = torch.empty(nrows, dtype=torch.complex128, device=cuda)
    _lib.check(_lib.load().qr_csr_spmv(nrows, ncols, ip.data_ptr(), ij.data_ptr(), dd.data_ptr(),
                                       vd.data_ptr(), y.data_ptr(), None))
    got = y.cpu().numpy()
    assert np.abs(got - want).max() <= 1e-12 * max(1.0, np.abs(want).max())


def test_chain22_sampled_rows_vs_make_row(cuda, oracle):
    """The chain at its benchmark size, n = 22 (G = 44, 1.85e8 stored
    entries, built on the device by the staged bulk-store kernel with the
    fold-value buffer for the x = 0 group of 21 ZZ bonds): about 200 rows
    spread over every region of the matrix against make_row
    (qrusty/src/accel.rs:171-210) restated by the oracle, bit for bit."""
    import torch
    t, _ = W.cfg1(with_state=False, n=22)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    nr, nz = op.csr_size()
    G = nz // nr
    assert G == 44
    ip, ij, dd = op.csr_device()
    torch.cuda.synchronize()
    op.sync_check()
    rng = np.random.default_rng(22)
    rows = np.unique(np.concatenate([
        [0, 1, 15, 16, 255, 256, nr // 2, nr - 2, nr - 1],
        rng.integers(0, nr, 190)])).astype(np.int64)
    r_dev = torch.from_numpy(rows).to(cuda)
    assert torch.equal(ip[r_dev], r_dev * G)
    assert int(ip[-1]) == nz
    pos = (r_dev[:, None] * G + torch.arange(G, device=cuda)[None, :]).reshape(-1)
    cols = ij[pos].cpu().numpy().view(np.uint64).reshape(len(rows), G)
    vals = dd[pos].cpu().numpy().reshape(len(rows), G)
    cp = oracle.make_params(t.phase, t.coeff)
    for k, r in enumerate(rows.tolist()):
        oc, ov = oracle.make_row(t.x, t.z, cp, r)
        assert np.array_equal(cols[k], oc), r
        assert np.array_equal(_bits(vals[k]), _bits(ov)), r
