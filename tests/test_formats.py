"""On-disk CSR formats through the C ABI (host-memory paths; no GPU needed).

rawio: files written by qr_rawio_write are byte-identical to the oracle's
restatement of qrusty/src/rawio.rs:128-149, and qr_rawio_read reads both byte
orders.  MatrixMarket: the reference's own round trips through scipy
(pyqrusty/tests/test_it.py:84-101, 146-215), gzip included, plus the value
text (shortest round-trip decimal, no exponent, as Rust's f64 Display)."""
import copy
import ctypes as C
import gzip

import numpy as np
import pytest
import scipy.sparse as sps
from scipy.io import mmread, mmwrite

from qrusty_gb300 import SpMat, csr_matrix
from qrusty_gb300 import _lib
from tests.helpers import terms_of_labels

I2 = np.eye(2, dtype=complex)
Y2 = np.array([[0, -1j], [1j, 0]])


def spmat_of_dense(d):
    s = sps.csr_matrix(d)
    return SpMat.new_unchecked(d.shape, s.data.astype(np.complex128), s.indices, s.indptr)


def oracle_spmat(oracle, golden, name):
    labels, coeffs = golden[name]
    n, x, z, ph, c = terms_of_labels(labels, coeffs)
    ip, ij, d = oracle.csr_build(n, x, z, oracle.make_params(ph, c), nthreads=4)
    return SpMat.new_unchecked((1 << n, 1 << n), d, ij, ip), (ip, ij, d, n)


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


# ---------------------------------------------------------------- rawio
@pytest.mark.parametrize("name", ["H2", "H4"])
def test_rawio_bytes_match_oracle(tmp_path, oracle, golden, name):
    m, (ip, ij, d, n) = oracle_spmat(oracle, golden, name)
    path = tmp_path / ("%s.raw" % name)
    m.rawio_write(str(path))
    assert path.read_bytes() == oracle.rawio_bytes(0, 1 << n, 1 << n, ip, ij, d)
    back = SpMat.rawio_read(str(path))
    shape, d2, ij2, ip2 = back.export()
    assert shape == (1 << n, 1 << n)
    assert np.array_equal(ip2, ip) and np.array_equal(ij2, ij)
    assert d2.tobytes() == d.tobytes()


def test_rawio_reads_other_byte_order(tmp_path, oracle):
    ip = np.array([0, 2, 3], dtype=np.uint64)
    ij = np.array([0, 1, 1], dtype=np.uint64)
    d = np.array([1 + 2j, -0.0 + 3.5j, 1e-300 - 7j])
    path = tmp_path / "be.raw"
    path.write_bytes(oracle.rawio_bytes(0, 2, 2, ip, ij, d, byteorder=">"))
    info = _lib.CsrFileInfo()
    _lib.check(_lib.load().qr_rawio_info(str(path).encode(), C.byref(info)))
    assert (info.nrows, info.ncols, info.indptr_len, info.nnz, info.byte_swapped) == (2, 2, 3, 3, 1)
    shape, d2, ij2, ip2 = SpMat.rawio_read(str(path)).export()
    assert np.array_equal(ip2, ip) and np.array_equal(ij2, ij) and d2.tobytes() == d.tobytes()


def test_rawio_gzip_and_errors(tmp_path, oracle, golden, lib):
    m, (ip, ij, d, n) = oracle_spmat(oracle, golden, "H2")
    gz = tmp_path / "h2.raw.gz"
    m.rawio_write(str(gz))
    assert gzip.decompress(gz.read_bytes()) == oracle.rawio_bytes(0, 1 << n, 1 << n, ip, ij, d)
    assert csr_matrix(SpMat.rawio_read(str(gz))).toarray().tobytes() == \
        csr_matrix(copy.copy(m)).toarray().tobytes()
    bad = tmp_path / "bad.raw"
    bad.write_bytes(oracle.rawio_bytes(7, 1, 1, [0, 0], [], []))
    info = _lib.CsrFileInfo()
    assert lib.qr_rawio_info(str(bad).encode(), C.byref(info)) == _lib.QR_EINVAL
    assert "bad storage" in _lib.last_error()
    short = tmp_path / "short.raw"
    short.write_bytes(oracle.rawio_bytes(0, 2, 2, ip[:3], [0, 1], [1j, 2j])[:-5])
    with pytest.raises(_lib.QrError, match="end of file"):
        SpMat.rawio_read(str(short))
    with pytest.raises(_lib.QrError):
        SpMat.rawio_read(str(tmp_path / "missing.raw"))


# ---------------------------------------------------------------- MatrixMarket
def test_i_plus_2y_written_reads_in_scipy(tmp_path):
    """test_it.py:84-101: (I + 2Y).matrixmarket_write, then scipy mmread."""
    m = spmat_of_dense(I2 + 2.0 * Y2)
    target = tmp_path / "I_plus_Y.mtx"
    m.matrixmarket_write(str(target))
    assert np.array_equal(I2 + 2.0 * Y2, mmread(str(target)).todense())
    text = target.read_text().splitlines()
    assert text[0] == "%%MatrixMarket matrix coordinate complex general"
    assert text[1] == "2 2 4"
    assert text[2:] == ["1 1 1 0", "1 2 0 -2", "2 1 0 2", "2 2 1 0"]


@pytest.mark.parametrize("gz", [False, True])
def test_write_roundtrip_fixture(tmp_path, oracle, golden, gz):
    """write_roundtrip / write_roundtrip_gzip (test_it.py:146-163) on H4."""
    m, _ = oracle_spmat(oracle, golden, "H4")
    path = tmp_path / ("H4.mtx.gz" if gz else "H4.mtx")
    m.matrixmarket_write(str(path))
    if gz:
        plain = tmp_path / "H4.mtx"
        plain.write_bytes(gzip.decompress(path.read_bytes()))
        path = plain
    ref = csr_matrix(copy.copy(m)).toarray()
    assert np.array_equal(ref, mmread(str(path)).toarray())
    back = SpMat.matrixmarket_read(str(path))
    assert csr_matrix(back).toarray().tobytes() == ref.tobytes()


@pytest.mark.parametrize("symmetry", [None, "symmetric", "hermitian", "skew-symmetric"])
@pytest.mark.parametrize("gz", [False, True])
def test_read_scipy_files(tmp_path, symmetry, gz):
    """write_roundtrip2 / write_roundtrip2_gzip (test_it.py:165-215): scipy
    writes (symmetric storage included), SpMat.matrixmarket_read reads."""
    rng = np.random.default_rng(3)
    a = rng.standard_normal((7, 7)) + 1j * rng.standard_normal((7, 7))
    a[rng.random((7, 7)) < 0.5] = 0
    if symmetry == "symmetric":
        a = a + a.T
    elif symmetry == "hermitian":
        a = a + a.conj().T
    elif symmetry == "skew-symmetric":
        a = a - a.T
    sp = sps.csr_matrix(a)
    path = tmp_path / "m.mtx"
    mmwrite(str(path), sp, symmetry=symmetry)
    if gz:
        gzpath = tmp_path / "m.mtx.gz"
        gzpath.write_bytes(gzip.compress(path.read_bytes()))
        path = gzpath
    m = SpMat.matrixmarket_read(str(path))
    assert np.array_equal(csr_matrix(m).toarray(), a)


def test_read_real_pattern_and_duplicates(tmp_path):
    p = tmp_path / "r.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n% comment\n3 4 4\n"
                 "1 2 1.5\n3 4 -2\n1 2 0.25\n2 1 1e3\n")
    shape, d, ij, ip = SpMat.matrixmarket_read(str(p)).export()
    assert shape == (3, 4)
    assert list(ip) == [0, 1, 2, 3] and list(ij) == [1, 0, 3]
    assert list(d) == [1.75, 1000.0, -2.0]
    q = tmp_path / "p.mtx"
    q.write_text("%%MatrixMarket matrix coordinate pattern symmetric\n2 2 2\n1 1\n2 1\n")
    assert np.array_equal(csr_matrix(SpMat.matrixmarket_read(str(q))).toarray(),
                          np.array([[1, 1], [1, 0]], dtype=complex))
    bad = tmp_path / "bad.mtx"
    bad.write_text("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n")
    with pytest.raises(Exception, match="matrixmarket_read"):
        SpMat.matrixmarket_read(str(bad))


def test_value_text_is_shortest_round_trip(tmp_path):
    vals = np.array([0.1 + 0.2j, 1e-7 - 3e21j, -0.0 + 1 / 3j, 123456.789 + 2.5e-300j])
    m = SpMat.new_unchecked((1, 4), vals, np.arange(4, dtype=np.uint64),
                            np.array([0, 4], dtype=np.uint64))
    p = tmp_path / "v.mtx"
    m.matrixmarket_write(str(p))
    lines = p.read_text().splitlines()[2:]
    for k, line in enumerate(lines):
        i, j, re, im = line.split()
        assert (int(i), int(j)) == (1, k + 1)
        for txt, v in ((re, vals[k].real), (im, vals[k].imag)):
            assert txt == np.format_float_positional(v, unique=True, trim="-")
            assert float(txt) == v and "e" not in txt


def test_write_symmetric_modes(tmp_path):
    a = np.array([[2, 1 - 1j, 0], [1 + 1j, 3, 4j], [0, -4j, 5]])
    m = spmat_of_dense(a)
    p = tmp_path / "h.mtx"
    m.matrixmarket_write_symmetric(str(p), "hermitian")
    lines = p.read_text().splitlines()
    assert lines[0] == "%%MatrixMarket matrix coordinate complex hermitian"
    assert lines[1] == "3 3 5"
    assert np.array_equal(mmread(str(p)).toarray(), a)
    assert np.array_equal(csr_matrix(SpMat.matrixmarket_read(str(p))).toarray(), a)
    with pytest.raises(Exception, match="unrecognized mode"):
        m.matrixmarket_write_symmetric(str(p), "bogus")
    m.export()
    with pytest.raises(Exception, match="already-destroyed"):
        m.matrixmarket_write(str(p))
