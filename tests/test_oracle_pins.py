"""Pin the CPU oracle (oracle/qrusty_oracle.c) to the reference's own tests.

The Rust reference cannot be compiled here, so the restatement is pinned by
re-running the reference's known-answer tests against it:
  * label-parse goldens          qrusty/src/lib.rs:608-693
  * 2x2 Pauli matrices, kron      qrusty/src/lib.rs:696-719, pyqrusty/tests/test_it.py:60-83
  * IX, XI, I, Y, YY rowwise==kron qrusty/src/lib.rs:722-768
  * I + 2X = [[1,2],[2,1]]        qrusty/src/lib.rs:775-813
  * H2/H4/H6 rowwise == kron, EXACT dense equality
                                  pyqrusty/tests/test_H.py:32-48 (fixtures from
                                  pyqrusty/tests/H_fixtures.py, tests/golden/)
  * CSR SpMV vs a second SpMV     qrusty/src/lib.rs:888-919, test_it.py:218-230
  * axpby / axpy / ax known answers pyqrusty/tests/test_it.py:232-276
  * precond / precond2 on H2       pyqrusty/tests/test_it.py:278-313 (the
                                  reference's printed rv, tests/golden/precond.npz)
plus structural invariants of make_row's output (accel.rs:171-210), and
sampled rows of the larger fixtures H8 / HJ against a pure-Python
restatement of make_params / make_row (tests/helpers.py), bit for bit.
"""
import os

import numpy as np
import pytest
import scipy.sparse as sps

from tests.helpers import (csr_to_dense, kron_dense, make_params_py, make_row_py,
                           rowwise_dense, terms_of_labels)

I2 = np.array([[1, 0], [0, 1]], dtype=complex)
X2 = np.array([[0, 1], [1, 0]], dtype=complex)
Y2 = np.array([[0, -1j], [1j, 0]], dtype=complex)
Z2 = np.array([[1, 0], [0, -1]], dtype=complex)


def oracle_csr(O, labels, coeffs, step=500):
    n, x, z, ph, c = terms_of_labels(labels, coeffs)
    cp = O.make_params(ph, c)
    return n, O.csr_build(n, x, z, cp, step=step, nthreads=4)


def oracle_dense(O, labels, coeffs):
    n, (indptr, indices, data) = oracle_csr(O, labels, coeffs)
    return csr_to_dense(indptr, indices, data, (1 << n, 1 << n))


@pytest.mark.parametrize("bad", ["W", "", "+i"])
def test_parse_rejects(oracle, bad):
    with pytest.raises(ValueError):
        oracle.parse_label(bad)


@pytest.mark.parametrize("label,bp,letters", [
    ("I", 0, "I"), ("+I", 0, "I"), ("+iI", 1, "I"), ("+jI", 1, "I"), ("-1jI", 3, "I"),
    ("-1I", 2, "I"), ("-1jIX", 3, "XI"), ("IXYZ", 0, "ZYXI"),
])
def test_parse_goldens(oracle, label, bp, letters):
    assert oracle.parse_label(label) == (bp, letters)


def test_mask_goldens(oracle):
    # single letters (z, x): I (F,F), X (F,T), Y (T,T), Z (T,F)
    assert oracle.label_masks("I")[:2] == (0, 0)
    assert oracle.label_masks("X")[:2] == (1, 0)
    assert oracle.label_masks("Y")[:2] == (1, 1)
    assert oracle.label_masks("Z")[:2] == (0, 1)
    x, z, _ = oracle.label_masks("IXYZ")
    assert [(x >> q) & 1 for q in range(4)] == [0, 1, 1, 0]
    assert [(z >> q) & 1 for q in range(4)] == [1, 1, 0, 0]
    x, z, ph = oracle.label_masks("-IIIIIIIIIIIIIIIIIIYXXY")
    assert oracle.parse_label("-IIIIIIIIIIIIIIIIIIYXXY")[0] == 2
    assert ph == 0
    assert [(z >> q) & 1 for q in range(22)] == [1, 0, 0, 1] + [0] * 18
    assert [(x >> q) & 1 for q in range(22)] == [1, 1, 1, 1] + [0] * 18


@pytest.mark.parametrize("label,mat", [("I", I2), ("X", X2), ("Y", Y2), ("Z", Z2),
                                       ("IX", np.kron(I2, X2)), ("XI", np.kron(X2, I2)),
                                       ("YY", np.kron(Y2, Y2))])
def test_single_paulis(oracle, label, mat):
    d = oracle_dense(oracle, [label], [1.0])
    assert np.array_equal(d, mat)
    assert np.array_equal(d, kron_dense([label], [1.0]))


def test_i_plus_2x(oracle):
    d = oracle_dense(oracle, ["I", "X"], [1.0, 2.0])
    assert np.array_equal(d, np.array([[1, 2], [2, 1]], dtype=complex))


def test_prefix_conventions(oracle):
    # rowwise multiplies by (-i)^(base+#Y); kron by i^base (-i)^#Y.  They agree
    # for even base, and conjugate the prefix factor for i / -i.
    for lab in ["Y", "XY", "IXYZ", "-YY", "iX", "-iY", "jZX", "-1jXY"]:
        d = oracle_dense(oracle, [lab], [0.75 - 0.25j])
        assert np.array_equal(d, rowwise_dense([lab], [0.75 - 0.25j]))
        if oracle.parse_label(lab)[0] % 2 == 0:
            assert np.array_equal(d, kron_dense([lab], [0.75 - 0.25j]))


@pytest.mark.parametrize("name", ["H2", "H4", "H6"])
def test_fixture_rowwise_equals_kron_exactly(oracle, golden, name):
    labels, coeffs = golden[name]
    d = oracle_dense(oracle, labels, coeffs)
    k = kron_dense(labels, coeffs)
    assert np.array_equal(d, k)


@pytest.mark.parametrize("name", ["H2", "H4", "H6"])
def test_row_structure(oracle, golden, name):
    labels, coeffs = golden[name]
    n, (indptr, indices, data) = oracle_csr(oracle, labels, coeffs, step=100)
    _, x, _, _, _ = terms_of_labels(labels, coeffs)
    G = len(np.unique(x))
    N = 1 << n
    assert np.array_equal(indptr, np.arange(N + 1, dtype=np.uint64) * np.uint64(G))
    rows = indices.reshape(N, G)
    assert np.all(np.diff(rows.astype(np.int64), axis=1) > 0)  # sorted, unique
    # column set of row r is {r ^ x_g}
    ux = np.unique(x)
    for r in (0, 1, N // 3, N - 1):
        assert np.array_equal(np.sort(np.uint64(r) ^ ux), rows[r])


@pytest.mark.parametrize("name,ranges", [
    ("H8", [(0, 48), (40000, 40032), (65520, 65536)]),
    ("HJ", [(0, 32), (1 << 26, (1 << 26) + 32), ((1 << 27) - 32, 1 << 27)]),
])
def test_large_fixture_rows_bit_exact(oracle, golden, name, ranges):
    """H8 (16 qubits, 5,793 terms) and HJ (27 qubits) from H_fixtures.py are
    too large for a dense Kronecker check: sampled row ranges of the oracle's
    chunked build must equal, bit for bit (signed zeros included), a
    pure-Python restatement of make_params and make_row."""
    labels, coeffs = golden[name]
    n, x, z, ph, c = terms_of_labels(labels, coeffs)
    cp = oracle.make_params(ph, c)
    cpy = np.array(make_params_py(ph, c), dtype=np.complex128)
    assert np.array_equal(cp.view(np.uint64), cpy.view(np.uint64))
    xl, zl, cl = x.tolist(), z.tolist(), list(cpy)
    for lo, hi in ranges:
        ip, ij, d = oracle.csr_build(n, x, z, cp, step=16, nthreads=2, rows=(lo, hi))
        assert len(ip) == hi - lo + 1
        for k, r in enumerate(range(lo, hi)):
            cols, vals = make_row_py(xl, zl, cl, r)
            a, b = int(ip[k] - ip[0]), int(ip[k + 1] - ip[0])
            assert ij[a:b].tolist() == cols
            want = np.array(vals, dtype=np.complex128)
            assert np.array_equal(d[a:b].view(np.uint64), want.view(np.uint64))


def test_explicit_zeros_kept(oracle):
    # X and -X cancel: make_row keeps the explicit zero (accel.rs:191-209)
    n, (indptr, indices, data) = oracle_csr(oracle, ["IX", "IX", "ZI"], [1.0, -1.0, 0.5])
    assert len(data) == 4 * 2
    assert np.count_nonzero(data == 0) == 4


def test_chunking_invariant(oracle, golden):
    labels, coeffs = golden["H4"]
    a = oracle_csr(oracle, labels, coeffs, step=1)[1]
    b = oracle_csr(oracle, labels, coeffs, step=1000)[1]
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


@pytest.mark.parametrize("name", ["H2", "H6"])
def test_spmv_vs_scipy(oracle, golden, name):
    labels, coeffs = golden[name]
    n, (indptr, indices, data) = oracle_csr(oracle, labels, coeffs)
    rng = np.random.default_rng(7)
    v = rng.uniform(0, 10, 1 << n).astype(np.complex128)
    y = oracle.spmv(indptr, indices, data, v)
    A = sps.csr_matrix((data, indices.astype(np.int64), indptr.astype(np.int64)),
                       shape=(1 << n, 1 << n))
    assert np.allclose(y, A.dot(v), rtol=0, atol=1e-7)
    # matrix-free restatement is row-for-row identical to CSR + SpMV
    _, x, z, ph, c = terms_of_labels(labels, coeffs)
    y2 = oracle.apply(n, x, z, oracle.make_params(ph, c), v)
    assert np.array_equal(y, y2)


# ---------------------------------------------------------------- vector helpers
X4 = np.array([1.0 + 2j, 2.0 + 3j, 3.0 + 4j, 4.0 + 5j])


def test_vector_helper_known_answers(oracle):
    """test_it.py:232-276: a = i, b = 1 on the 4-element vector (exact in
    binary, so equality), and 2^20 random entries against numpy's formula."""
    y = np.ones(4, dtype=complex)
    assert np.array_equal(oracle.vec("axpby", X4, y, 1j, 1.0), 1j * X4 + 1.0 * y)
    assert np.array_equal(oracle.vec("axpy", X4, y, 1j), 1j * X4 + y)
    assert np.array_equal(oracle.vec("ax", X4, None, 1j), 1j * X4)
    rng = np.random.default_rng(11)
    xs = rng.random(1 << 20) + rng.random(1 << 20) * 1j
    ys = rng.random(1 << 20) + rng.random(1 << 20) * 1j
    a, b = 0.3 - 1.7j, -2.5 + 0.25j
    assert np.allclose(oracle.vec("axpby", xs, ys, a, b), a * xs + b * ys, rtol=0, atol=1e-14)
    assert np.allclose(oracle.vec("axpy", xs, ys, a), a * xs + ys, rtol=0, atol=1e-14)
    assert np.allclose(oracle.vec("ax", xs, None, a), a * xs, rtol=0, atol=1e-14)


def _h2_diagonal(oracle, golden):
    labels, coeffs = golden["H2"]
    n, (indptr, indices, data) = oracle_csr(oracle, labels, coeffs)
    d = np.zeros(1 << n, dtype=complex)
    for r in range(1 << n):
        lo, hi = int(indptr[r]), int(indptr[r + 1])
        hit = np.nonzero(indices[lo:hi] == r)[0]
        if len(hit):
            d[r] = data[lo + hit[0]]
    return d


def test_precond_golden(oracle, golden):
    """precond2(H2.diagonal(), dx, e, tol) against the result the reference
    printed in its test (9 significant digits) and against its numpy
    restatement dx / reg(diag - e, tol) (test_it.py:270-313)."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "precond.npz"))
    d = _h2_diagonal(oracle, golden)
    got = oracle.vec("precond2", d, g["dx"], complex(g["e"]), tol=float(g["tol"]))
    assert np.allclose(got, g["rv"], rtol=1e-8, atol=1e-300)
    v = d - complex(g["e"])
    v = np.where(np.abs(v) < float(g["tol"]), float(g["tol"]), v)
    assert np.allclose(got, g["dx"] / v, rtol=1e-15, atol=0)


def test_precond_regularises_small_pivots(oracle):
    diag = np.array([1.0 + 0j, 2.0 + 1e-20j, 3.0 + 0j])
    dx = np.array([1.0 + 1j, 1.0 + 1j, 1.0 + 1j])
    got = oracle.vec("precond2", diag, dx, 2.0, tol=1e-6)
    assert got[1] == (1.0 + 1j) / 1e-6
    assert got[0] == (1.0 + 1j) / (-1.0) and got[2] == (1.0 + 1j) / 1.0


def test_vector_helpers_complex64(oracle):
    """complex64: the same sequence in float; a, b rounded to float."""
    rng = np.random.default_rng(12)
    xs = (rng.random(1001) + rng.random(1001) * 1j).astype(np.complex64)
    ys = (rng.random(1001) + rng.random(1001) * 1j).astype(np.complex64)
    a = np.complex64(0.3 - 1.7j)
    got = oracle.vec("axpy", xs, ys, complex(a))
    assert got.dtype == np.complex64
    ar, ai = np.float32(a.real), np.float32(a.imag)
    want_re = (ar * xs.real - ai * xs.imag) + ys.real
    want_im = (ar * xs.imag + ai * xs.real) + ys.imag
    assert np.array_equal(got.real, want_re) and np.array_equal(got.imag, want_im)


@pytest.mark.parametrize("name", ["H2", "H4", "H6"])
def test_op_diagonal_is_csr_diagonal(oracle, golden, name):
    labels, coeffs = golden[name]
    n, x, z, ph, c = terms_of_labels(labels, coeffs)
    cp = oracle.make_params(ph, c)
    indptr, indices, data = oracle.csr_build(n, x, z, cp, nthreads=4)
    d = oracle.op_diagonal(x, z, cp, 0, 1 << n)
    for r in range(1 << n):
        lo, hi = int(indptr[r]), int(indptr[r + 1])
        hit = np.nonzero(indices[lo:hi] == r)[0]
        want = data[lo + hit[0]] if len(hit) else 0j
        assert d[r].tobytes() == np.complex128(want).tobytes()
