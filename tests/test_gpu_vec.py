"""Eigensolver-loop vector helpers on the GPU: axpby / axpy / ax, precond /
precond2, SpMat.diagonal and the operator diagonal.

complex128 results are compared with the CPU oracle BIT FOR BIT (both follow
num-complex's operation sequence with no FMA contraction); complex64 results
bit for bit against the oracle's float restatement.  The single tolerance is
hypot's: a pivot |diag - e| within 2 ulp of tol may be regularised on one
side only; the inputs here keep every pivot far from tol."""
import ctypes as C
import os

import numpy as np
import pytest

from qrusty_gb300 import (PauliOperator, SparsePauliOp, SpMat, Pauli, ax, axpby, axpy, precond,
                          precond2)
from qrusty_gb300 import _lib
from qrusty_gb300 import workloads as W

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def same_bits(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.dtype == b.dtype and a.shape == b.shape and a.tobytes() == b.tobytes()


def rand_c(rng, n, dtype=np.complex128):
    return (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(dtype)


def test_reference_known_answers(cuda):
    """pyqrusty/tests/test_it.py:232-276 through the pyqrusty-style API."""
    x = np.array([1.0 + 2j, 2.0 + 3j, 3.0 + 4j, 4.0 + 5j])
    y = np.ones(4, dtype=complex)
    a, b = 0.0 + 1.0j, 1.0 + 0.0j
    assert np.allclose(axpby(a, x, b, y), a * x + b * y)
    assert np.allclose(axpy(a, x, y), a * x + y)
    assert np.allclose(ax(a, x), a * x)
    rows = 1 << 20
    rng = np.random.default_rng(0)
    xs = rng.random(rows) + rng.random(rows) * 1j
    ys = rng.random(rows) + rng.random(rows) * 1j
    assert np.allclose(axpby(a, xs, b, ys), a * xs + b * ys)
    assert np.allclose(axpy(a, xs, ys), a * xs + ys)
    assert np.allclose(ax(a, xs), a * xs)


@pytest.mark.parametrize("n", [1, 2, 3, 1000, 4097, 1 << 20])
@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_bit_exact_vs_oracle(cuda, oracle, n, dtype):
    rng = np.random.default_rng(n)
    x, y = rand_c(rng, n, dtype), rand_c(rng, n, dtype)
    a, b = 0.7 - 1.3j, -0.25 + 2.0j
    import torch
    xd, yd = torch.from_numpy(x).to(cuda), torch.from_numpy(y).to(cuda)
    assert same_bits(axpby(a, xd, b, yd).cpu().numpy(), oracle.vec("axpby", x, y, a, b))
    assert same_bits(axpy(a, xd, yd).cpu().numpy(), oracle.vec("axpy", x, y, a))
    assert same_bits(ax(a, xd).cpu().numpy(), oracle.vec("ax", x, None, a))
    d = rand_c(rng, n, dtype)
    e = 0.1 + 0.05j
    assert same_bits(precond2(torch.from_numpy(d).to(cuda), yd, e, 1e-3).cpu().numpy(),
                     oracle.vec("precond2", d, y, e, tol=1e-3))


def test_complex64_unaligned_and_aliased(cuda, oracle):
    """Odd offsets (8-byte aligned views) take the scalar path; z may be
    the same buffer as x (C ABI)."""
    import torch
    rng = np.random.default_rng(5)
    x, y = rand_c(rng, 1001, np.complex64), rand_c(rng, 1001, np.complex64)
    xd, yd = torch.from_numpy(x).to(cuda), torch.from_numpy(y).to(cuda)
    a = 1.5 - 0.5j
    got = axpy(a, xd[1:], yd[1:]).cpu().numpy()
    assert same_bits(got, oracle.vec("axpy", x[1:], y[1:], a))
    z = xd.clone()
    av = (C.c_double * 2)(a.real, a.imag)
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(_lib.load().qr_axpy(_lib.QR_C64C, z.numel(), av, z.data_ptr(), yd.data_ptr(),
                                   z.data_ptr(), st))
    assert same_bits(z.cpu().numpy(), oracle.vec("axpy", x, y, a))
    # zero length is a no-op
    _lib.check(_lib.load().qr_ax(_lib.QR_C128, 0, av, None, None, st))


def test_precond_reference_golden(cuda, oracle, golden):
    """pyqrusty/tests/test_it.py:303-313: precond(H2 matrix, dx, e, tol) and
    precond2(H2.diagonal(), ...) against the reference's printed rv."""
    g = np.load(os.path.join(GOLDEN, "precond.npz"))
    labels, coeffs = golden["H2"]
    H2 = SparsePauliOp([Pauli(s) for s in labels], coeffs)
    m = H2.to_matrix()
    tol, dx, e, rv = float(g["tol"]), g["dx"], complex(g["e"]), g["rv"]
    r1 = precond(m, dx, e, tol)
    r2 = precond2(m.diagonal(), dx, e, tol)
    assert np.allclose(r1, rv, rtol=1e-8, atol=1e-300)
    assert same_bits(r1, r2)
    assert same_bits(r1, oracle.vec("precond2", m.diagonal(), dx, e, tol=tol))


def test_spmat_diagonal_reference_cases(cuda):
    """pyqrusty/tests/test_it.py:46-58 (square and 3x2)."""
    import scipy.sparse as sps
    d = np.array([[1.0, 2.0], [3.0, 4.0]], dtype=complex)
    s = sps.csr_matrix(d)
    m = SpMat.new_unchecked(d.shape, s.data, s.indices, s.indptr)
    assert np.array_equal(m.diagonal(), np.diagonal(d))
    d3 = np.array([[1.0, 2.0], [3.0, 4.0], [5.0, 6.0]], dtype=complex)
    s3 = sps.csr_matrix(d3)
    m3 = SpMat.new_unchecked(d3.shape, s3.data, s3.indices, s3.indptr)
    assert np.array_equal(m3.diagonal(), np.diagonal(d3))
    # a row without a stored diagonal entry reads 0
    dz = np.array([[0.0, 2.0], [3.0, 4.0]], dtype=complex)
    sz = sps.csr_matrix(dz)
    mz = SpMat.new_unchecked(dz.shape, sz.data, sz.indices, sz.indptr)
    assert np.array_equal(mz.diagonal(), np.diagonal(dz))
    m.export()
    with pytest.raises(Exception, match="already-exported"):
        m.diagonal()
    with pytest.raises(Exception, match="exported sparse matrix"):
        precond(m, np.ones(2), 0.0, 1e-14)


@pytest.mark.parametrize("which", ["cfg0", "jw14", "chain12", "nodiag"])
def test_operator_diagonal(cuda, oracle, which):
    """qr_op_diagonal == the CSR's diagonal bit for bit (complex128), and
    its complex64 form is that value rounded."""
    import torch
    rng = np.random.default_rng(3)
    if which == "cfg0":
        t = W.cfg0()[0]
    elif which == "jw14":
        t = W.cfg2(n=14)
    elif which == "chain12":
        t = W.cfg1(with_state=False, n=12)[0]
    else:
        t = W.random_letters_op(rng, 10, 40)
        keep = t.x != 0
        t = W.Terms(t.n, t.x[keep], t.z[keep], t.phase[keep], t.coeff[keep])
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    d128 = op.diagonal().cpu().numpy()
    cp = oracle.make_params(t.phase, t.coeff)
    want = oracle.op_diagonal(t.x, t.z, cp, 0, 1 << t.n)
    assert same_bits(d128, want)
    ip, ij, dd = op.csr_device()
    m = SpMat.new_unchecked((1 << t.n, 1 << t.n), dd.cpu().numpy(), ij.cpu().numpy(),
                            ip.cpu().numpy())
    assert same_bits(m.diagonal(), want)
    d64 = op.diagonal(dtype=torch.complex64).cpu().numpy()
    assert same_bits(d64, want.astype(np.complex64))
    if which == "nodiag":
        assert not np.any(d128)


def test_argument_errors(cuda):
    with pytest.raises(Exception, match="different lengths"):
        axpy(1.0, np.ones(3), np.ones(4))
    av = (C.c_double * 2)(1.0, 0.0)
    rc = _lib.load().qr_ax(7, 4, av, None, None, None)
    assert rc == _lib.QR_EINVAL


@pytest.mark.parametrize("which", ["jw14", "chain12"])
@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_fused_apply_axpby(cuda, which, dtype):
    """alpha (H psi) + beta v fused into the apply kernel equals apply then
    axpby bit for bit; v may be the output buffer (the residual update)."""
    import torch
    t = W.cfg2(n=14) if which == "jw14" else W.cfg1(with_state=False, n=12)[0]
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    tdt = torch.complex128 if dtype == "c128" else torch.complex64
    g = torch.Generator(device=cuda).manual_seed(5)
    N = 1 << t.n
    psi = torch.randn(2 * N, dtype=tdt, device=cuda, generator=g)
    v = torch.randn(2 * N, dtype=tdt, device=cuda, generator=g)
    a, b = 1.0 - 0.25j, -0.8125 + 0.5j
    want = axpby(a, op.apply(psi), b, v)
    got = op.apply_axpby(psi, v, a, b)
    assert torch.equal(torch.view_as_real(got), torch.view_as_real(want))
    inplace = v.clone()
    op.apply_axpby(psi, inplace, a, b, out=inplace)
    assert torch.equal(torch.view_as_real(inplace), torch.view_as_real(want))
    # v = psi: the eigensolver residual H psi - theta psi
    want2 = axpby(a, op.apply(psi), b, psi)
    got2 = op.apply_axpby(psi, psi, a, b)
    assert torch.equal(torch.view_as_real(got2), torch.view_as_real(want2))
    buf = torch.zeros(2 * N + 2, dtype=tdt, device=cuda)
    with pytest.raises(_lib.QrError, match="v overlaps y"):
        op.apply_axpby(psi, buf[2:], a, b, out=buf[:-2])
