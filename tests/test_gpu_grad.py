"""FP64 reductions, per-term gradients, coefficient updates and the autograd
Function for y = H(c) psi (the differentiation workload: n = 20, 2,000
random-letter terms, complex64 psi).

Tolerances: c128 results <= 1e-12 relative to the FP64 oracle; c64c inner
products / gradients <= 1e-5 relative (complex64 inputs carry ~6e-8 relative
rounding each, accumulated over 2^20 amplitudes in FP64)."""
import numpy as np
import pytest

from qrusty_gb300 import PauliOperator, vdot
from qrusty_gb300 import workloads as W
from qrusty_gb300.autograd import PauliTerms, pauli_apply

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def test_vdot(cuda):
    import torch
    rng = np.random.default_rng(1)
    a = W.random_state(rng, 1 << 16, nstates=3)
    b = W.random_state(rng, 1 << 16, nstates=3)
    want = np.array([np.vdot(a[s], b[s]) for s in range(3)])
    got = vdot(torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda)).cpu().numpy()
    assert rel(got, want) <= 1e-12
    a64, b64 = a.astype(np.complex64), b.astype(np.complex64)
    want64 = np.array([np.vdot(a64[s].astype(np.complex128), b64[s].astype(np.complex128))
                       for s in range(3)])
    got64 = vdot(torch.from_numpy(a64).to(cuda), torch.from_numpy(b64).to(cuda)).cpu().numpy()
    assert rel(got64, want64) <= 1e-6


@pytest.mark.parametrize("which", ["cfg0", "chain14"])
def test_expect(cuda, oracle, which):
    import torch
    if which == "cfg0":
        t, psi = W.cfg0()
    else:
        t, psi = W.cfg1(n=14)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    hpsi = oracle.apply(t.n, t.x, t.z, oracle.make_params(t.phase, t.coeff), psi)
    want = np.vdot(psi, hpsi)
    p = torch.from_numpy(psi).to(cuda)
    e128 = op.expect(p).cpu().numpy()[0]
    e64 = op.expect(p.to(torch.complex64)).cpu().numpy()[0]
    assert abs(e128 - want) <= 1e-12 * max(1.0, abs(want))
    assert abs(e64 - want) <= 1e-5 * max(1.0, abs(want))
    # Hermitian operator (real coefficients): expectation is real
    assert abs(e128.imag) <= 1e-12


@pytest.mark.parametrize("n,T", [(8, 30), (12, 200), (14, 150)])
def test_term_grad_vs_oracle(cuda, oracle, n, T):
    import torch
    rng = np.random.default_rng(n)
    t = W.random_letters_op(rng, n, T)
    # duplicate a few strings so merged strings map back to several inputs
    x = np.concatenate([t.x, t.x[:5]])
    z = np.concatenate([t.z, t.z[:5]])
    ph = np.concatenate([t.phase, (t.phase[:5] + 2) % 4]).astype(np.uint8)
    c = np.concatenate([t.coeff, t.coeff[:5]])
    psi = W.random_state(rng, 1 << n)
    g = W.random_state(rng, 1 << n)
    op = PauliOperator(n, x, z, ph, c)
    want = oracle.term_grad(n, x, z, ph, psi, g)
    pt, gt = torch.from_numpy(psi).to(cuda), torch.from_numpy(g).to(cuda)
    got = op.term_grad(pt, gt).cpu().numpy()
    assert rel(got, want) <= 1e-12
    got64 = op.term_grad(pt.to(torch.complex64), gt.to(torch.complex64)).cpu().numpy()
    assert rel(got64, want) <= 1e-5


def _jw_like(rng, n, T):
    """Hopping-like strings X_i Z..Z X_j / Y_i Z..Z Y_j plus random letters:
    x masks with bits on every row position (partner rows permuted by bits
    0-8, 9-11 and the partner tile), z with bits 9-11 set and clear."""
    t = W.random_letters_op(rng, n, T // 2)
    xs, zs, ph = [t.x], [t.z], [t.phase]
    i = rng.integers(0, n - 1, T - T // 2)
    j = np.minimum(i + 1 + rng.integers(0, n - 1, len(i)), n - 1)
    x = (np.uint64(1) << i.astype(np.uint64)) | (np.uint64(1) << j.astype(np.uint64))
    between = ((np.uint64(1) << j.astype(np.uint64)) - np.uint64(1)) & ~(
        (np.uint64(2) << i.astype(np.uint64)) - np.uint64(1))
    xs.append(x)
    zs.append(between | np.where(rng.random(len(i)) < 0.5, x, np.uint64(0)))
    ph.append(rng.integers(0, 4, len(i)).astype(np.uint8))
    c = rng.standard_normal(T).astype(np.complex128)
    return (np.concatenate(xs), np.concatenate(zs), np.concatenate(ph), c)


@pytest.mark.parametrize("n,T,ns", [(12, 300, 1), (13, 500, 2), (16, 900, 3), (18, 2000, 1)])
def test_term_grad_tiles_c64(cuda, oracle, n, T, ns):
    """The tiled complex64 gradient kernel (n >= 12: strings batched by
    partner tile, staged tiles, sign butterfly, FP64 warp sums) against the
    oracle on the same complex64 values, summed over several states, and
    bit-identical when called again (fixed summation order)."""
    import torch
    rng = np.random.default_rng(200 + n)
    x, z, ph, c = _jw_like(rng, n, T)
    op = PauliOperator(n, x, z, ph, c)
    psi = W.random_state(rng, 1 << n, nstates=ns).astype(np.complex64).reshape(ns, -1)
    g = W.random_state(rng, 1 << n, nstates=ns).astype(np.complex64).reshape(ns, -1)
    want = sum(oracle.term_grad(n, x, z, ph, psi[s].astype(np.complex128),
                                g[s].astype(np.complex128)) for s in range(ns))
    pt = torch.from_numpy(psi.reshape(-1)).to(cuda)
    gt = torch.from_numpy(g.reshape(-1)).to(cuda)
    got = op.term_grad(pt, gt)
    again = op.term_grad(pt, gt)
    assert torch.equal(torch.view_as_real(got), torch.view_as_real(again))
    err = np.abs(got.cpu().numpy() - want).max() / np.abs(want).max()
    assert err <= 1e-6, err


def test_set_coeffs(cuda, oracle):
    import torch
    t, psi = W.cfg0()
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    p = torch.from_numpy(psi).to(cuda)
    op.apply(p)  # build plans with the old coefficients
    op.apply(p.to(torch.complex64))
    c2 = np.random.default_rng(3).standard_normal(t.T) * (1 + 0.5j)
    op.set_coeffs(c2)
    ref = oracle.apply(t.n, t.x, t.z, oracle.make_params(t.phase, c2), psi)
    assert rel(op.apply(p).cpu().numpy(), ref) <= 1e-12
    assert rel(op.apply(p.to(torch.complex64)).cpu().numpy(), ref) <= 1e-6
    # CSR tables follow the new coefficients too (bit-exact)
    ip, ij, d = op.csr_host()
    oi, oj, od = oracle.csr_build(t.n, t.x, t.z, oracle.make_params(t.phase, c2))
    assert np.array_equal(ij, oj) and np.array_equal(d.view(np.uint64), od.view(np.uint64))


def test_autograd_differentiation_workload(cuda, oracle):
    """n = 20, 2,000 terms, real c ~ N(0, 1); L = Re<y, w>; grad_c vs the FP64
    definition (all 2,000) and central finite differences (FP64 forward,
    step 1e-3, 16 sampled coefficients); grad_psi vs the c128 adjoint."""
    import torch
    t, psi, w = W.cfg4()
    terms = PauliTerms(t.n, t.x, t.z, t.phase)
    c = torch.tensor(t.coeff.real, dtype=torch.float64, requires_grad=True)
    p = torch.from_numpy(psi.astype(np.complex64)).to(cuda).requires_grad_(True)
    w64 = torch.from_numpy(w.astype(np.complex64)).to(cuda)
    y = pauli_apply(c, p, terms)
    L = torch.vdot(y, w64).real
    L.backward()
    gc = c.grad.numpy()
    gp = p.grad
    # FP64 definition: grad_c_k = Re <P_k psi, w> with psi, w as stored (c64)
    ref_c = oracle.term_grad(t.n, t.x, t.z, t.phase, psi.astype(np.complex64).astype(np.complex128),
                             w.astype(np.complex64).astype(np.complex128)).real
    assert rel(gc, ref_c) <= 1e-5
    # central finite differences with the c128 forward
    p128 = p.detach().to(torch.complex128)
    w128 = w64.to(torch.complex128)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    h = 1e-3
    ks = np.random.default_rng(0).choice(t.T, 16, replace=False)
    for k in ks:
        vals = []
        for sgn in (+1, -1):
            cc = t.coeff.real.copy()
            cc[k] += sgn * h
            op.set_coeffs(cc.astype(np.complex128))
            vals.append(float(torch.vdot(op.apply(p128), w128).real))
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(fd - gc[k]) <= 1e-5 * max(1.0, abs(fd)), (k, fd, gc[k])
        assert abs(fd - ref_c[k]) <= 1e-9 * max(1.0, abs(fd)), (k, fd, ref_c[k])
    # grad_psi = H^dagger w: against the c128 adjoint kernel
    op.set_coeffs(t.coeff)
    ref_p = op.apply(w128, adjoint=True)
    assert float(torch.linalg.vector_norm(gp.to(torch.complex128) - ref_p)
                 / torch.linalg.vector_norm(ref_p)) <= 1e-6


def test_autograd_complex_coeffs_c128(cuda):
    """Complex coefficients and complex128 states: grad_c = <P_k psi, g>,
    checked against torch's own autograd through a dense H at n = 8."""
    import torch
    rng = np.random.default_rng(4)
    t = W.random_letters_op(rng, 8, 25)
    terms = PauliTerms(t.n, t.x, t.z, t.phase)
    c0 = t.coeff + 0.3j * rng.standard_normal(t.T)
    psi = W.random_state(rng, 256)
    w = W.random_state(rng, 256)
    c = torch.tensor(c0, dtype=torch.complex128, requires_grad=True)
    p = torch.from_numpy(psi).to(cuda).requires_grad_(True)
    L = torch.vdot(pauli_apply(c, p, terms), torch.from_numpy(w).to(cuda)).real
    L.backward()
    # dense reference: H = sum_k c_k B_k with B_k built column by column
    N = 256
    r = np.arange(N)
    units = np.array([1, -1j, -1, 1j])
    Bs = []
    for k in range(t.T):
        B = np.zeros((N, N), dtype=np.complex128)
        sgn = np.array([(-1) ** bin(int(v) & int(t.z[k])).count("1") for v in r])
        B[r, r ^ int(t.x[k])] = units[t.phase[k]] * sgn
        Bs.append(torch.from_numpy(B))
    cr = torch.tensor(c0, dtype=torch.complex128, requires_grad=True)
    pr = torch.from_numpy(psi).requires_grad_(True)
    H = sum(cr[k] * Bs[k] for k in range(t.T))
    Lr = torch.vdot(H @ pr, torch.from_numpy(w)).real
    Lr.backward()
    assert rel(c.grad.numpy(), cr.grad.numpy()) <= 1e-12
    assert rel(p.grad.cpu().numpy(), pr.grad.numpy()) <= 1e-12
