"""Coefficient updates on the device (qr_op_set_coeffs_device).

The kernels redo, from coefficients in device memory, the FP64 operations
the host plan builder performs (make_params' product,
qrusty/src/accel.rs:141-157, the merged sums, every table entry), so after
an update every kernel must return bit for bit what an operator created with
those coefficients returns: both dtypes, forward and adjoint, diagonal-
vector operators and term-by-term (rank > 4) groups, batches.  Host-side
consumers (CSR build, operator diagonal, plans built later) fetch the
coefficients once and must match the oracle bit for bit.  A training step
(forward, backward to c and psi, SGD update) with coefficients on the GPU
is captured into a CUDA graph -- which no host synchronisation survives --
and its replays must equal the eager steps.
"""
import numpy as np
import pytest

from qrusty_gb300 import Batch, PauliOperator
from qrusty_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _fat_groups_op(rng, n=10, T=60):
    """x in a few masks, z random: groups whose z span has rank > 4 (the
    complex128 plan folds them term by term; complex64 splits them)."""
    xs = np.array([0b11, 0b101, 0b1000000001], dtype=np.uint64)
    x = xs[rng.integers(0, len(xs), T)]
    z = rng.integers(0, 1 << n, T).astype(np.uint64)
    ph = rng.integers(0, 4, T).astype(np.uint8)
    c = (rng.standard_normal(T) + 1j * rng.standard_normal(T)).astype(np.complex128)
    return W.Terms(n, x, z, ph, c)


def _cases():
    rng = np.random.default_rng(123)
    yield "jw16", W.cfg2(n=16, npair=700, nz=300)           # diagonal vector, pairs
    yield "letters14", W.random_letters_op(rng, 14, 1500)   # several table chunks
    yield "chain13", W.cfg1(with_state=False, n=13)[0]      # x = 0 group of rank 12
    yield "fat10", _fat_groups_op(rng)
    yield "letters11", W.random_letters_op(rng, 11, 300)   # one tile, 4 amplitudes


@pytest.mark.parametrize("name,t", list(_cases()))
def test_device_update_bit_identical(cuda, oracle, name, t):
    import torch
    rng = np.random.default_rng(7)
    c1 = (rng.standard_normal(t.T) + 0.5j * rng.standard_normal(t.T)).astype(np.complex128)
    c1[:3] = c1[:3].real  # a few real ones
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    psi = W.random_state(np.random.default_rng(8), 1 << t.n, nstates=2)
    p128 = torch.from_numpy(psi).to(cuda)
    p64 = p128.to(torch.complex64)
    # build every plan with the old coefficients
    for p in (p128, p64):
        for adj in (False, True):
            op.apply(p, adjoint=adj)
    torch.cuda.synchronize()
    op.set_coeffs_device(torch.from_numpy(c1).to(cuda))
    fresh = PauliOperator(t.n, t.x, t.z, t.phase, c1)
    for p in (p128, p64):
        for adj in (False, True):
            a = op.apply(p, adjoint=adj)
            b = fresh.apply(p, adjoint=adj)
            op.sync_check()
            assert torch.equal(torch.view_as_real(a), torch.view_as_real(b)), (name, p.dtype, adj)
    # host-side consumers fetch the device coefficients: CSR bit-exact
    ip, ij, d = op.csr_host()
    oi, oj, od = oracle.csr_build(t.n, t.x, t.z, oracle.make_params(t.phase, c1))
    assert np.array_equal(ij, oj)
    assert np.array_equal(d.view(np.uint64), od.view(np.uint64))
    assert torch.equal(op.diagonal(), fresh.diagonal())


def test_device_update_then_host_update(cuda):
    """A host update after a device one wins; a plan first built after a
    device update uses the device coefficients."""
    import torch
    t = W.cfg2(n=14, npair=300, nz=100)
    rng = np.random.default_rng(1)
    c1 = rng.standard_normal(t.T).astype(np.complex128)
    c2 = rng.standard_normal(t.T).astype(np.complex128)
    psi = torch.from_numpy(W.random_state(rng, 1 << t.n)).to(cuda)
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    op.set_coeffs_device(torch.from_numpy(c1).to(cuda))
    # no plan existed: the first apply builds it from the device values
    assert torch.equal(op.apply(psi), PauliOperator(t.n, t.x, t.z, t.phase, c1).apply(psi))
    op.set_coeffs(c2)
    assert torch.equal(op.apply(psi), PauliOperator(t.n, t.x, t.z, t.phase, c2).apply(psi))
    op.set_coeffs_device(torch.from_numpy(c1).to(cuda))
    assert torch.equal(op.apply(psi), PauliOperator(t.n, t.x, t.z, t.phase, c1).apply(psi))


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_batch_follows_device_update(cuda, mode):
    import torch
    rng = np.random.default_rng(2)
    terms = [W.random_letters_op(rng, int(rng.integers(10, 14)), int(rng.integers(50, 600)))
             for _ in range(5)]
    ops = [PauliOperator(t.n, t.x, t.z, t.phase, t.coeff) for t in terms]
    g = torch.Generator(device=cuda).manual_seed(4)
    psis = [torch.complex(torch.randn(2 << t.n, device=cuda, generator=g),
                          torch.randn(2 << t.n, device=cuda, generator=g)) for t in terms]
    ys = [torch.empty_like(p) for p in psis]
    b = Batch(ops, [2] * len(ops))
    b.set_mode(mode)
    b.apply(psis, ys)
    c1 = rng.standard_normal(terms[3].T).astype(np.complex128)
    ops[3].set_coeffs_device(torch.from_numpy(c1).to(cuda))
    b.apply(psis, ys)
    terms[3].coeff = c1
    fresh = [PauliOperator(t.n, t.x, t.z, t.phase, t.coeff) for t in terms]
    b2 = Batch(fresh, [2] * len(ops))
    b2.set_mode(mode)
    ys2 = [torch.empty_like(p) for p in psis]
    b2.apply(psis, ys2)
    torch.cuda.synchronize()
    for u, v in zip(ys, ys2):
        assert torch.equal(torch.view_as_real(u), torch.view_as_real(v))


def test_training_step_captured_in_a_graph(cuda):
    """The configs-4 shape at n = 14: forward, backward to c and psi, SGD on
    c, with c on the GPU.  The step captures into a CUDA graph (no host
    synchronisation inside it) and K replays equal K eager steps."""
    import torch
    from qrusty_gb300.autograd import PauliTerms, pauli_apply
    rng = np.random.default_rng(14)
    t = W.random_letters_op(rng, 14, 400)
    psi = W.random_state(rng, 1 << t.n).astype(np.complex64)
    w = W.random_state(rng, 1 << t.n).astype(np.complex64)
    c0 = torch.tensor(t.coeff.real, dtype=torch.float64, device=cuda)

    def run(capture, K=4):
        terms = PauliTerms(t.n, t.x, t.z, t.phase)
        c = c0.clone().requires_grad_(True)
        p = torch.from_numpy(psi).to(cuda).requires_grad_(True)
        wd = torch.from_numpy(w).to(cuda)
        lr = 1e-2

        def step():
            y = pauli_apply(c, p, terms)
            torch.vdot(y, wd).real.backward()
            with torch.no_grad():
                c.sub_(lr * c.grad)
                c.grad.zero_()
                p.grad.zero_()

        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            for _ in range(2):  # plans, grad tables and allocator warm-up
                step()
        torch.cuda.current_stream().wait_stream(s)
        if not capture:
            for _ in range(K):
                step()
            torch.cuda.synchronize()
            return c.detach().clone()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            step()
        for _ in range(K):
            graph.replay()
        torch.cuda.synchronize()
        return c.detach().clone()

    eager = run(False)
    graphed = run(True)
    assert torch.equal(eager, graphed)
    assert not torch.equal(eager, c0)
