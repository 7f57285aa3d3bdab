"""Batched H psi (one persistent, graph-replayed launch over many uneven
operators) vs the per-operator kernels.  Tolerance: compensated-c64 results
within 1e-6 relative of the per-operator complex128 results (themselves
checked against the FP64 oracle in test_gpu_apply.py)."""
import numpy as np
import pytest

from qrusty_gb300 import Batch, PauliOperator
from qrusty_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def rel(a, b):
    import torch
    return float(torch.linalg.vector_norm(a.to(torch.complex128) - b) / torch.linalg.vector_norm(b))


def make_batch(ops_terms, nstates, cuda, seed):
    import torch
    g = torch.Generator(device=cuda).manual_seed(seed)
    ops, psis, ys = [], [], []
    for t, ns in zip(ops_terms, nstates):
        ops.append(PauliOperator(t.n, t.x, t.z, t.phase, t.coeff))
        p = torch.complex(torch.randn(ns << t.n, device=cuda, generator=g),
                          torch.randn(ns << t.n, device=cuda, generator=g))
        psis.append(p.to(torch.complex64))
        ys.append(torch.empty_like(psis[-1]))
    return ops, psis, ys


def check_against_c128(ops, psis, ys):
    import torch
    worst = 0.0
    for op, p, y in zip(ops, psis, ys):
        ref = op.apply(p.to(torch.complex128))
        e = rel(y, ref)
        worst = max(worst, e)
    return worst


@pytest.mark.parametrize("mode", [-1, 0, 1])
def test_batch_uneven_small(cuda, mode):
    """Both launch forms (persistent work-list kernel, graph of per-operator
    kernels) and the timed choice between them."""
    rng = np.random.default_rng(42)
    terms, nstates = [], []
    for k in range(24):
        n = int(rng.integers(3, 15))
        T = int(rng.integers(5, 300))
        t = W.random_letters_op(rng, n, T)
        if k % 3 == 0:
            t.coeff = t.coeff * (1 + 0.4j)
        terms.append(t)
        nstates.append(int(rng.integers(1, 5)))
    terms.append(W.cfg1(with_state=False, n=13)[0])  # diagonal-vector operator
    nstates.append(2)
    ops, psis, ys = make_batch(terms, nstates, cuda, 1)
    b = Batch(ops, nstates)
    assert b.mode == -1
    b.set_mode(mode)
    b.apply(psis, ys)
    assert b.tile_bits in (10, 11, 12)
    assert b.mode in ((0, 1) if mode == -1 else (mode,))
    assert check_against_c128(ops, psis, ys) <= 1e-6
    # graph replay with the same buffers, then with new output buffers
    import torch
    first = [y.clone() for y in ys]
    b.apply(psis, ys)
    for a_, b_ in zip(first, ys):
        assert torch.equal(a_, b_)
    ys2 = [torch.empty_like(y) for y in ys]
    b.apply(psis, ys2)
    torch.cuda.synchronize()
    for a_, b_ in zip(first, ys2):
        assert torch.equal(a_, b_)
    with pytest.raises(Exception, match="already chosen"):
        b.set_mode(0)


def test_batch_matches_single_operator_kernel(cuda):
    import torch
    t = W.cfg2(n=16, npair=600, nz=200)
    ops, psis, ys = make_batch([t], [3], cuda, 7)
    b = Batch(ops, [3])
    b.apply(psis, ys)
    single = ops[0].apply(psis[0])
    assert rel(ys[0], single.to(torch.complex128)) <= 1e-6


def test_batch_uneven_workload(cuda):
    """The uneven batch workload: 256 operators, n ~ U{10..20}, T ~ U{50..5000}
    random-letter terms, 8 states each, one launch."""
    terms = W.cfg3()
    ops, psis, ys = make_batch(terms, [8] * len(terms), cuda, 3)
    b = Batch(ops, [8] * len(terms))
    b.apply(psis, ys)
    assert check_against_c128(ops, psis, ys) <= 1e-6
