"""Batched H psi (one persistent, graph-replayed launch over many uneven
operators).  Tolerance: compensated-c64 results within 1e-6 relative of the
FP64 oracle (row blocks of every state of a dozen operators spanning every
qubit count of the uneven workload), and of the per-operator complex128
kernel for the rest."""
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


def check_against_oracle(oracle, terms, psis, ys, pick, rows=4096, seed=0):
    """Rel. error of batched results against the FP64 oracle, per state, on
    every row (2^n <= 2 rows) or on a random block of ``rows`` rows."""
    rng = np.random.default_rng(seed)
    worst = 0.0
    for i in pick:
        t = terms[i]
        N = 1 << t.n
        cp = oracle.make_params(t.phase, t.coeff)
        P = psis[i].cpu().numpy().reshape(-1, N).astype(np.complex128)
        Y = ys[i].cpu().numpy().reshape(-1, N).astype(np.complex128)
        for s in range(P.shape[0]):
            lo = 0 if N <= 2 * rows else int(rng.integers(0, N - rows))
            hi = N if N <= 2 * rows else lo + rows
            ref = oracle.apply_rows(t.x, t.z, cp, P[s], lo, hi)
            e = float(np.linalg.norm(Y[s, lo:hi] - ref) / np.linalg.norm(ref))
            worst = max(worst, e)
    return worst


def spread_pick(terms):
    """One operator per qubit count (smallest and largest term count for the
    two extreme qubit counts): a dozen or more operators of the workload."""
    by_n = {}
    for i, t in enumerate(terms):
        by_n.setdefault(t.n, []).append(i)
    pick = []
    ns = sorted(by_n)
    for n in ns:
        idx = sorted(by_n[n], key=lambda i: terms[i].T)
        pick.append(idx[-1])
        if n in (ns[0], ns[-1]) and len(idx) > 1:
            pick.append(idx[0])
    return pick


def check_against_c128(ops, psis, ys):
    import torch
    worst = 0.0
    for op, p, y in zip(ops, psis, ys):
        ref = op.apply(p.to(torch.complex128))
        e = rel(y, ref)
        worst = max(worst, e)
    return worst


@pytest.mark.parametrize("mode", [-1, 0, 1, 2])
def test_batch_uneven_small(cuda, mode):
    """Every launch form (persistent work-list kernel, graph of per-operator
    kernels, both: persistent for the small operators) and the timed choice."""
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
    assert b.mode in ((0, 1, 2) if mode == -1 else (mode,))
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


def test_batch_uneven_workload(cuda, oracle):
    """The uneven batch workload: 256 operators, n ~ U{10..20}, T ~ U{50..5000}
    random-letter terms, 8 states each, one launch; a dozen operators against
    the oracle, every state, the rest against the complex128 kernel."""
    terms = W.cfg3()
    ops, psis, ys = make_batch(terms, [8] * len(terms), cuda, 3)
    b = Batch(ops, [8] * len(terms))
    b.apply(psis, ys)
    pick = spread_pick(terms)
    assert len(pick) >= 12 and len({terms[i].n for i in pick}) == 11
    assert check_against_oracle(oracle, terms, psis, ys, pick) <= 1e-6
    assert check_against_c128(ops, psis, ys) <= 1e-6


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_batch_forms_vs_oracle(cuda, oracle, mode):
    """Each launch form, forced, on a dozen operators of the uneven workload
    (every qubit count) against the FP64 oracle, every state."""
    terms = W.cfg3()
    pick = spread_pick(terms)
    sub = [terms[i] for i in pick]
    ops, psis, ys = make_batch(sub, [8] * len(sub), cuda, 11)
    b = Batch(ops, [8] * len(sub))
    b.set_mode(mode)
    b.apply(psis, ys)
    assert b.mode == mode
    assert check_against_oracle(oracle, sub, psis, ys, range(len(sub))) <= 1e-6


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_batch_after_set_coeffs(cuda, oracle, mode):
    """A coefficient update of one operator reaches the batch's next apply."""
    import torch
    rng = np.random.default_rng(5)
    terms = [W.random_letters_op(rng, int(rng.integers(10, 15)), int(rng.integers(50, 700)))
             for _ in range(6)]
    ops, psis, ys = make_batch(terms, [2] * len(terms), cuda, 12)
    b = Batch(ops, [2] * len(terms))
    b.set_mode(mode)
    b.apply(psis, ys)
    assert check_against_oracle(oracle, terms, psis, ys, range(len(terms))) <= 1e-6
    terms[2].coeff = terms[2].coeff * -0.5 + 0.25j
    ops[2].set_coeffs(terms[2].coeff)
    b.apply(psis, ys)
    torch.cuda.synchronize()
    assert check_against_oracle(oracle, terms, psis, ys, range(len(terms))) <= 1e-6
