"""The 64-bit row-word kernel instantiations, run at small n.

qrusty's masks are u64 (qrusty/src/lib.rs:161-176), so operators with
n > 32 take kernels whose row arithmetic, parities and placement are 64-bit
(csr_fill_kernel<true>, csr_fill_staged_kernel<true>, apply_c64c_tab and
apply_c64c_pair with WIDE = true).  A state of 2^33 amplitudes does not fit
a test, so the operator's test hook forces those instantiations at n <= 20:
they must give the oracle's CSR bit for bit, and H psi identical bit for bit
to the 32-bit instantiations (the same products in the same order).
"""
import numpy as np
import pytest

from qrusty_gb300 import PauliOperator
from qrusty_gb300 import workloads as W
from tests.helpers import terms_of_labels

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def _csr_cases(golden):
    t0, _ = W.cfg0(with_state=False)
    t1, _ = W.cfg1(with_state=False, n=12)
    t2 = W.cfg2(n=12, npair=600, nz=150)
    rng = np.random.default_rng(9)
    t3 = W.random_letters_op(rng, 9, 400)  # G > 256: the direct-store kernel
    yield "cfg0", (t0.n, t0.x, t0.z, t0.phase, t0.coeff)
    yield "chain12", (t1.n, t1.x, t1.z, t1.phase, t1.coeff)
    yield "jw12", (t2.n, t2.x, t2.z, t2.phase, t2.coeff)
    yield "letters9", (t3.n, t3.x, t3.z, t3.phase, t3.coeff)
    yield "H6", terms_of_labels(*golden["H6"])


def test_csr_wide_bit_exact(cuda, oracle, golden):
    for name, (n, x, z, ph, c) in _csr_cases(golden):
        op = PauliOperator(n, x, z, ph, c)
        op.set_test_hooks(force_wide=True)
        ip, ij, d = op.csr_host()
        op.sync_check()
        oi, oj, od = oracle.csr_build(n, x, z, oracle.make_params(ph, c))
        assert np.array_equal(ip, oi), name
        assert np.array_equal(ij, oj), name
        assert np.array_equal(_bits(d), _bits(od)), name


def test_csr_wide_device_staged(cuda, oracle):
    """Device build (aligned outputs: the staged bulk-store kernel, with the
    fold-value buffer for the chain's x = 0 group) against the narrow build."""
    import torch
    t, _ = W.cfg1(with_state=False, n=16)
    narrow = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    wide = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    wide.set_test_hooks(force_wide=True)
    a = narrow.csr_device()
    b = wide.csr_device()
    torch.cuda.synchronize()
    narrow.sync_check()
    wide.sync_check()
    assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])
    assert torch.equal(torch.view_as_real(a[2]).view(torch.int64),
                       torch.view_as_real(b[2]).view(torch.int64))
    rng = np.random.default_rng(4)
    cp = oracle.make_params(t.phase, t.coeff)
    G = int(a[0][1])
    ij = b[1].cpu().numpy().view(np.uint64)
    d = b[2].cpu().numpy()
    for r in [0, (1 << t.n) - 1] + [int(v) for v in rng.integers(0, 1 << t.n, 30)]:
        cols, vals = oracle.make_row(t.x, t.z, cp, r)
        assert np.array_equal(ij[r * G:(r + 1) * G], cols)
        assert np.array_equal(_bits(d[r * G:(r + 1) * G]), _bits(vals))


@pytest.mark.parametrize("case", ["pair", "chunked", "single_tile"])
def test_apply_c64c_wide_identical(cuda, oracle, case):
    import torch
    if case == "pair":  # <= 512 sub-groups: partner tiles in pairs
        t = W.cfg2(n=18, npair=900, nz=300)
    elif case == "chunked":  # > 512 sub-groups: table rebuilt per chunk
        t = W.random_letters_op(np.random.default_rng(31), 15, 1200)
    else:  # n = 11: one output tile, 512 threads x 4 amplitudes
        t = W.random_letters_op(np.random.default_rng(32), 11, 300)
    narrow = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    wide = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    wide.set_test_hooks(force_wide=True)
    psi = W.random_state(np.random.default_rng(8), 1 << t.n, nstates=2)
    p = torch.from_numpy(psi.astype(np.complex64)).to(cuda)
    for adj in (False, True):
        y_n = narrow.apply(p, adjoint=adj)
        y_w = wide.apply(p, adjoint=adj)
        narrow.sync_check()
        wide.sync_check()
        assert torch.equal(y_n, y_w)
    y = wide.apply(p).cpu().numpy().astype(np.complex128)
    cp = oracle.make_params(t.phase, t.coeff)
    for s in range(2):
        ref = oracle.apply(t.n, t.x, t.z, cp, psi[s].astype(np.complex64).astype(np.complex128))
        assert np.linalg.norm(y[s] - ref) <= 1e-6 * np.linalg.norm(ref)
