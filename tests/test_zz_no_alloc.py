"""qr_vdot_noalloc: the allocation-free inner product.

It exists for callers that cannot allocate device memory while they run
(their memory is reserved up front by another allocator, or their steady-
state loop must not take cudaMalloc's synchronisation or pool growth).  Its
partial sums live in a fixed __device__ array inside libqrusty_gpu, so this
test checks, through the C ABI, that two calls in a row give the same FP64
results as qr_vdot (which uses stream-ordered scratch), within the 1e-12
relative tolerance the other inner-product tests use, and that a request
beyond the array's capacity is refused.  It sits in its own file, collected
last, and passes alone in a fresh process as well as after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from qrusty_gb300 import _lib
from qrusty_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MAX_PARTIALS = 16384  # QR_VDOT_NOALLOC_MAX_PARTIALS in include/qrusty_gpu.h


def _call(fn, n, dtype, a, b, ns, out):
    import torch
    st = torch.cuda.current_stream(a.device).cuda_stream
    rc = fn(n, dtype, a.data_ptr(), b.data_ptr(), ns, out.data_ptr(), st)
    torch.cuda.synchronize()
    return rc


@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_noalloc_matches_vdot_twice(cuda, dtype):
    import torch
    L = _lib.load()
    n, ns = 18, 3
    rng = np.random.default_rng(11)
    a = W.random_state(rng, 1 << n, nstates=ns)
    b = W.random_state(rng, 1 << n, nstates=ns)
    if dtype == "c64":
        a, b = a.astype(np.complex64), b.astype(np.complex64)
        code = _lib.QR_C64C
    else:
        code = _lib.QR_C128
    at = torch.from_numpy(a).to(cuda)
    bt = torch.from_numpy(b).to(cuda)
    want = torch.empty(ns, dtype=torch.complex128, device=cuda)
    _lib.check(_call(L.qr_vdot, n, code, at, bt, ns, want))
    want = want.cpu().numpy()
    for _ in range(2):  # the shared array keeps the previous call's contents
        got = torch.full((ns,), complex("nan"), dtype=torch.complex128, device=cuda)
        _lib.check(_call(L.qr_vdot_noalloc, n, code, at, bt, ns, got))
        got = got.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want)
    # swapped arguments give the conjugate (complex64 inputs: products are
    # FP32-rounded, so the symmetry holds to the 1e-6 used for c64 inputs)
    got = torch.empty(ns, dtype=torch.complex128, device=cuda)
    _lib.check(_call(L.qr_vdot_noalloc, n, code, bt, at, ns, got))
    tol = 1e-12 if dtype == "c128" else 1e-6
    assert np.linalg.norm(got.cpu().numpy() - np.conj(want)) <= tol * np.linalg.norm(want)


def test_noalloc_rejects_beyond_capacity(cuda):
    import torch
    L = _lib.load()
    n, ns = 1, MAX_PARTIALS + 1
    a = torch.zeros((ns, 2), dtype=torch.complex128, device=cuda)
    out = torch.empty(ns, dtype=torch.complex128, device=cuda)
    rc = _call(L.qr_vdot_noalloc, n, _lib.QR_C128, a, a, ns, out)
    assert rc == _lib.QR_EINVAL
    assert "QR_VDOT_NOALLOC_MAX_PARTIALS" in _lib.last_error()


@pytest.mark.parametrize("n,ns,dtype", [(18, 512, "c64"), (4, MAX_PARTIALS, "c128")])
def test_noalloc_capped_block_count(cuda, n, ns, dtype):
    """Many states: the per-state block count is cut so that nstates x blocks
    fits the fixed array (n = 18, 512 states: 64 blocks per state cut to 32;
    n = 4, 16,384 states: exactly QR_VDOT_NOALLOC_MAX_PARTIALS partial sums).
    Only the summation order differs from qr_vdot."""
    import torch
    L = _lib.load()
    g = torch.Generator(device=cuda).manual_seed(3)
    tdt = torch.complex64 if dtype == "c64" else torch.complex128
    rdt = torch.float32 if dtype == "c64" else torch.float64
    code = _lib.QR_C64C if dtype == "c64" else _lib.QR_C128
    N = 1 << n
    a = torch.complex(torch.randn(ns * N, device=cuda, dtype=rdt, generator=g),
                      torch.randn(ns * N, device=cuda, dtype=rdt, generator=g)).to(tdt)
    b = torch.complex(torch.randn(ns * N, device=cuda, dtype=rdt, generator=g),
                      torch.randn(ns * N, device=cuda, dtype=rdt, generator=g)).to(tdt)
    want = torch.empty(ns, dtype=torch.complex128, device=cuda)
    _lib.check(_call(L.qr_vdot, n, code, a, b, ns, want))
    for _ in range(2):
        got = torch.full((ns,), complex("nan"), dtype=torch.complex128, device=cuda)
        _lib.check(_call(L.qr_vdot_noalloc, n, code, a, b, ns, got))
        d = (got - want).abs()
        assert bool(torch.all(torch.isfinite(got)))
        assert float(d.max()) <= 1e-12 * float(want.abs().max()) * 10
        assert float(torch.linalg.vector_norm(got - want)) <= 1e-12 * float(
            torch.linalg.vector_norm(want))
