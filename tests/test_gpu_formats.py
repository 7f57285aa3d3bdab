"""On-disk CSR formats from and into device memory: a CSR built on the GPU
goes to disk through the pinned staging path and comes back bit for bit."""
import ctypes as C

import numpy as np
import pytest

from qrusty_gb300 import PauliOperator, SpMat
from qrusty_gb300 import _lib
from qrusty_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("suffix", [".raw", ".raw.gz"])
def test_rawio_device_roundtrip(cuda, oracle, tmp_path, suffix):
    import torch
    t = W.cfg1(with_state=False, n=16)[0]  # 2^16 rows x 44: 69 MB of CSR, > one staging chunk
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    ip, ij, d = op.csr_device()
    L = _lib.load()
    path = str(tmp_path / ("chain" + suffix)).encode()
    N = 1 << t.n
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(L.qr_rawio_write(path, 0, N, N, ip.data_ptr(), ip.numel(), ij.data_ptr(),
                                d.data_ptr(), d.numel(), _lib.QR_MEM_DEVICE, st))
    if suffix == ".raw":
        want = oracle.rawio_bytes(0, N, N, ip.cpu().numpy().view(np.uint64),
                                  ij.cpu().numpy().view(np.uint64), d.cpu().numpy())
        assert (tmp_path / "chain.raw").read_bytes() == want
    info = _lib.CsrFileInfo()
    _lib.check(L.qr_rawio_info(path, C.byref(info)))
    assert (info.nrows, info.indptr_len, info.nnz) == (N, N + 1, d.numel())
    ip2, ij2 = torch.empty_like(ip), torch.empty_like(ij)
    d2 = torch.empty_like(d)
    _lib.check(L.qr_rawio_read(path, ip2.data_ptr(), ij2.data_ptr(), d2.data_ptr(),
                               _lib.QR_MEM_DEVICE, st))
    assert torch.equal(ip2, ip) and torch.equal(ij2, ij)
    assert torch.equal(d2.view(torch.float64), d.view(torch.float64))


def test_matrixmarket_device_roundtrip(cuda, tmp_path):
    import torch
    t = W.cfg0()[0]
    op = PauliOperator(t.n, t.x, t.z, t.phase, t.coeff)
    ip, ij, d = op.csr_device()
    L = _lib.load()
    path = str(tmp_path / "cfg0.mtx").encode()
    N = 1 << t.n
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(L.qr_mm_write(path, N, N, ip.data_ptr(), ij.data_ptr(), d.data_ptr(), 0,
                             _lib.QR_MEM_DEVICE, st))
    back = SpMat.matrixmarket_read(path.decode())
    shape, d2, ij2, ip2 = back.export()
    # the text round trip is exact (shortest round-trip decimals); explicit
    # zeros are kept on both sides
    assert np.array_equal(ip2, ip.cpu().numpy().view(np.uint64))
    assert np.array_equal(ij2, ij.cpu().numpy().view(np.uint64))
    assert d2.tobytes() == d.cpu().numpy().tobytes()
    h = C.c_void_p()
    nr, nc, nz = C.c_uint64(), C.c_uint64(), C.c_uint64()
    _lib.check(L.qr_mm_open(path, C.byref(h), C.byref(nr), C.byref(nc), C.byref(nz)))
    ip3, ij3 = torch.empty_like(ip), torch.empty_like(ij)
    d3 = torch.empty_like(d)
    _lib.check(L.qr_mm_fetch(h, ip3.data_ptr(), ij3.data_ptr(), d3.data_ptr(),
                             _lib.QR_MEM_DEVICE, st))
    L.qr_mm_close(h)
    assert torch.equal(ip3, ip) and torch.equal(ij3, ij)
    assert torch.equal(d3.view(torch.float64), d.view(torch.float64))
