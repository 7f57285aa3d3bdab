"""The C ABI library loads and exports every symbol include/qrusty_gpu.h
declares; argument validation answers without touching a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from qrusty_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "qrusty_gpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|uint64_t)\s+(qr_\w+)\s*\(", src, flags=re.M)))


def test_header_matches_binding():
    assert declared_functions() == sorted(_lib.EXPORTS)


def test_library_exports_all_symbols():
    L = _lib.load()
    for name in declared_functions():
        assert hasattr(L, name), name


def _create(n, x, z, ph, c):
    L = _lib.load()
    h = C.c_void_p()
    x = np.ascontiguousarray(x, dtype=np.uint64)
    z = np.ascontiguousarray(z, dtype=np.uint64)
    ph = np.ascontiguousarray(ph, dtype=np.uint8)
    c = np.ascontiguousarray(c, dtype=np.complex128)
    rc = L.qr_op_create(n, len(x), x.ctypes.data, z.ctypes.data, ph.ctypes.data, c.ctypes.data,
                        C.byref(h))
    return rc, h


@pytest.mark.parametrize("n,x,z,ph,msg", [
    (0, [0], [0], [0], "outside"),
    (64, [0], [0], [0], "outside"),
    (3, [8], [0], [0], "beyond"),
    (3, [0], [9], [0], "beyond"),
    (3, [1], [0], [4], "phase"),
])
def test_create_validation(n, x, z, ph, msg):
    rc, h = _create(n, x, z, ph, [1.0])
    assert rc == _lib.QR_EINVAL
    assert msg in _lib.last_error()
    assert not h.value


def test_create_empty_and_null():
    L = _lib.load()
    h = C.c_void_p()
    assert L.qr_op_create(2, 0, None, None, None, None, C.byref(h)) == _lib.QR_EINVAL
    assert "at least one pauli" in _lib.last_error()
    assert L.qr_op_create(2, 1, None, None, None, None, C.byref(h)) == _lib.QR_EINVAL
    assert L.qr_op_create(2, 1, None, None, None, None, None) == _lib.QR_EINVAL


def test_null_handles_rejected():
    L = _lib.load()
    assert L.qr_apply(None, 0, None, None, 1, 0, None) == _lib.QR_EINVAL
    assert L.qr_csr_build(None, None, None, None, 0, None) == _lib.QR_EINVAL
    assert L.qr_op_destroy(None) == _lib.QR_OK
    assert L.qr_csr_spmv(4, 4, None, None, None, None, None, None) == _lib.QR_EINVAL
    buf = C.create_string_buffer(8)
    n = L.qr_last_error(buf, 8)
    assert n >= len(buf.value) and len(buf.value) <= 7
