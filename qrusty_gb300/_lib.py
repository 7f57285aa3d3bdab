"""ctypes loader for libqrusty_gpu.so (the C ABI of include/qrusty_gpu.h).

The library is the only compute path: there is no CPU fallback, and a
missing or stale build raises instead of degrading silently.
"""
from __future__ import annotations

import ctypes as C
import os

import importlib

QR_OK = 0
QR_EINVAL = -1
QR_ECUDA = -2
QR_ENOMEM = -3
QR_EKERNEL = -4
QR_ESTATE = -5

QR_MEM_DEVICE = 0
QR_MEM_HOST = 1

QR_C128 = 0
QR_C64C = 1

# Every entry point include/qrusty_gpu.h declares (checked by the tests).
EXPORTS = (
    "qr_op_create", "qr_op_destroy", "qr_op_get_info", "qr_csr_size", "qr_csr_build",
    "qr_apply", "qr_check", "qr_apply_host", "qr_csr_spmv", "qr_op_set_coeffs", "qr_vdot",
    "qr_expect", "qr_term_grad", "qr_vdot_noalloc", "qr_batch_create", "qr_batch_destroy",
    "qr_batch_apply", "qr_batch_tile_bits", "qr_batch_mode", "qr_batch_set_mode", "qr_axpby", "qr_axpy", "qr_ax", "qr_precond2",
    "qr_csr_diagonal", "qr_op_diagonal", "qr_apply_axpby", "qr_rawio_info", "qr_rawio_read", "qr_rawio_write",
    "qr_mm_write", "qr_mm_open", "qr_mm_fetch", "qr_mm_close", "qr_last_error", "qr_launch_count",
    "qr_op_set_test_hooks", "qr_op_set_coeffs_device", "qr_op_get_groups",
)

QR_TEST_FORCE_WIDE = 1


class CsrFileInfo(C.Structure):
    _fields_ = [("storage", C.c_uint64), ("nrows", C.c_uint64), ("ncols", C.c_uint64),
                ("indptr_len", C.c_uint64), ("nnz", C.c_uint64), ("byte_swapped", C.c_int32)]


class QrError(RuntimeError):
    """A libqrusty_gpu call returned a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


class OpInfo(C.Structure):
    _fields_ = [("n", C.c_int32), ("tile_bits", C.c_int32), ("nterms", C.c_uint64),
                ("ngroups", C.c_uint64), ("nmerged", C.c_uint64), ("nblocks", C.c_uint64),
                ("nfat", C.c_uint64), ("nsub", C.c_uint64), ("has_diag", C.c_int32),
                ("device", C.c_int32)]


_lib = None


def lib_path() -> str:
    return importlib.import_module(__package__ + ".build").LIB


def load(build_if_missing: bool = True):
    """Load libqrusty_gpu.so (building it with nvcc if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    _build = importlib.import_module(__package__ + ".build")  # loaded on first use only
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError("libqrusty_gpu.so is not built: run __graft_entry__.build()")
        _build.build()
    L = C.CDLL(path)
    vp, u64, i32 = C.c_void_p, C.c_uint64, C.c_int32
    L.qr_op_create.argtypes = [i32, u64, vp, vp, vp, vp, C.POINTER(vp)]
    L.qr_op_destroy.argtypes = [vp]
    L.qr_op_get_info.argtypes = [vp, C.POINTER(OpInfo)]
    L.qr_op_get_groups.argtypes = [vp, C.POINTER(u64), vp, vp, vp, vp]
    L.qr_csr_size.argtypes = [vp, C.POINTER(u64), C.POINTER(u64)]
    L.qr_csr_build.argtypes = [vp, vp, vp, vp, i32, vp]
    L.qr_apply.argtypes = [vp, i32, vp, vp, i32, i32, vp]
    L.qr_check.argtypes = [vp, vp]
    L.qr_apply_host.argtypes = [vp, i32, vp, vp, i32, i32]
    L.qr_csr_spmv.argtypes = [u64, u64, vp, vp, vp, vp, vp, vp]
    L.qr_op_set_coeffs.argtypes = [vp, vp]
    L.qr_op_set_test_hooks.argtypes = [vp, C.c_uint32, u64, C.c_int64]
    L.qr_op_set_coeffs_device.argtypes = [vp, vp, vp]
    L.qr_vdot.argtypes = [i32, i32, vp, vp, i32, vp, vp]
    L.qr_expect.argtypes = [vp, i32, vp, i32, vp, vp]
    L.qr_vdot_noalloc.argtypes = [i32, i32, vp, vp, i32, vp, vp]
    L.qr_batch_create.argtypes = [i32, vp, vp, C.POINTER(vp)]
    L.qr_batch_destroy.argtypes = [vp]
    L.qr_batch_apply.argtypes = [vp, vp, vp, vp]
    L.qr_batch_tile_bits.argtypes = [vp]
    L.qr_batch_mode.argtypes = [vp]
    L.qr_batch_set_mode.argtypes = [vp, i32]
    L.qr_term_grad.argtypes = [vp, i32, vp, vp, i32, vp, vp]
    L.qr_axpby.argtypes = [i32, u64, vp, vp, vp, vp, vp, vp]
    L.qr_axpy.argtypes = [i32, u64, vp, vp, vp, vp, vp]
    L.qr_ax.argtypes = [i32, u64, vp, vp, vp, vp]
    L.qr_precond2.argtypes = [i32, u64, vp, vp, vp, C.c_double, vp, vp]
    L.qr_csr_diagonal.argtypes = [u64, u64, vp, vp, vp, vp, vp]
    L.qr_op_diagonal.argtypes = [vp, i32, vp, vp]
    L.qr_apply_axpby.argtypes = [vp, i32, vp, vp, vp, vp, vp, i32, vp]
    L.qr_rawio_info.argtypes = [C.c_char_p, C.POINTER(CsrFileInfo)]
    L.qr_rawio_read.argtypes = [C.c_char_p, vp, vp, vp, i32, vp]
    L.qr_rawio_write.argtypes = [C.c_char_p, u64, u64, u64, vp, u64, vp, vp, u64, i32, vp]
    L.qr_mm_write.argtypes = [C.c_char_p, u64, u64, vp, vp, vp, i32, i32, vp]
    L.qr_mm_open.argtypes = [C.c_char_p, C.POINTER(vp), C.POINTER(u64), C.POINTER(u64),
                             C.POINTER(u64)]
    L.qr_mm_fetch.argtypes = [vp, vp, vp, vp, i32, vp]
    L.qr_mm_close.argtypes = [vp]
    L.qr_last_error.argtypes = [C.c_char_p, C.c_size_t]
    for name in EXPORTS:
        getattr(L, name).restype = C.c_int
    L.qr_launch_count.argtypes = []
    L.qr_launch_count.restype = C.c_uint64
    _lib = L
    return L


def last_error() -> str:
    L = load()
    buf = C.create_string_buffer(1024)
    L.qr_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int) -> None:
    if rc != QR_OK:
        raise QrError(rc, last_error() or ("libqrusty_gpu error %d" % rc))


def launch_count() -> int:
    return int(load().qr_launch_count())
