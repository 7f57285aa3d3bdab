"""ctypes binding for the CPU oracle (oracle/qrusty_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()``
and bench.py's CPU-baseline / reference arm, as the checker and the timed
CPU baseline.  The GPU product path (``qrusty_gb300``) never imports it.

Parity status: pinned against the reference's own known-answer tests and
fixture Hamiltonians (tests/test_oracle_pins.py); the Rust reference itself
cannot be compiled in this environment.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "qrusty_oracle.c")
_OUT_DIR = os.path.join(_HERE, "_build")
_LIB = os.path.join(_OUT_DIR, "liboracle.so")

_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_c128p = np.ctypeslib.ndpointer(dtype=np.complex128, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (no FMA contraction, portable flags)."""
    os.makedirs(_OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(_LIB)
            and os.path.getmtime(_LIB) >= os.path.getmtime(_SRC)):
        return _LIB
    tmp = _LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-pthread",
           "-ffp-contract=off", "-o", tmp, _SRC, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, _LIB)
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        L.or_parse_label.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                     C.c_char_p, C.c_int]
        L.or_parse_label.restype = C.c_int
        L.or_label_masks.argtypes = [C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_uint64),
                                     C.POINTER(C.c_uint64), C.POINTER(C.c_int)]
        L.or_label_masks.restype = None
        L.or_make_params.argtypes = [C.c_size_t, _u8p, _f64p, _f64p]
        L.or_make_params.restype = None
        L.or_make_row.argtypes = [C.c_size_t, _u64p, _u64p, _f64p, C.c_uint64, _u64p, _f64p]
        L.or_make_row.restype = C.c_size_t
        L.or_csr_build.argtypes = [C.c_size_t, C.c_int, _u64p, _u64p, _f64p, C.c_uint64,
                                   C.c_uint64, C.c_size_t, C.c_int]
        L.or_csr_build.restype = C.c_void_p
        L.or_csr_nnz.argtypes = [C.c_void_p]
        L.or_csr_nnz.restype = C.c_size_t
        L.or_csr_fetch.argtypes = [C.c_void_p, _u64p, _u64p, _f64p]
        L.or_csr_fetch.restype = None
        L.or_csr_free.argtypes = [C.c_void_p]
        L.or_csr_free.restype = None
        L.or_spmv.argtypes = [C.c_size_t, _u64p, _u64p, _f64p, _f64p, _f64p, C.c_size_t, C.c_int]
        L.or_spmv.restype = None
        L.or_apply_rows.argtypes = [C.c_size_t, _u64p, _u64p, _f64p, C.c_uint64, C.c_uint64,
                                    _f64p, _f64p, C.c_int]
        L.or_apply_rows.restype = None
        L.or_term_grad.argtypes = [C.c_size_t, C.c_int, _u64p, _u64p, _u8p, _f64p, _f64p, _f64p,
                                   C.c_int]
        L.or_term_grad.restype = None
        L.or_vec.argtypes = [C.c_int, C.c_int, C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p,
                             _f64p, C.c_void_p, C.c_double]
        L.or_vec.restype = None
        L.or_op_diagonal.argtypes = [C.c_size_t, _u64p, _u64p, _f64p, C.c_uint64, C.c_uint64,
                                     _f64p]
        L.or_op_diagonal.restype = None
        _lib = L
    return _lib


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


# --------------------------------------------------------------------------
# Thin numpy-level wrappers
# --------------------------------------------------------------------------

def parse_label(label: str):
    """(base_phase, letters in qubit order) or raises ValueError."""
    bp = C.c_int(0)
    n = C.c_int(0)
    buf = C.create_string_buffer(max(1, len(label)) + 1)
    rc = lib().or_parse_label(label.encode(), C.byref(bp), C.byref(n), buf, len(label))
    if rc != 0:
        raise ValueError("error: malformed label")
    return bp.value, buf.raw[: n.value].decode()


def label_masks(label: str):
    """(x, z, phase) of a label, restating lib.rs:161-181."""
    bp, letters = parse_label(label)
    x = C.c_uint64(0)
    z = C.c_uint64(0)
    ph = C.c_int(0)
    lib().or_label_masks(letters.encode(), len(letters), bp, C.byref(x), C.byref(z), C.byref(ph))
    return x.value, z.value, ph.value


def make_params(phase, coeff):
    phase = np.ascontiguousarray(phase, dtype=np.uint8)
    cf = np.ascontiguousarray(np.asarray(coeff, dtype=np.complex128)).view(np.float64)
    out = np.empty_like(cf)
    lib().or_make_params(len(phase), phase, cf, out)
    return out.view(np.complex128)


def make_row(x, z, cprime, row):
    x = np.ascontiguousarray(x, dtype=np.uint64)
    z = np.ascontiguousarray(z, dtype=np.uint64)
    cp = np.ascontiguousarray(cprime, dtype=np.complex128).view(np.float64)
    cols = np.empty(len(x), dtype=np.uint64)
    vals = np.empty(2 * len(x), dtype=np.float64)
    k = lib().or_make_row(len(x), z, x, cp, row, cols, vals)
    return cols[:k].copy(), vals[: 2 * k].view(np.complex128).copy()


def csr_build(n, x, z, cprime, step=1024, nthreads=None, rows=None):
    """(indptr, indices, data) as make_unsafe_vectors_chunked builds them;
    rows=(lo, hi) builds only that row range (indices stay global)."""
    x = np.ascontiguousarray(x, dtype=np.uint64)
    z = np.ascontiguousarray(z, dtype=np.uint64)
    cp = np.ascontiguousarray(cprime, dtype=np.complex128).view(np.float64)
    lo, hi = rows if rows is not None else (0, 1 << n)
    L = lib()
    h = L.or_csr_build(len(x), n, z, x, cp, lo, hi, step, nthreads or default_threads())
    try:
        nnz = L.or_csr_nnz(h)
        indptr = np.empty(hi - lo + 1, dtype=np.uint64)
        indices = np.empty(nnz, dtype=np.uint64)
        data = np.empty(2 * nnz, dtype=np.float64)
        L.or_csr_fetch(h, indptr, indices, data)
    finally:
        L.or_csr_free(h)
    return indptr, indices, data.view(np.complex128)


def spmv(indptr, indices, data, v, step=1024, nthreads=None):
    """y = A v for a (row-range) CSR; len(y) = len(indptr) - 1."""
    indptr = np.ascontiguousarray(indptr, dtype=np.uint64)
    indices = np.ascontiguousarray(indices, dtype=np.uint64)
    d = np.ascontiguousarray(data, dtype=np.complex128).view(np.float64)
    vv = np.ascontiguousarray(v, dtype=np.complex128).view(np.float64)
    nrows = len(indptr) - 1
    y = np.empty(2 * nrows, dtype=np.float64)
    lib().or_spmv(nrows, indptr, indices, d, vv, y, step, nthreads or default_threads())
    return y.view(np.complex128)


def apply_rows(x, z, cprime, psi, row_lo, row_hi, nthreads=None):
    """Matrix-free restatement of CSR-build + SpMV for rows [row_lo, row_hi)."""
    x = np.ascontiguousarray(x, dtype=np.uint64)
    z = np.ascontiguousarray(z, dtype=np.uint64)
    cp = np.ascontiguousarray(cprime, dtype=np.complex128).view(np.float64)
    p = np.ascontiguousarray(psi, dtype=np.complex128).view(np.float64)
    y = np.empty(2 * (row_hi - row_lo), dtype=np.float64)
    lib().or_apply_rows(len(x), z, x, cp, row_lo, row_hi, p, y, nthreads or default_threads())
    return y.view(np.complex128)


def apply(n, x, z, cprime, psi, nthreads=None):
    return apply_rows(x, z, cprime, psi, 0, 1 << n, nthreads)


def term_grad(n, x, z, phase, psi, g, nthreads=None):
    """<P_k psi, g> per term in FP64 (definition check for the autograd
    backward; no reference counterpart)."""
    x = np.ascontiguousarray(x, dtype=np.uint64)
    z = np.ascontiguousarray(z, dtype=np.uint64)
    ph = np.ascontiguousarray(phase, dtype=np.uint8)
    p = np.ascontiguousarray(psi, dtype=np.complex128).view(np.float64)
    gg = np.ascontiguousarray(g, dtype=np.complex128).view(np.float64)
    out = np.empty(2 * len(x), dtype=np.float64)
    lib().or_term_grad(len(x), n, z, x, ph, p, gg, out, nthreads or default_threads())
    return out.view(np.complex128)


_VEC_OPS = {"axpby": 0, "axpy": 1, "ax": 2, "precond2": 3}


def vec(op, x, y=None, a=0j, b=0j, tol=0.0):
    """Element-wise helper ``op`` (axpby / axpy / ax / precond2) on complex128
    or complex64 arrays; precond2 takes x = diag, y = dx, a = e."""
    x = np.ascontiguousarray(x)
    if x.dtype not in (np.complex128, np.complex64):
        raise TypeError("complex128 or complex64 arrays")
    f32 = x.dtype == np.complex64
    yv = None if y is None else np.ascontiguousarray(y, dtype=x.dtype)
    z = np.empty_like(x)
    av = np.array([complex(a).real, complex(a).imag])
    bv = np.array([complex(b).real, complex(b).imag])
    lib().or_vec(_VEC_OPS[op], int(f32), x.size, x.ctypes.data,
                 None if yv is None else yv.ctypes.data, z.ctypes.data, av,
                 bv.ctypes.data if op == "axpby" else None, float(tol))
    return z


def op_diagonal(x, z, cprime, row0, nrows):
    out = np.empty(2 * nrows)
    lib().or_op_diagonal(len(x), np.ascontiguousarray(z, dtype=np.uint64),
                         np.ascontiguousarray(x, dtype=np.uint64),
                         np.ascontiguousarray(cprime, dtype=np.complex128).view(np.float64),
                         int(row0), int(nrows), out)
    return out.view(np.complex128)


# --------------------------------------------------------------------------
# rawio file layout (qrusty/src/rawio.rs:128-179), restated with numpy
# --------------------------------------------------------------------------
def rawio_bytes(storage, nrows, ncols, indptr, indices, data, byteorder="<"):
    """Bytes of rawio::write (rawio.rs:128-149) as a machine of the given
    byte order writes them: mark b"MI" in that order, u64 storage / rows /
    cols, then (u64 length, words) for indptr, indices and data."""
    u64 = np.dtype(byteorder + "u8")
    f64 = np.dtype(byteorder + "f8")
    mark = b"MI" if byteorder == "<" else b"IM"
    parts = [mark, np.array([storage, nrows, ncols], dtype=u64).tobytes()]
    for arr, dt in ((np.asarray(indptr, np.uint64), u64), (np.asarray(indices, np.uint64), u64)):
        parts.append(np.array([len(arr)], dtype=u64).tobytes())
        parts.append(arr.astype(dt).tobytes())
    d = np.ascontiguousarray(np.asarray(data, np.complex128)).view(np.float64)
    parts.append(np.array([len(d) // 2], dtype=u64).tobytes())
    parts.append(d.astype(f64).tobytes())
    return b"".join(parts)


def rawio_parse(buf):
    """rawio::read (rawio.rs:151-179): the reader swaps when the mark is not
    b"MI" in its own (little-endian here) order."""
    order = "<" if buf[:2] == b"MI" else ">"
    u64 = np.dtype(order + "u8")
    storage, nrows, ncols = (int(v) for v in np.frombuffer(buf, u64, 3, 2))
    if storage > 1:
        raise ValueError("rawio::read: bad storage found")
    off = 26

    def record(off, kind):
        n = int(np.frombuffer(buf, u64, 1, off)[0])
        words = n * (2 if kind == "c" else 1)
        dt = np.dtype(order + ("f8" if kind == "c" else "u8"))
        arr = np.frombuffer(buf, dt, words, off + 8)
        return arr, off + 8 + arr.nbytes

    indptr, off = record(off, "u")
    indices, off = record(off, "u")
    data, off = record(off, "c")
    return (storage, nrows, ncols, indptr.astype(np.uint64), indices.astype(np.uint64),
            data.astype(np.float64).view(np.complex128))
