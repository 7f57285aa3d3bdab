"""pyqrusty-compatible Python edge over libqrusty_gpu.

Mirrors the classes and functions of qrusty's pyo3 binding
(pyqrusty/src/lib.rs, pyqrusty/python/pyqrusty/__init__.py) for the
Pauli-operator hot path -- same names, argument meaning and error messages --
with every numeric result computed by the sm_103a kernels behind the C ABI
(include/qrusty_gpu.h):

* ``Pauli`` (pyqrusty/src/lib.rs:262-303; parsing qrusty/src/lib.rs:125-181)
* ``SparsePauliOp`` (pyqrusty/src/lib.rs:305-433; qrusty/src/lib.rs:345-586)
  with ``to_matrix`` / ``to_matrix_mode`` routed to the GPU CSR builder and
  a matrix-free ``apply`` (H psi on the GPU)
* ``SpMat`` (pyqrusty/src/lib.rs:33-260): CSR holder with ``export``,
  ``matrixmarket_write / _write_symmetric / _read`` and qrusty's binary
  ``rawio`` format (qrusty/src/rawio.rs), ".gz" paths compressed
* ``spmat_dot_densevec`` (pyqrusty/src/lib.rs:476-491): GPU CSR * vector
* ``csr_matrix`` (pyqrusty/python/pyqrusty/__init__.py:14-17)
* the eigensolver-loop vector helpers ``axpby`` / ``axpy`` / ``ax``
  (qrusty/src/accel.rs:374-393), ``precond`` / ``precond2``
  (pyqrusty/src/lib.rs:436-469) and ``SpMat.diagonal`` (:118-125), on the GPU

Out of scope here (matrix algebra around the path, not the path):
``+``/``-``/``scale`` on SpMat, ``a_spmat_p_b_spmat``, zero counting.
"""
from __future__ import annotations

import ctypes as C
import math
import re
from typing import Optional

import numpy as np

from . import _lib
from ._lib import QR_C128, QR_C64C, QR_MEM_HOST, QrError, check

__all__ = ["Pauli", "SparsePauliOp", "SpMat", "PauliOperator", "spmat_dot_densevec",
           "csr_matrix", "QrError", "parse_mode", "vdot", "Batch", "axpby", "axpy", "ax",
           "precond", "precond2"]

_LABEL_RE = re.compile(r"^([+-]?)1?([ij]?)([IXYZ]+)$")


def _rust_f64(x: float) -> str:
    """f64 Display as Rust formats it: shortest round-trip digits, never
    exponent notation, "-0" for negative zero, "NaN", "inf"."""
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    return np.format_float_positional(float(x), unique=True, trim="-")


def _complex_to_string(c: complex) -> str:
    """qrusty/src/util.rs complex64_to_string: format!("{}+{}j", re, im)."""
    return "%s+%sj" % (_rust_f64(c.real), _rust_f64(c.imag))


class Pauli:
    """One Pauli string, parsed as qrusty's Pauli::parse_label
    (qrusty/src/lib.rs:125-149): ``^([+-]?)1?([ij]?)([IXYZ]+)$``, base phase
    1 for i/j plus 2 for a leading '-', letters reversed so that qubit 0 is
    the rightmost character."""

    __slots__ = ("_base_phase", "_letters")

    def __init__(self, label: str):
        m = _LABEL_RE.match(label)
        if m is None:
            raise Exception("error: malformed label")
        sign, imag, paulistr = m.group(1), m.group(2), m.group(3)
        phase = 1 if imag in ("i", "j") else 0
        if sign == "-":
            phase += 2
        self._base_phase = phase
        self._letters = paulistr[::-1]  # qubit order

    # -- pyqrusty surface
    def num_qubits(self) -> int:
        return len(self._letters)

    def label(self) -> str:
        return self._letters[::-1]

    def __repr__(self) -> str:
        return "Pauli('%s')" % self.label()

    def __str__(self) -> str:
        return self.label()

    def to_matrix(self) -> "SpMat":
        """Single-Pauli matrix in the kron convention (qrusty/src/lib.rs:203-213)."""
        return SparsePauliOp([self], [1.0 + 0.0j]).to_matrix()

    # -- masks (qrusty/src/lib.rs:161-190)
    def base_phase(self) -> int:
        return self._base_phase

    def x_indices(self) -> int:
        return sum(1 << i for i, c in enumerate(self._letters) if c in "XY")

    def z_indices(self) -> int:
        return sum(1 << i for i, c in enumerate(self._letters) if c in "YZ")

    def phase(self) -> int:
        return (self._base_phase + self._letters.count("Y")) % 4

    def xs(self):
        return [c in "XY" for c in self._letters]

    def zs(self):
        return [c in "YZ" for c in self._letters]


# AccelMode (qrusty/src/lib.rs:270-331).  Kron-family modes build each Pauli
# as i^base * (x) 2x2 factors (Pauli::to_matrix, lib.rs:203-213); the others
# multiply by (-i)^phase as make_params does (accel.rs:141-157).  The two
# agree unless a label carries an i / -i prefix.
_KRON_MODES = {None, "Binary", "Reduce", "Rayon"}
_RUC_RE = re.compile(r"RowwiseUnsafeChunked/(\d+)")
_RC_RE = re.compile(r"RayonChunked/(\d+)")


def parse_mode(value: str):
    """AccelMode::try_from (qrusty/src/lib.rs:293-331); returns
    (name, step) or raises ValueError."""
    if value in ("Binary", "Accel", "Rowwise", "RowwiseUnsafe"):
        return value, None
    m = _RUC_RE.search(value)
    if m:
        return "RowwiseUnsafeChunked", int(m.group(1))
    if value in ("Reduce", "Rayon"):
        return value, None
    m = _RC_RE.search(value)
    if m:
        return "RayonChunked", int(m.group(1))
    raise ValueError("AccelMode:try_from: unrecognized argument string")


class PauliOperator:
    """Owner of one ``qr_op`` handle: the operator's term tables on the GPU.

    Terms are (x, z, phase, coeff) as qrusty's make_params consumes them.
    """

    def __init__(self, n: int, x, z, phase, coeffs):
        L = _lib.load()
        self.n = int(n)
        self._x = np.ascontiguousarray(x, dtype=np.uint64)
        self._z = np.ascontiguousarray(z, dtype=np.uint64)
        self._ph = np.ascontiguousarray(phase, dtype=np.uint8)
        self._c = np.ascontiguousarray(coeffs, dtype=np.complex128)
        T = len(self._x)
        if not (len(self._z) == len(self._ph) == len(self._c) == T):
            raise ValueError("term arrays differ in length")
        h = C.c_void_p()
        check(L.qr_op_create(self.n, T, self._x.ctypes.data, self._z.ctypes.data,
                             self._ph.ctypes.data, self._c.ctypes.data, C.byref(h)))
        self._h = h
        self.nterms = T

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().qr_op_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def info(self) -> dict:
        inf = _lib.OpInfo()
        check(_lib.load().qr_op_get_info(self._h, C.byref(inf)))
        return {f: getattr(inf, f) for f, _ in inf._fields_}

    def groups(self) -> dict:
        """The term grouping made on the device at creation: ``gx`` (distinct
        x, ascending), ``goff`` (group offsets into ``order``), ``order``
        (input index of each term, stably sorted by x) and ``mmap`` (merged
        (x, z) string of each input term, first-occurrence numbering)."""
        L = _lib.load()
        ng = C.c_uint64()
        check(L.qr_op_get_groups(self._h, C.byref(ng), None, None, None, None))
        G, T = ng.value, self.nterms
        gx = np.empty(G, dtype=np.uint64)
        goff = np.empty(G + 1, dtype=np.uint32)
        order = np.empty(T, dtype=np.uint32)
        mmap = np.empty(T, dtype=np.uint32)
        check(L.qr_op_get_groups(self._h, C.byref(ng), gx.ctypes.data, goff.ctypes.data,
                                 order.ctypes.data, mmap.ctypes.data))
        return {"gx": gx, "goff": goff, "order": order, "mmap": mmap}

    def csr_size(self):
        nr, nz = C.c_uint64(), C.c_uint64()
        check(_lib.load().qr_csr_size(self._h, C.byref(nr), C.byref(nz)))
        return nr.value, nz.value

    def csr_host(self):
        """(indptr u64, indices u64, data c128) numpy arrays built on the GPU."""
        nr, nz = self.csr_size()
        indptr = np.empty(nr + 1, dtype=np.uint64)
        indices = np.empty(nz, dtype=np.uint64)
        data = np.empty(nz, dtype=np.complex128)
        check(_lib.load().qr_csr_build(self._h, indptr.ctypes.data, indices.ctypes.data,
                                       data.ctypes.data, QR_MEM_HOST, None))
        return indptr, indices, data

    def csr_device(self, stream=None):
        """(indptr, indices, data) as torch CUDA tensors (data complex128)."""
        import torch
        nr, nz = self.csr_size()
        dev = torch.device("cuda", torch.cuda.current_device())
        indptr = torch.empty(nr + 1, dtype=torch.int64, device=dev)
        indices = torch.empty(nz, dtype=torch.int64, device=dev)
        data = torch.empty(nz, dtype=torch.complex128, device=dev)
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(_lib.load().qr_csr_build(self._h, indptr.data_ptr(), indices.data_ptr(),
                                       data.data_ptr(), _lib.QR_MEM_DEVICE, st))
        return indptr, indices, data

    def apply(self, psi, out=None, adjoint: bool = False, stream=None):
        """y = H psi (or H^dagger psi) on the GPU.

        torch CUDA tensor in (complex64 -> compensated c64 kernel, complex128
        -> plain c128 kernel), shape (2^n,) or (S, 2^n): asynchronous on the
        current stream, returns a tensor.  numpy array in: copies to the
        device, applies, copies back (synchronous), returns numpy."""
        N = 1 << self.n
        if isinstance(psi, np.ndarray):
            if psi.dtype == np.complex64:
                dt = QR_C64C
            elif psi.dtype == np.complex128:
                dt = QR_C128
            else:
                raise TypeError("psi must be complex64 or complex128")
            p = np.ascontiguousarray(psi)
            if p.size % N:
                raise ValueError("psi length %d is not a multiple of 2^n=%d" % (p.size, N))
            y = np.empty_like(p) if out is None else out
            check(_lib.load().qr_apply_host(self._h, dt, p.ctypes.data, y.ctypes.data,
                                            p.size // N, int(bool(adjoint))))
            return y
        import torch
        if not (isinstance(psi, torch.Tensor) and psi.is_cuda):
            raise TypeError("psi must be a numpy array or a CUDA torch tensor")
        if psi.dtype == torch.complex64:
            dt = QR_C64C
        elif psi.dtype == torch.complex128:
            dt = QR_C128
        else:
            raise TypeError("psi must be complex64 or complex128")
        p = psi.contiguous()
        if p.numel() % N:
            raise ValueError("psi length %d is not a multiple of 2^n=%d" % (p.numel(), N))
        y = torch.empty_like(p) if out is None else out
        st = stream if stream is not None else torch.cuda.current_stream(p.device).cuda_stream
        check(_lib.load().qr_apply(self._h, dt, p.data_ptr(), y.data_ptr(), p.numel() // N,
                                   int(bool(adjoint)), st))
        return y

    def set_coeffs(self, coeffs):
        """Replace the coefficients (same terms); plans are rebuilt lazily."""
        c = np.ascontiguousarray(coeffs, dtype=np.complex128)
        if c.shape != (self.nterms,):
            raise ValueError("expected %d coefficients" % self.nterms)
        check(_lib.load().qr_op_set_coeffs(self._h, c.ctypes.data))
        self._c = c

    def set_coeffs_device(self, coeffs, stream=None):
        """Replace the coefficients from a CUDA tensor (T values, real or
        complex) without a host synchronisation: kernels on ``stream`` (the
        current stream by default) rebuild every built plan's coefficient
        tables in place (``qr_op_set_coeffs_device``)."""
        import torch
        if not (isinstance(coeffs, torch.Tensor) and coeffs.is_cuda):
            raise TypeError("coeffs must be a CUDA tensor")
        if coeffs.numel() != self.nterms:
            raise ValueError("expected %d coefficients" % self.nterms)
        c = coeffs.detach().reshape(-1)
        if c.is_complex():
            c = c.to(torch.complex128)
        else:
            c = torch.complex(c.to(torch.float64), torch.zeros_like(c, dtype=torch.float64))
        c = c.contiguous()
        st = stream if stream is not None else torch.cuda.current_stream(c.device).cuda_stream
        check(_lib.load().qr_op_set_coeffs_device(self._h, c.data_ptr(), st))
        self._c = None  # the host copy is no longer current
        return c

    @staticmethod
    def _dtype_of(t):
        import torch
        if t.dtype == torch.complex64:
            return QR_C64C
        if t.dtype == torch.complex128:
            return QR_C128
        raise TypeError("states must be complex64 or complex128")

    def expect(self, psi):
        """<psi|H|psi> per state (FP64 reduction), complex128 CUDA tensor."""
        import torch
        N = 1 << self.n
        p = psi.contiguous()
        ns = p.numel() // N
        out = torch.empty(ns, dtype=torch.complex128, device=p.device)
        st = torch.cuda.current_stream(p.device).cuda_stream
        check(_lib.load().qr_expect(self._h, self._dtype_of(p), p.data_ptr(), ns,
                                    out.data_ptr(), st))
        return out

    def term_grad(self, psi, g):
        """sum_s <P_k psi_s, g_s> for every input term k (complex128 tensor)."""
        import torch
        N = 1 << self.n
        p, gg = psi.contiguous(), g.contiguous()
        if p.dtype != gg.dtype or p.shape != gg.shape:
            raise ValueError("psi and g must have the same dtype and shape")
        ns = p.numel() // N
        out = torch.empty(self.nterms, dtype=torch.complex128, device=p.device)
        st = torch.cuda.current_stream(p.device).cuda_stream
        check(_lib.load().qr_term_grad(self._h, self._dtype_of(p), p.data_ptr(), gg.data_ptr(),
                                       ns, out.data_ptr(), st))
        return out

    def apply_axpby(self, psi, v, alpha=1.0, beta=0.0, out=None):
        """alpha * (H psi) + beta * v in one kernel (CUDA tensors of one dtype;
        v may be ``out``).  Equals ``axpby(alpha, H.apply(psi), beta, v)``
        bit for bit."""
        import torch
        N = 1 << self.n
        p, vv = psi.contiguous(), v.contiguous()
        if p.dtype != vv.dtype or p.numel() != vv.numel():
            raise ValueError("psi and v must have the same dtype and size")
        y = torch.empty_like(p) if out is None else out
        st = torch.cuda.current_stream(p.device).cuda_stream
        check(_lib.load().qr_apply_axpby(self._h, self._dtype_of(p), _scalar2(alpha), p.data_ptr(),
                                         _scalar2(beta), vv.data_ptr(), y.data_ptr(),
                                         p.numel() // N, st))
        return y

    def diagonal(self, dtype=None, device=None):
        """Diagonal of H (2^n entries) without building the CSR: for
        complex128 equal bit for bit to the diagonal of ``csr_device()``."""
        import torch
        dtype = torch.complex128 if dtype is None else dtype
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
        out = torch.empty(1 << self.n, dtype=dtype, device=dev)
        st = torch.cuda.current_stream(out.device).cuda_stream
        check(_lib.load().qr_op_diagonal(self._h, self._dtype_of(out), out.data_ptr(), st))
        return out

    def sync_check(self, stream=None):
        import torch
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(_lib.load().qr_check(self._h, st))

    def set_test_hooks(self, force_wide=False, wait_ns=0, withhold_step=-1):
        """Test-only knobs of ``qr_op_set_test_hooks``: 64-bit row-word
        kernels at any n, a shorter mbarrier wait bound, and a ring step whose
        partner copy CTA 0 never issues.  Defaults restore normal operation."""
        flags = _lib.QR_TEST_FORCE_WIDE if force_wide else 0
        check(_lib.load().qr_op_set_test_hooks(self._h, flags, int(wait_ns), int(withhold_step)))


def _letters_masks(paulis):
    x = np.fromiter((p.x_indices() for p in paulis), dtype=np.uint64, count=len(paulis))
    z = np.fromiter((p.z_indices() for p in paulis), dtype=np.uint64, count=len(paulis))
    return x, z


class SparsePauliOp:
    """Sum of (Pauli, coeff) pairs in insertion order
    (qrusty/src/lib.rs:345-376, pyqrusty/src/lib.rs:305-433).
    Duplicate strings are not merged."""

    def __init__(self, paulis, coeffs):
        paulis = list(paulis)
        coeffs = [complex(c) for c in coeffs]
        if len(paulis) != len(coeffs):
            raise Exception("SparsePauliOp::new: paulis and coeffs must have same length")
        if len(paulis) == 0:
            raise Exception("SparsePauliOp::new: at least one pauli must be supplied")
        nq = paulis[0].num_qubits()
        if any(p.num_qubits() != nq for p in paulis):
            raise Exception("SparsePauliOp::new: all supplied paulis must have the same #qubits")
        self._paulis = paulis
        self._coeffs = coeffs
        self._ops = {}

    @classmethod
    def from_labels(cls, labels, coeffs):
        return cls([Pauli(l) for l in labels], coeffs)

    def __len__(self) -> int:
        return len(self._paulis)

    def __getitem__(self, idx):
        if isinstance(idx, slice):
            start, stop, step = idx.indices(len(self._paulis))
            return [(self._paulis[i], self._coeffs[i]) for i in range(start, stop, step)]
        idx = int(idx)
        if not (0 <= idx < len(self._paulis)):
            raise Exception("__getitem__ called on invalid index %d" % idx)
        return (self._paulis[idx], self._coeffs[idx])

    def num_qubits(self) -> int:
        return self._paulis[0].num_qubits()

    def __repr__(self) -> str:
        labels = "','".join(p.label() for p in self._paulis)
        coeffs = ", ".join(_complex_to_string(c) for c in self._coeffs)
        return "SparsePauliOp('%s', [%s])" % (labels, coeffs)

    __str__ = __repr__

    def __add__(self, other: "SparsePauliOp") -> "SparsePauliOp":
        return SparsePauliOp(self._paulis + other._paulis, self._coeffs + other._coeffs)

    # -- GPU operator for one phase convention
    def operator(self, convention: str = "rowwise") -> PauliOperator:
        op = self._ops.get(convention)
        if op is None:
            x, z = _letters_masks(self._paulis)
            ph = np.fromiter((p.phase() for p in self._paulis), dtype=np.uint8,
                             count=len(self._paulis))
            if convention == "kron":
                bp = np.fromiter((p.base_phase() for p in self._paulis), dtype=np.uint8,
                                 count=len(self._paulis))
                ph = ((ph.astype(np.int64) + 2 * bp) % 4).astype(np.uint8)
            elif convention != "rowwise":
                raise ValueError("convention must be 'rowwise' or 'kron'")
            op = PauliOperator(self.num_qubits(), x, z, ph, np.array(self._coeffs))
            self._ops[convention] = op
        return op

    def to_matrix(self) -> "SpMat":
        """Kron-convention matrix (qrusty/src/lib.rs:401-412), built on the GPU."""
        return SpMat._from_op(self.operator("kron"))

    def to_matrix_mode(self, mode: str = "") -> "SpMat":
        """pyqrusty/src/lib.rs:406-415.  "" -> to_matrix(); every AccelMode
        builds the CSR on the GPU (no CPU path)."""
        if mode == "":
            return self.to_matrix()
        try:
            name, _step = parse_mode(mode)
        except ValueError:
            raise Exception("to_matrix_mode: unrecognized mode %s" % mode) from None
        conv = "kron" if name in _KRON_MODES else "rowwise"
        return SpMat._from_op(self.operator(conv))

    # pyqrusty/src/lib.rs:382-404 (qrusty/src/lib.rs:401-524): the same
    # matrix through the named builders, all built on the GPU
    def to_matrix_binary(self) -> "SpMat":
        return self.to_matrix_mode("Binary")

    def to_matrix_accel(self) -> "SpMat":
        return self.to_matrix_mode("Accel")

    def to_matrix_reduce(self) -> "SpMat":
        return self.to_matrix_mode("Reduce")

    def to_matrix_rayon(self) -> "SpMat":
        return self.to_matrix_mode("Rayon")

    def to_matrix_rayon_chunked(self, step: int) -> "SpMat":
        return self.to_matrix_mode("RayonChunked/%d" % int(step))

    def apply(self, psi, out=None, adjoint: bool = False):
        """Matrix-free y = H psi on the GPU (rowwise convention); see
        PauliOperator.apply."""
        return self.operator("rowwise").apply(psi, out=out, adjoint=adjoint)


class SpMat:
    """CSR matrix holder (pyqrusty/src/lib.rs:33-214): complex128 data,
    u64 indices/indptr.  ``export`` moves the arrays out and leaves the
    matrix empty, after which other methods raise as the reference does."""

    def __init__(self, shape, data, indices, indptr):
        self._it = (tuple(int(s) for s in shape), np.ascontiguousarray(data, dtype=np.complex128),
                    np.ascontiguousarray(indices, dtype=np.uint64),
                    np.ascontiguousarray(indptr, dtype=np.uint64))
        self._dev = None

    @classmethod
    def _from_op(cls, op: PauliOperator) -> "SpMat":
        indptr, indices, data = op.csr_host()
        N = 1 << op.n
        return cls((N, N), data, indices, indptr)

    @staticmethod
    def new_unchecked(shape, data, indices, indptr) -> "SpMat":
        return SpMat(shape, data, indices, indptr)

    def _get(self, msg):
        if self._it is None:
            raise Exception(msg)
        return self._it

    def shape(self):
        return self._get("SpMat.shape(): matrix is already dropped")[0]

    def nnz(self) -> int:
        return len(self._get("cannot get NNZ of an exported sparse matrix")[1])

    def diagonal(self):
        """Stored diagonal, 0 where a row has none (pyqrusty/src/lib.rs:118-125),
        extracted on the GPU (qr_csr_diagonal).  numpy complex128."""
        shape = self._get("SpMat.diagonal(): already-exported sparse matrix")[0]
        return _spmat_diag_device(self).cpu().numpy()

    def __repr__(self) -> str:
        if self._it is None:
            return "<already-dropped sparse matrix of type Complex64>"
        (rows, cols), data = self._it[0], self._it[1]
        return ("<%dx%d sparse matrix of type Complex64\n\twith %d stored elements in "
                "Compressed Sparse Row format>" % (rows, cols, len(data)))

    __str__ = __repr__

    def __copy__(self) -> "SpMat":
        m = SpMat.__new__(SpMat)
        m._it = None if self._it is None else (self._it[0], self._it[1].copy(),
                                               self._it[2].copy(), self._it[3].copy())
        m._dev = None
        return m

    def export(self):
        if self._it is None:
            raise Exception("cannot export from an already-exported sparse matrix")
        shape, data, indices, indptr = self._it
        self._it = None
        self._dev = None
        return (shape, data, indices, indptr)

    def export_device(self):
        """``export`` into CUDA tensors: ((rows, cols), data complex128,
        indices int64, indptr int64) on the current device, reusing the device
        copy a GPU call already made; the SpMat is left empty."""
        if self._it is None:
            raise Exception("cannot export from an already-exported sparse matrix")
        shape = self._it[0]
        indptr, indices, data = self._device()
        self._it = None
        self._dev = None
        return (shape, data, indices, indptr)

    # ------------------------------------------------------------ file formats
    def matrixmarket_write(self, save_path: str) -> None:
        """MatrixMarket coordinate complex general (pyqrusty/src/lib.rs:216-229);
        ".gz" paths are gzip-compressed."""
        self._mm_write(save_path, 0)

    _SYM_MODES = {"": 0, "general": 0, "symmetric": 1, "skew-symmetric": 2, "hermitian": 3}

    def matrixmarket_write_symmetric(self, save_path: str, mode: str = "general") -> None:
        """Symmetric-storage MatrixMarket (pyqrusty/src/lib.rs:248-260): the
        lower triangle under a symmetric / skew-symmetric / hermitian header."""
        if mode not in self._SYM_MODES:
            raise Exception("matrixmarket_write_symmetric: unrecognized mode %s" % mode)
        self._mm_write(save_path, self._SYM_MODES[mode])

    def _mm_write(self, path, sym):
        shape, data, indices, indptr = self._get(
            "cannot write an already-destroyed sparse matrix")
        check(_lib.load().qr_mm_write(str(path).encode(), shape[0], shape[1], indptr.ctypes.data,
                                      indices.ctypes.data, data.ctypes.data, sym,
                                      _lib.QR_MEM_HOST, None))

    @staticmethod
    def matrixmarket_read(read_path: str) -> "SpMat":
        """MatrixMarket coordinate file (any field, any symmetry; ".gz"
        accepted) to CSR (pyqrusty/src/lib.rs:231-246)."""
        L = _lib.load()
        h = C.c_void_p()
        nr, nc, nz = C.c_uint64(), C.c_uint64(), C.c_uint64()
        rc = L.qr_mm_open(str(read_path).encode(), C.byref(h), C.byref(nr), C.byref(nc),
                          C.byref(nz))
        if rc != 0:
            raise Exception(_lib.last_error())
        try:
            indptr = np.empty(nr.value + 1, dtype=np.uint64)
            indices = np.empty(nz.value, dtype=np.uint64)
            data = np.empty(nz.value, dtype=np.complex128)
            check(L.qr_mm_fetch(h, indptr.ctypes.data, indices.ctypes.data, data.ctypes.data,
                                _lib.QR_MEM_HOST, None))
        finally:
            L.qr_mm_close(h)
        return SpMat((nr.value, nc.value), data, indices, indptr)

    def rawio_write(self, save_path: str) -> None:
        """qrusty's binary CSR file (qrusty/src/rawio.rs:128-149)."""
        shape, data, indices, indptr = self._get(
            "cannot write an already-destroyed sparse matrix")
        check(_lib.load().qr_rawio_write(str(save_path).encode(), 0, shape[0], shape[1],
                                         indptr.ctypes.data, len(indptr), indices.ctypes.data,
                                         data.ctypes.data, len(data), _lib.QR_MEM_HOST, None))

    @staticmethod
    def rawio_read(read_path: str) -> "SpMat":
        """Read qrusty's binary CSR file (qrusty/src/rawio.rs:151-179),
        either byte order."""
        L = _lib.load()
        info = _lib.CsrFileInfo()
        check(L.qr_rawio_info(str(read_path).encode(), C.byref(info)))
        if info.storage != 0:
            raise Exception("rawio_read: CSC storage is not a SpMat")
        indptr = np.empty(info.indptr_len, dtype=np.uint64)
        indices = np.empty(info.nnz, dtype=np.uint64)
        data = np.empty(info.nnz, dtype=np.complex128)
        check(L.qr_rawio_read(str(read_path).encode(), indptr.ctypes.data, indices.ctypes.data,
                              data.ctypes.data, _lib.QR_MEM_HOST, None))
        return SpMat((info.nrows, info.ncols), data, indices, indptr)

    def _device(self):
        import torch
        shape, data, indices, indptr = self._get(
            "cannot multiply with an exported sparse matrix")
        if self._dev is None:
            dev = torch.device("cuda", torch.cuda.current_device())
            self._dev = (torch.from_numpy(indptr.view(np.int64)).to(dev),
                         torch.from_numpy(indices.view(np.int64)).to(dev),
                         torch.from_numpy(data).to(dev))
        return self._dev


def spmat_dot_densevec(spmat: SpMat, x):
    """y = spmat * x on the GPU (pyqrusty/src/lib.rs:476-491,
    qrusty/src/accel.rs:338-370).  numpy complex128 in and out."""
    import torch
    if spmat._it is None:
        raise Exception("cannot multiply with an exported sparse matrix")
    shape = spmat._it[0]
    xv = np.ascontiguousarray(np.asarray(x, dtype=np.complex128))
    if xv.ndim != 1 or xv.shape[0] != shape[1]:
        raise Exception("spmat_dot_densevec: vector length %d != %d columns"
                        % (xv.shape[0] if xv.ndim else 0, shape[1]))
    ip_h, data_h = spmat._it[3], spmat._it[1]
    if len(ip_h) != shape[0] + 1 or int(ip_h[-1]) != len(data_h) or \
            np.any(np.diff(ip_h.astype(np.int64)) < 0):
        raise Exception("spmat_dot_densevec: malformed CSR row pointers")
    indptr, indices, data = spmat._device()
    dev = data.device
    xd = torch.from_numpy(xv).to(dev)
    yd = torch.empty(shape[0], dtype=torch.complex128, device=dev)
    st = torch.cuda.current_stream(dev).cuda_stream
    check(_lib.load().qr_csr_spmv(shape[0], shape[1], indptr.data_ptr(), indices.data_ptr(),
                                  data.data_ptr(), xd.data_ptr(), yd.data_ptr(), st))
    return yd.cpu().numpy()


def _spmat_diag_device(spmat: "SpMat"):
    import torch
    shape = spmat._it[0]
    indptr, indices, data = spmat._device()
    nd = min(shape)
    out = torch.empty(nd, dtype=torch.complex128, device=data.device)
    st = torch.cuda.current_stream(data.device).cuda_stream
    check(_lib.load().qr_csr_diagonal(shape[0], shape[1], indptr.data_ptr(), indices.data_ptr(),
                                      data.data_ptr(), out.data_ptr(), st))
    return out


def _vec_operand(v, name):
    """(CUDA tensor, came-from-numpy) for a 1-D complex vector argument."""
    import torch
    if isinstance(v, torch.Tensor):
        if not v.is_cuda:
            raise TypeError("%s: tensors must be on a CUDA device" % name)
        if v.dtype not in (torch.complex64, torch.complex128):
            raise TypeError("%s: tensors must be complex64 or complex128" % name)
        return v.contiguous(), False
    a = np.ascontiguousarray(np.asarray(v, dtype=np.complex128))
    if a.ndim != 1:
        raise ValueError("%s: expected a 1-D array" % name)
    return torch.from_numpy(a).to("cuda"), True


def _scalar2(c):
    c = complex(c)
    return (C.c_double * 2)(c.real, c.imag)


def _vec_call(name, fn, a, x, y=None, b=None, tol=None):
    import torch
    xd, host = _vec_operand(x, name)
    yd = None
    if y is not None:
        yd, yhost = _vec_operand(y, name)
        host = host and yhost
        if yd.dtype != xd.dtype or yd.device != xd.device:
            yd = yd.to(device=xd.device, dtype=xd.dtype)
        if yd.numel() != xd.numel():
            raise Exception("%s: vectors of different lengths (%d, %d)"
                            % (name, xd.numel(), yd.numel()))
    z = torch.empty_like(xd)
    dt = QR_C64C if xd.dtype == torch.complex64 else QR_C128
    st = torch.cuda.current_stream(xd.device).cuda_stream
    L = _lib.load()
    if fn == "axpby":
        check(L.qr_axpby(dt, xd.numel(), _scalar2(a), xd.data_ptr(), _scalar2(b), yd.data_ptr(),
                         z.data_ptr(), st))
    elif fn == "axpy":
        check(L.qr_axpy(dt, xd.numel(), _scalar2(a), xd.data_ptr(), yd.data_ptr(), z.data_ptr(),
                        st))
    elif fn == "ax":
        check(L.qr_ax(dt, xd.numel(), _scalar2(a), xd.data_ptr(), z.data_ptr(), st))
    else:  # precond2: x = diag, y = dx, a = e
        check(L.qr_precond2(dt, xd.numel(), xd.data_ptr(), yd.data_ptr(), _scalar2(a),
                            float(tol), z.data_ptr(), st))
    return z.cpu().numpy() if host else z


def axpby(a, x, b, y):
    """a*x + b*y element-wise (qrusty/src/accel.rs:374-379).  numpy in ->
    numpy out (complex128); CUDA tensors in -> tensor out, same dtype."""
    return _vec_call("axpby", "axpby", a, x, y=y, b=b)


def axpy(a, x, y):
    """a*x + y element-wise (qrusty/src/accel.rs:381-386)."""
    return _vec_call("axpy", "axpy", a, x, y=y)


def ax(a, x):
    """a*x element-wise (qrusty/src/accel.rs:388-393)."""
    return _vec_call("ax", "ax", a, x)


def precond2(diag, dx, e, tol):
    """dx / reg(diag - e, tol), reg(v) = tol where |v| < tol
    (pyqrusty/src/lib.rs:436-440, 457-469)."""
    return _vec_call("precond2", "precond2", e, diag, y=dx, tol=tol)


def precond(spmat: "SpMat", dx, e, tol):
    """precond2 with the matrix's stored diagonal (pyqrusty/src/lib.rs:442-455,
    binding :563-577)."""
    if spmat._it is None:
        raise Exception("cannot call precond with an exported sparse matrix")
    d = _spmat_diag_device(spmat)
    dxd, host = _vec_operand(dx, "precond")
    if dxd.numel() != d.numel():
        raise Exception("precond: vector length %d != diagonal length %d"
                        % (dxd.numel(), d.numel()))
    out = _vec_call("precond", "precond2", e, d.to(dxd.dtype), y=dxd, tol=tol)
    return out.cpu().numpy() if host else out


class Batch:
    """Many operators, each with its own complex64 states, applied in ONE
    persistent kernel launch replayed from a CUDA graph (qr_batch_*).  The
    first ``apply`` autotunes the amplitude-tile width on the given buffers."""

    def __init__(self, ops, nstates):
        self.ops = list(ops)
        self.nstates = [int(s) for s in nstates]
        if len(self.ops) != len(self.nstates) or not self.ops:
            raise ValueError("ops and nstates must be non-empty and of equal length")
        n = len(self.ops)
        hs = (C.c_void_p * n)(*[op.handle.value for op in self.ops])
        ns = (C.c_int32 * n)(*self.nstates)
        h = C.c_void_p()
        check(_lib.load().qr_batch_create(n, hs, ns, C.byref(h)))
        self._h = h

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().qr_batch_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def mode(self) -> int:
        """0: one persistent work-list kernel, 1: graph of per-operator
        kernels, 2: both (the persistent kernel for the small operators);
        chosen by timing on the first apply; -1 before it."""
        return int(_lib.load().qr_batch_mode(self._h))

    def set_mode(self, mode: int) -> None:
        """Fix the mode instead of timing (before the first apply)."""
        check(_lib.load().qr_batch_set_mode(self._h, int(mode)))

    @property
    def tile_bits(self) -> int:
        return int(_lib.load().qr_batch_tile_bits(self._h))

    def apply(self, psis, ys, stream=None):
        """psis[i], ys[i]: CUDA complex64 tensors of nstates[i] x 2^n_i amplitudes."""
        import torch
        n = len(self.ops)
        if len(psis) != n or len(ys) != n:
            raise ValueError("one psi and one y per operator")
        for i, (p, y) in enumerate(zip(psis, ys)):
            want = self.nstates[i] << self.ops[i].n
            for tns in (p, y):
                if tns.dtype != torch.complex64 or not tns.is_cuda or not tns.is_contiguous():
                    raise TypeError("batched states must be contiguous CUDA complex64 tensors")
                if tns.numel() != want:
                    raise ValueError("operator %d expects %d amplitudes" % (i, want))
        pp = (C.c_void_p * n)(*[p.data_ptr() for p in psis])
        yy = (C.c_void_p * n)(*[y.data_ptr() for y in ys])
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(_lib.load().qr_batch_apply(self._h, pp, yy, st))
        return ys


def vdot(a, b):
    """<a_s, b_s> per state in FP64 for CUDA tensors of 2^n (or S x 2^n)
    complex64 / complex128 amplitudes; complex128 tensor of S values."""
    import torch
    if a.dtype != b.dtype or a.shape != b.shape:
        raise ValueError("a and b must have the same dtype and shape")
    N = a.shape[-1]
    n = N.bit_length() - 1
    if N != 1 << n:
        raise ValueError("last dimension must be a power of two")
    ns = a.numel() // N
    out = torch.empty(ns, dtype=torch.complex128, device=a.device)
    st = torch.cuda.current_stream(a.device).cuda_stream
    check(_lib.load().qr_vdot(n, PauliOperator._dtype_of(a), a.contiguous().data_ptr(),
                              b.contiguous().data_ptr(), ns, out.data_ptr(), st))
    return out


def csr_matrix(m: SpMat):
    """pyqrusty/python/pyqrusty/__init__.py:14-17."""
    (shape, data, indices, indptr) = m.export()
    from scipy.sparse import csr_matrix as _csr
    return _csr((data, indices, indptr), shape=shape, dtype=complex)
