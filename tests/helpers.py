"""Independent numpy restatements used by the tests as second checkers.

kron_dense restates qrusty's Kronecker path: SimplePauli::to_matrix
(qrusty/src/lib.rs:93-114), Pauli::to_matrix (lib.rs:203-213: kron of the
2x2 factors, scaled by base_coeff = i^base_phase) and SparsePauliOp::to_matrix
(lib.rs:401-412: sum = c_0 P_0, then sum = sum + c_k P_k in term order).
Every factor is +-1 or +-i, so each term's entries are exact and the term-
order sum reproduces the reference's values bit for bit (up to the sign of
zero).
"""
from __future__ import annotations

import re

import numpy as np

_LABEL_RE = re.compile(r"^([+-]?)1?([ij]?)([IXYZ]+)$")
_BASE = [1.0 + 0.0j, 1.0j, -1.0 + 0.0j, -1.0j]


def parse(label):
    m = _LABEL_RE.match(label)
    if not m:
        raise ValueError(label)
    bp = (1 if m.group(2) else 0) + (2 if m.group(1) == "-" else 0)
    return bp, m.group(3)[::-1]


def kron_dense(labels, coeffs):
    n = len(parse(labels[0])[1])
    N = 1 << n
    M = np.zeros((N, N), dtype=np.complex128)
    r = np.arange(N, dtype=np.int64)
    for lab, c in zip(labels, coeffs):
        bp, letters = parse(lab)
        val = np.full(N, _BASE[bp], dtype=np.complex128)
        x = 0
        for q, L in enumerate(letters):
            bit = (r >> q) & 1
            if L == "X":
                x |= 1 << q
            elif L == "Y":
                x |= 1 << q
                val = val * np.where(bit == 0, -1j, 1j)
            elif L == "Z":
                val = val * np.where(bit == 0, 1.0 + 0j, -1.0 + 0j)
        cols = r ^ x
        M[r, cols] = M[r, cols] + complex(c) * val
    return M


def rowwise_dense(labels, coeffs):
    """Rowwise convention: (-i)^(base + #Y) instead of i^base (-i)^#Y."""
    fixed = []
    for lab in labels:
        bp, letters = parse(lab)
        # i^bp -> (-i)^bp: flip the i prefix (base 1 <-> 3)
        nb = (4 - bp) % 4 if bp % 2 else bp
        pre = {0: "", 1: "i", 2: "-", 3: "-i"}[nb]
        fixed.append(pre + letters[::-1])
    return kron_dense(fixed, coeffs)


def csr_to_dense(indptr, indices, data, shape):
    M = np.zeros(shape, dtype=np.complex128)
    for r in range(shape[0]):
        lo, hi = int(indptr[r]), int(indptr[r + 1])
        M[r, indices[lo:hi].astype(np.int64)] += data[lo:hi]
    return M


def terms_of_labels(labels, coeffs):
    """(n, x, z, phase, coeff) arrays in make_params' convention."""
    xs, zs, ph = [], [], []
    n = None
    for lab in labels:
        bp, letters = parse(lab)
        n = len(letters)
        x = z = 0
        ny = 0
        for q, L in enumerate(letters):
            if L in "XY":
                x |= 1 << q
            if L in "YZ":
                z |= 1 << q
            ny += L == "Y"
        xs.append(x)
        zs.append(z)
        ph.append((bp + ny) % 4)
    return (n, np.array(xs, dtype=np.uint64), np.array(zs, dtype=np.uint64),
            np.array(ph, dtype=np.uint8), np.asarray(coeffs, dtype=np.complex128))


# Pure-Python restatement of the rowwise path, independent of the C oracle.
_UNIT_PHASE = [complex(1.0, 0.0), complex(0.0, -1.0), complex(-1.0, 0.0), complex(0.0, 1.0)]


def make_params_py(phase, coeffs):
    """qrusty/src/accel.rs:141-157: c'_k = m(phase_k) * c_k, m = 1, -i, -1, i,
    with num-complex's product (ac - bd, ad + bc); CPython's complex product
    is the same formula, and every factor of m is 0 or +-1, so each product
    is exact."""
    return [_UNIT_PHASE[int(p) % 4] * complex(c) for p, c in zip(phase, coeffs)]


def make_row_py(x, z, cprime, r):
    """qrusty/src/accel.rs:171-210 for row r: (r ^ x_k, +-c'_k) per term, the
    sign flipped (both parts) when popcount(r & z_k) is odd, a stable sort by
    column, then a left fold that merges equal columns by adding in term
    order starting from the first value (explicit zeros kept)."""
    v = [(r ^ xk, -ck if bin(r & zk).count("1") & 1 else ck)
         for xk, zk, ck in zip(x, z, cprime)]
    v.sort(key=lambda e: e[0])
    cols, vals = [], []
    for col, val in v:
        if cols and cols[-1] == col:
            vals[-1] = vals[-1] + val
        else:
            cols.append(col)
            vals.append(val)
    return cols, vals
