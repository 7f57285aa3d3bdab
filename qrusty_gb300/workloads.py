"""Seeded synthetic operators and states for the benchmark workloads.

No public dataset is involved: every workload is drawn from
``numpy.random.default_rng(20260 + k)`` in the draw order documented per
function, so tests, the CPU baseline and the GPU benchmark see identical
inputs.  Operators are returned as term arrays (x, z, phase, coeff) in the
convention of qrusty's make_params (qrusty/src/accel.rs:141-157).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SEED0 = 20260
LETTER_P = (0.55, 0.15, 0.15, 0.15)  # I, X, Y, Z


@dataclass
class Terms:
    n: int
    x: np.ndarray       # uint64
    z: np.ndarray       # uint64
    phase: np.ndarray   # uint8
    coeff: np.ndarray   # complex128
    name: str = ""

    @property
    def T(self) -> int:
        return len(self.x)

    def labels(self):
        """Pauli labels (qubit 0 rightmost), e.g. for SparsePauliOp."""
        out = []
        for xk, zk in zip(self.x.tolist(), self.z.tolist()):
            s = []
            for q in range(self.n):
                xb, zb = (xk >> q) & 1, (zk >> q) & 1
                s.append("IXZY"[xb + 2 * zb])
            out.append("".join(reversed(s)))
        return out


def terms_from_letters(letters: np.ndarray, coeff) -> Terms:
    """letters: (T, n) ints 0..3 = I, X, Y, Z with column q = qubit q."""
    T, n = letters.shape
    w = (np.uint64(1) << np.arange(n, dtype=np.uint64))
    xm = ((letters == 1) | (letters == 2)).astype(np.uint64)
    zm = ((letters == 2) | (letters == 3)).astype(np.uint64)
    x = (xm * w).sum(axis=1, dtype=np.uint64)
    z = (zm * w).sum(axis=1, dtype=np.uint64)
    phase = ((letters == 2).sum(axis=1) % 4).astype(np.uint8)
    return Terms(n, x, z, phase, np.asarray(coeff, dtype=np.complex128))


def terms_from_labels(labels, coeffs) -> Terms:
    """Plain labels (no sign / i prefix) to term arrays."""
    n = len(labels[0])
    code = {"I": 0, "X": 1, "Y": 2, "Z": 3}
    letters = np.array([[code[c] for c in reversed(l)] for l in labels], dtype=np.int64)
    t = terms_from_letters(letters, coeffs)
    t.n = n
    return t


def random_state(rng, N: int, dtype=np.complex128, nstates: int = 1) -> np.ndarray:
    """Unit-norm state(s): re, im ~ N(0, 1) drawn in that order, normalised."""
    re = rng.standard_normal((nstates, N))
    im = rng.standard_normal((nstates, N))
    psi = re + 1j * im
    psi /= np.linalg.norm(psi, axis=1, keepdims=True)
    psi = psi.astype(dtype)
    return psi[0] if nstates == 1 else psi


def random_letters_op(rng, n: int, T: int, real_coeff=True) -> Terms:
    """Letters i.i.d. from {I,X,Y,Z} with P = (0.55, 0.15, 0.15, 0.15);
    coefficients ~ N(0, 1) real.  Draw order: letters, then coefficients."""
    letters = rng.choice(4, size=(T, n), p=LETTER_P)
    c = rng.standard_normal(T)
    return terms_from_letters(letters, c.astype(np.complex128))


def cfg0(with_state=True):
    """n=12, 200 terms of random letters, one c128 unit-norm state."""
    rng = np.random.default_rng(SEED0 + 0)
    t = random_letters_op(rng, 12, 200)
    t.name = "cfg0: n=12, 200 random-letter terms"
    psi = random_state(rng, 1 << 12) if with_state else None
    return t, psi


def chain_op(n: int, rng) -> Terms:
    """Open 1-D TFIM + XXZ chain: for i < n-1, Z_iZ_{i+1}, X_iX_{i+1},
    Y_iY_{i+1} with J ~ U[0.5, 1.5] each (drawn zz, xx, yy per bond), then
    X_i with h ~ U[0, 2] for every site."""
    xs, zs, ph, cs = [], [], [], []
    for i in range(n - 1):
        J = rng.uniform(0.5, 1.5, 3)
        b = (1 << i) | (1 << (i + 1))
        xs += [0, b, b]
        zs += [b, 0, b]
        ph += [0, 0, 2]  # two Y letters: phase 2
        cs += list(J)
    h = rng.uniform(0.0, 2.0, n)
    for i in range(n):
        xs.append(1 << i)
        zs.append(0)
        ph.append(0)
        cs.append(h[i])
    return Terms(n, np.array(xs, dtype=np.uint64), np.array(zs, dtype=np.uint64),
                 np.array(ph, dtype=np.uint8), np.array(cs, dtype=np.complex128))


def cfg1(with_state=True, n=22):
    rng = np.random.default_rng(SEED0 + 1)
    t = chain_op(n, rng)
    t.name = "cfg1: n=%d TFIM+XXZ open chain, %d terms" % (n, t.T)
    psi = random_state(rng, 1 << n) if with_state else None
    return t, psi


def jw_op(n: int, npair: int, nz: int, rng, sigma=0.1) -> Terms:
    """Jordan-Wigner-style operator: npair terms each with a random pair
    i < j (X or Y at i and at j, Z on every qubit strictly between), then nz
    pure-Z terms on 1-4 random distinct qubits; coefficients ~ N(0, sigma)
    real.  Draw order per pair term: the pair, letter at i, letter at j;
    then per Z term: its size, its qubits; then all coefficients."""
    xs, zs, ph = [], [], []
    for _ in range(npair):
        i, j = sorted(int(v) for v in rng.choice(n, 2, replace=False))
        a = int(rng.integers(2))  # 0: X, 1: Y at i
        b = int(rng.integers(2))  # at j
        x = (1 << i) | (1 << j)
        z = ((1 << j) - (1 << (i + 1))) if j > i + 1 else 0  # Z strictly between
        if a:
            z |= 1 << i
        if b:
            z |= 1 << j
        xs.append(x)
        zs.append(z)
        ph.append((a + b) % 4)
    for _ in range(nz):
        k = int(rng.integers(1, 5))
        qs = rng.choice(n, k, replace=False)
        z = 0
        for q in qs:
            z |= 1 << int(q)
        xs.append(0)
        zs.append(z)
        ph.append(0)
    c = rng.normal(0.0, sigma, npair + nz)
    return Terms(n, np.array(xs, dtype=np.uint64), np.array(zs, dtype=np.uint64),
                 np.array(ph, dtype=np.uint8), c.astype(np.complex128))


def cfg2(n=26, npair=8000, nz=2000):
    """n=26, 8,000 pair terms + 2,000 pure-Z terms, sigma = 0.1 (no state:
    states at this size are drawn on the device by the caller)."""
    rng = np.random.default_rng(SEED0 + 2)
    t = jw_op(n, npair, nz, rng)
    t.name = "cfg2: n=%d Jordan-Wigner-style, %d terms" % (n, t.T)
    return t


def cfg3(nops=256, nstates=8, nmin=10, nmax=20, tmin=50, tmax=5000):
    """Uneven batch: per operator n ~ U{nmin..nmax}, T ~ U{tmin..tmax},
    letters as cfg0 (draw order: n, T, letters, coefficients)."""
    rng = np.random.default_rng(SEED0 + 3)
    ops = []
    for _ in range(nops):
        n = int(rng.integers(nmin, nmax + 1))
        T = int(rng.integers(tmin, tmax + 1))
        ops.append(random_letters_op(rng, n, T))
    return ops


def cfg4(n=20, T=2000):
    """n=20, 2,000 random-letter terms, real c ~ N(0, 1); psi and w unit-norm."""
    rng = np.random.default_rng(SEED0 + 4)
    t = random_letters_op(rng, n, T)
    t.name = "cfg4: n=%d, %d random-letter terms" % (n, T)
    psi = random_state(rng, 1 << n)
    w = random_state(rng, 1 << n)
    return t, psi, w


def alg_blocks(t: Terms, tile_bits: int = 13) -> int:
    """P = number of distinct partner tiles x >> tile_bits (the algorithmic
    read count per output tile, besides the output write)."""
    b = min(tile_bits, t.n)
    return len(np.unique(t.x >> np.uint64(b)))
