"""Host-side logic of the pyqrusty mirror (no GPU): parsing, validation,
reprs and mode strings, following the reference's own Python tests
(pyqrusty/tests/test_it.py, test_H.py) and qrusty/src/lib.rs."""
import numpy as np
import pytest

from qrusty_gb300 import Pauli, SparsePauliOp, parse_mode
from qrusty_gb300.pyqrusty import _complex_to_string, _rust_f64


@pytest.mark.parametrize("label", ["I", "+I", "+iI", "+jI", "-1jI", "-1I", "-1jIX", "IXYZ",
                                   "-IIIIIIIIIIIIIIIIIIYXXY", "iXYZ", "-YY"])
def test_parse_matches_oracle(oracle, label):
    p = Pauli(label)
    bp, letters = oracle.parse_label(label)
    assert p.base_phase() == bp
    assert p.label() == letters[::-1]
    x, z, ph = oracle.label_masks(label)
    assert (p.x_indices(), p.z_indices(), p.phase()) == (x, z, ph)


@pytest.mark.parametrize("bad", ["W", "", "+i", "XYQ", "1-X", "ii"])
def test_parse_rejects(bad):
    with pytest.raises(Exception, match="malformed label"):
        Pauli(bad)


def test_paulis():  # test_it.py:28-32
    p = Pauli("IXYZ")
    assert p.num_qubits() == 4
    assert p.label() == "IXYZ"
    assert repr(p) == "Pauli('IXYZ')"
    assert p.xs() == [False, True, True, False]
    assert p.zs() == [True, True, False, False]


def test_spop_wrong_lengths():  # test_it.py:34-38
    with pytest.raises(Exception):
        SparsePauliOp([Pauli("I"), Pauli("IXYZ")], [1.0 + 0.0j, 1.0 + 0.0j])


def test_spop_errors():  # qrusty/src/lib.rs:354-376
    with pytest.raises(Exception, match="same length"):
        SparsePauliOp([Pauli("I")], [1.0, 2.0])
    with pytest.raises(Exception, match="at least one pauli"):
        SparsePauliOp([], [])
    with pytest.raises(Exception, match="same #qubits"):
        SparsePauliOp([Pauli("I"), Pauli("II")], [1.0, 1.0])


def test_spop_repr():  # test_it.py:40-44
    spop = SparsePauliOp([Pauli("IIII"), Pauli("IXYZ")], [1.0 + 0.0j, 1.0 + 0.0j])
    assert repr(spop) == "SparsePauliOp('IIII','IXYZ', [1+0j, 1+0j])"


def test_slice(golden):  # test_it.py:211-216
    labels, coeffs = golden["H2"]
    H2 = SparsePauliOp([Pauli(l) for l in labels], list(coeffs))
    assert repr(H2[3]) == "(Pauli('IIXX'), (-0.00170526+0j))"
    s = H2[3:8:2]
    assert repr(s) == ("[(Pauli('IIXX'), (-0.00170526+0j)), (Pauli('IZII'), (0.18388659+0j)), "
                       "(Pauli('XXII'), (-0.00170526+0j))]")
    assert len(H2) == 27
    with pytest.raises(Exception, match="invalid index"):
        H2[27]
    with pytest.raises(Exception, match="invalid index"):
        H2[-1]


def test_rust_float_display():
    assert _rust_f64(1.0) == "1"
    assert _rust_f64(0.0) == "0"
    assert _rust_f64(-0.0) == "-0"
    assert _rust_f64(-0.5) == "-0.5"
    assert _rust_f64(1e-8) == "0.00000001"
    assert _rust_f64(1e21) == "1000000000000000000000"
    assert _rust_f64(float("nan")) == "NaN"
    assert _complex_to_string(1 - 2j) == "1+-2j"


@pytest.mark.parametrize("mode,expect", [
    ("Binary", ("Binary", None)), ("Accel", ("Accel", None)), ("Rowwise", ("Rowwise", None)),
    ("RowwiseUnsafe", ("RowwiseUnsafe", None)),
    ("RowwiseUnsafeChunked/100", ("RowwiseUnsafeChunked", 100)),
    ("RowwiseUnsafeChunked/1000", ("RowwiseUnsafeChunked", 1000)),
    ("Reduce", ("Reduce", None)), ("Rayon", ("Rayon", None)),
    ("RayonChunked/7", ("RayonChunked", 7)),
])
def test_modes(mode, expect):  # qrusty/src/lib.rs:293-331
    assert parse_mode(mode) == expect


def test_mode_rejects():  # test_H.py:28-30
    for bad in ["foo", "rowwise", "RowwiseUnsafeChunked/", ""]:
        with pytest.raises(ValueError):
            parse_mode(bad)
    H = SparsePauliOp([Pauli("XY")], [1.0])
    with pytest.raises(Exception, match="unrecognized mode foo"):
        H.to_matrix_mode("foo")


def test_workload_terms_roundtrip():
    from qrusty_gb300 import workloads as W
    from tests.helpers import terms_of_labels
    t, _ = W.cfg0(with_state=False)
    n, x, z, ph, c = terms_of_labels(t.labels(), t.coeff)
    assert n == t.n
    assert np.array_equal(x, t.x) and np.array_equal(z, t.z) and np.array_equal(ph, t.phase)
    t2 = W.cfg2(n=10, npair=50, nz=20)
    n, x, z, ph, c = terms_of_labels(t2.labels(), t2.coeff)
    assert np.array_equal(x, t2.x) and np.array_equal(z, t2.z) and np.array_equal(ph, t2.phase)
