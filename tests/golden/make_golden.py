"""Generate tests/golden/hamiltonians.npz from the reference's own fixtures.

The qrusty reference keeps its molecular test Hamiltonians as Python source
(pyqrusty/tests/H_fixtures.py: ``build_spop(labels, coeffs)`` calls over
pyqrusty's ``Pauli`` / ``SparsePauliOp``).  pyqrusty itself cannot be built
here (no Rust toolchain), so this script executes the fixture file against a
recording stand-in for those two classes and stores every fixture's labels
and coefficients verbatim.  The committed .npz is what the tests read; this
script is only re-run by hand, in a checkout that has the reference:

    python tests/golden/make_golden.py /path/to/qrusty
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

KEEP = ("H2", "H4", "H6", "H8", "HJ")


def load_fixtures(ref_root: str):
    stub = types.ModuleType("pyqrusty")

    class Pauli:  # records the label only
        def __init__(self, label):
            self.label = label

    class SparsePauliOp:
        def __init__(self, paulis, coeffs):
            self.labels = [p.label for p in paulis]
            self.coeffs = list(coeffs)

    stub.Pauli = Pauli
    stub.SparsePauliOp = SparsePauliOp
    stub.__all__ = ["Pauli", "SparsePauliOp"]
    sys.modules["pyqrusty"] = stub
    path = os.path.join(ref_root, "pyqrusty", "tests", "H_fixtures.py")
    ns: dict = {"__name__": "H_fixtures"}
    with open(path) as f:
        code = compile(f.read(), path, "exec")
    exec(code, ns)
    return {k: ns[k] for k in KEEP}


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("QRUSTY_REF", "")
    if not ref_root:
        raise SystemExit("usage: make_golden.py <qrusty checkout>")
    fx = load_fixtures(ref_root)
    out = {}
    for name, op in fx.items():
        out[name + "_labels"] = np.array(op.labels)
        out[name + "_coeffs"] = np.array(op.coeffs, dtype=np.complex128)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hamiltonians.npz")
    np.savez_compressed(dst, **out)
    for name, op in fx.items():
        print(name, len(op.labels), "terms,", len(op.labels[0]), "qubits")
    print("wrote", dst)


if __name__ == "__main__":
    main()
