"""Generate tests/golden/*.npz from the reference's own fixtures.

hamiltonians.npz -- the molecular test Hamiltonians (see below).
precond.npz      -- the precond known-answer vectors of
                    pyqrusty/tests/test_it.py:285-313 (tol, dx, e, rv: the
                    reference's printed result of dx / reg(H2.diag - e, tol)),
                    read from the test module's top-level assignments.

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

import ast
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


PRECOND_NAMES = ("tol", "dx", "e", "rv")


def load_precond_vectors(ref_root: str):
    """Evaluate only the top-level ``tol = / dx = / e = / rv =`` assignments of
    pyqrusty/tests/test_it.py (numpy literals), nothing else of the module."""
    path = os.path.join(ref_root, "pyqrusty", "tests", "test_it.py")
    with open(path) as f:
        tree = ast.parse(f.read(), path)
    keep = [node for node in tree.body if isinstance(node, ast.Assign)
            and len(node.targets) == 1 and isinstance(node.targets[0], ast.Name)
            and node.targets[0].id in PRECOND_NAMES]
    ns: dict = {"np": np}
    exec(compile(ast.Module(body=keep, type_ignores=[]), path, "exec"), ns)
    return {k: ns[k] for k in PRECOND_NAMES}


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
    pv = load_precond_vectors(ref_root)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "precond.npz")
    np.savez_compressed(dst, tol=np.float64(pv["tol"]), dx=np.asarray(pv["dx"], np.complex128),
                        e=np.complex128(pv["e"]), rv=np.asarray(pv["rv"], np.complex128))
    print("wrote", dst)


if __name__ == "__main__":
    main()
