"""``pyqrusty``: qrusty's Python import name, served by qrusty_gb300.

qrusty's pyo3 package exposes these names (pyqrusty/python/pyqrusty/
__init__.py:11-17 of the qrusty repository); code written against it --
including qrusty's own tests of this path, pyqrusty/tests/test_H.py and the
CSR / SpMV / vector-helper / file-format tests of test_it.py -- runs
unchanged with ``from pyqrusty import *``, every CSR build and product on
the GPU.  SpMat algebra (``+``, ``-``, ``scale``, ``a_spmat_p_b_spmat``,
zero counting) is outside this path and not provided.
"""
from qrusty_gb300.pyqrusty import (Pauli, SparsePauliOp, SpMat, ax, axpby, axpy, csr_matrix,
                                   precond, precond2, spmat_dot_densevec)

__all__ = ["Pauli", "SparsePauliOp", "SpMat", "spmat_dot_densevec", "axpby", "axpy", "ax",
           "precond", "precond2", "csr_matrix"]
