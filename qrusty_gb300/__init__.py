"""qrusty_gb300: GB300-native (sm_103a) Pauli-operator hot path of qrusty.

``from qrusty_gb300 import *`` gives the names of qrusty's ``pyqrusty``
package for this path (Pauli, SparsePauliOp, SpMat, spmat_dot_densevec,
csr_matrix), backed by libqrusty_gpu.so (C ABI: include/qrusty_gpu.h).
"""
from .pyqrusty import (Batch, Pauli, PauliOperator, QrError, SparsePauliOp, SpMat, ax, axpby,
                       axpy, csr_matrix, parse_mode, precond, precond2, spmat_dot_densevec, vdot)

__all__ = ["Pauli", "SparsePauliOp", "SpMat", "spmat_dot_densevec", "csr_matrix",
           "PauliOperator", "QrError", "parse_mode", "vdot", "Batch", "axpby", "axpy", "ax",
           "precond", "precond2"]
