"""Differentiable y = H(c) psi on the GPU.

``pauli_apply(coeffs, psi, terms)`` is a ``torch.autograd.Function`` with a
hand-written backward:

* grad_psi = H(c)^dagger g   -- the same apply kernel with conjugated,
  re-signed coefficients (``qr_apply(..., adjoint=1)``);
* grad_c_k = <P_k psi, g>    -- one FP64-accumulated reduction per term
  (``qr_term_grad``); its real part for real coefficients.

Here P_k is term k without its coefficient, (1, -i, -1, +i)[phase_k] X^x Z^z,
and <a, b> = sum conj(a) b.  complex64 states run the compensated-c64
kernels, complex128 states the plain c128 kernels.
"""
from __future__ import annotations

import numpy as np
import torch

from .pyqrusty import PauliOperator


class PauliTerms:
    """The coefficient-free part of a Pauli sum: n and per-term (x, z, phase)
    in make_params' convention.  Holds one GPU operator whose coefficients
    are refreshed from the tensor passed to each forward."""

    def __init__(self, n, x, z, phase):
        self.n = int(n)
        self.x = np.ascontiguousarray(x, dtype=np.uint64)
        self.z = np.ascontiguousarray(z, dtype=np.uint64)
        self.phase = np.ascontiguousarray(phase, dtype=np.uint8)
        self.T = len(self.x)
        self._op = None
        self._cur = None

    def operator(self, coeffs: np.ndarray) -> PauliOperator:
        c = np.ascontiguousarray(coeffs, dtype=np.complex128)
        if self._op is None:
            self._op = PauliOperator(self.n, self.x, self.z, self.phase, c)
        elif self._cur is None or not np.array_equal(self._cur, c):
            self._op.set_coeffs(c)
        self._cur = c.copy()
        return self._op


class _PauliApply(torch.autograd.Function):
    @staticmethod
    def forward(ctx, coeffs, psi, terms):
        c_host = coeffs.detach().to("cpu", torch.complex128).numpy()
        op = terms.operator(c_host)
        y = op.apply(psi.contiguous())
        ctx.save_for_backward(psi)
        ctx.terms = terms
        ctx.c_host = c_host
        ctx.real = not coeffs.is_complex()
        ctx.cdtype = coeffs.dtype
        ctx.cdevice = coeffs.device
        return y

    @staticmethod
    def backward(ctx, gy):
        (psi,) = ctx.saved_tensors
        op = ctx.terms.operator(ctx.c_host)
        gy = gy.contiguous()
        grad_c = grad_psi = None
        if ctx.needs_input_grad[1]:
            grad_psi = op.apply(gy, adjoint=True)
        if ctx.needs_input_grad[0]:
            tg = op.term_grad(psi.contiguous(), gy)
            grad_c = (tg.real if ctx.real else tg).to(device=ctx.cdevice, dtype=ctx.cdtype)
        return grad_c, grad_psi, None


def pauli_apply(coeffs: torch.Tensor, psi: torch.Tensor, terms: PauliTerms) -> torch.Tensor:
    """y = H(coeffs) psi, differentiable in coeffs (real or complex, CPU or
    CUDA tensor of T values) and psi (CUDA complex64 / complex128)."""
    return _PauliApply.apply(coeffs, psi, terms)
