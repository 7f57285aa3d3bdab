"""Differentiable y = H(c) psi on the GPU.

``pauli_apply(coeffs, psi, terms)`` is a ``torch.autograd.Function`` with a
hand-written backward:

* grad_psi = H(c)^dagger g   -- the same apply kernel with conjugated,
  re-signed coefficients (``qr_apply(..., adjoint=1)``);
* grad_c_k = <P_k psi, g>    -- one FP64-accumulated reduction per term
  (``qr_term_grad``); its real part for real coefficients.

When both are needed the two run on two streams at once (they read the
same psi / g and write different outputs).

Here P_k is term k without its coefficient, (1, -i, -1, +i)[phase_k] X^x Z^z,
and <a, b> = sum conj(a) b.  complex64 states run the compensated-c64
kernels, complex128 states the plain c128 kernels.

Coefficients on the GPU stay there: each forward hands them to
``qr_op_set_coeffs_device``, whose kernels rebuild the operator's plan
tables on the current stream, so a training step (forward, backward,
optimizer update) has no host synchronisation once the plans exist.
Coefficients in host memory take ``qr_op_set_coeffs`` (synchronous).
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
        self._dev_ref = None
        self._dev_ver = -1
        self._side = {}

    def side_stream(self, device) -> "torch.cuda.Stream":
        """A second stream per device for the backward's term gradients."""
        key = torch.device(device).index
        if key not in self._side:
            self._side[key] = torch.cuda.Stream(device=device)
        return self._side[key]

    def _ensure(self, c_host=None) -> PauliOperator:
        if self._op is None:
            c = np.zeros(self.T, dtype=np.complex128) if c_host is None else c_host
            self._op = PauliOperator(self.n, self.x, self.z, self.phase, c)
            self._cur = None if c_host is None else c_host.copy()
        return self._op

    def operator(self, coeffs) -> PauliOperator:
        """The operator with these coefficients: a CUDA tensor updates it on
        the device (no host synchronisation), anything else on the host."""
        if isinstance(coeffs, torch.Tensor) and coeffs.is_cuda:
            op = self._ensure()
            # the same tensor object at the same version was loaded last time
            # (a backward after its forward): nothing to do.  The reference
            # held here keeps its memory from being reused by another tensor.
            if not (coeffs is self._dev_ref and coeffs._version == self._dev_ver):
                op.set_coeffs_device(coeffs)
                self._dev_ref, self._dev_ver = coeffs, coeffs._version
            self._cur = None
            return op
        c = np.ascontiguousarray(
            coeffs.detach().to("cpu", torch.complex128).numpy()
            if isinstance(coeffs, torch.Tensor) else coeffs, dtype=np.complex128)
        if self._op is None:
            return self._ensure(c)
        if self._cur is None or not np.array_equal(self._cur, c):
            self._op.set_coeffs(c)
            self._cur = c.copy()
        self._dev_ref = None
        return self._op


class _PauliApply(torch.autograd.Function):
    @staticmethod
    def forward(ctx, coeffs, psi, terms):
        op = terms.operator(coeffs)
        y = op.apply(psi.contiguous())
        ctx.save_for_backward(psi, coeffs)
        ctx.terms = terms
        ctx.real = not coeffs.is_complex()
        ctx.cdtype = coeffs.dtype
        ctx.cdevice = coeffs.device
        return y

    @staticmethod
    def backward(ctx, gy):
        psi, coeffs = ctx.saved_tensors
        # the operator may have seen other coefficients since this forward
        op = ctx.terms.operator(coeffs)
        gy = gy.contiguous()
        grad_c = grad_psi = None
        need_c, need_psi = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        if need_c and need_psi and gy.is_cuda:
            # The two halves are independent: the term gradients run on a
            # side stream beside the adjoint apply, so the reduction's CTAs
            # (which take work items from a counter) fill the SMs that the
            # apply's last wave of output tiles leaves idle.
            main = torch.cuda.current_stream(gy.device)
            side = ctx.terms.side_stream(gy.device)
            p = psi.contiguous()
            side.wait_stream(main)
            with torch.cuda.stream(side):
                tg = op.term_grad(p, gy)
            grad_psi = op.apply(gy, adjoint=True)
            main.wait_stream(side)
            tg.record_stream(main)  # allocated on the side stream, read on main
            grad_c = (tg.real if ctx.real else tg).to(device=ctx.cdevice, dtype=ctx.cdtype)
            return grad_c, grad_psi, None
        if need_psi:
            grad_psi = op.apply(gy, adjoint=True)
        if need_c:
            tg = op.term_grad(psi.contiguous(), gy)
            grad_c = (tg.real if ctx.real else tg).to(device=ctx.cdevice, dtype=ctx.cdtype)
        return grad_c, grad_psi, None


def pauli_apply(coeffs: torch.Tensor, psi: torch.Tensor, terms: PauliTerms) -> torch.Tensor:
    """y = H(coeffs) psi, differentiable in coeffs (real or complex, CPU or
    CUDA tensor of T values) and psi (CUDA complex64 / complex128)."""
    return _PauliApply.apply(coeffs, psi, terms)
