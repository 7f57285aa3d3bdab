"""The eigensolver loop the vector helpers exist for (the sandbox's use,
pyqrusty/sandbox/test1.py): a Davidson iteration for the lowest eigenvalue of
the H4 / H6 fixture Hamiltonians built only from this library's GPU calls --
H psi with the residual fused (apply_axpby), FP64 inner products (vdot),
axpby, the operator diagonal and precond2 -- checked against numpy's dense
eigensolver on the oracle's CSR."""
import numpy as np
import pytest

from qrusty_gb300 import PauliOperator, axpby, precond2, vdot
from tests.helpers import csr_to_dense, terms_of_labels

pytestmark = pytest.mark.gpu


def davidson_lowest(op, n, iters=60, tol=1e-10):
    import torch
    dev = torch.device("cuda", 0)
    N = 1 << n
    diag = op.diagonal()
    x = torch.zeros(N, dtype=torch.complex128, device=dev)
    x[int(torch.argmin(diag.real))] = 1.0  # start at the smallest diagonal entry
    V = [x]
    HV = [op.apply(x)]
    theta = None
    for _ in range(iters):
        k = len(V)
        Hs = np.empty((k, k), dtype=complex)
        for i in range(k):
            for j in range(k):
                Hs[i, j] = complex(vdot(V[i], HV[j]).item())
        w, U = np.linalg.eigh((Hs + Hs.conj().T) / 2)
        theta = float(w[0])
        u = U[:, 0]
        xr = sum(complex(u[i]) * V[i] for i in range(k))
        # residual r = H x - theta x, fused into the apply kernel
        r = op.apply_axpby(xr, xr, 1.0, -theta)
        if float(torch.linalg.vector_norm(r)) < tol:
            break
        t = precond2(diag, r, theta, 1e-8)  # Davidson correction dx / (diag - theta)
        for vi in V:  # Gram-Schmidt twice
            t = axpby(1.0, t, -complex(vdot(vi, t).item()), vi)
        for vi in V:
            t = axpby(1.0, t, -complex(vdot(vi, t).item()), vi)
        nt = float(torch.linalg.vector_norm(t))
        if nt < 1e-12:
            break
        t = t / nt
        V.append(t)
        HV.append(op.apply(t))
    return theta


@pytest.mark.parametrize("name", ["H4", "H6"])
def test_davidson_ground_energy(cuda, oracle, golden, name):
    labels, coeffs = golden[name]
    n, x, z, ph, c = terms_of_labels(labels, coeffs)
    op = PauliOperator(n, x, z, ph, c)
    e = davidson_lowest(op, n)
    ip, ij, d = oracle.csr_build(n, x, z, oracle.make_params(ph, c), nthreads=4)
    dense = csr_to_dense(ip, ij, d, (1 << n, 1 << n))
    want = float(np.linalg.eigvalsh((dense + dense.conj().T) / 2)[0])
    assert abs(e - want) <= 1e-8 * max(1.0, abs(want)), (e, want)
