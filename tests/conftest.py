import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and libqrusty_gpu.so")


@pytest.fixture(scope="session")
def golden():
    d = np.load(os.path.join(GOLDEN, "hamiltonians.npz"))
    out = {}
    for key in d.files:
        if key.endswith("_labels"):
            name = key[: -len("_labels")]
            out[name] = ([str(s) for s in d[key]], d[name + "_coeffs"])
    return out


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test needs CUDA; none visible")
    from qrusty_gb300 import _lib
    _lib.load()
    return torch.device("cuda", 0)
