import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_ROOT = os.path.join(ROOT, "melvin.py_gb300")
for p in (ROOT, PKG_ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device and the built native library")


@pytest.fixture(scope="session")
def golden():
    with np.load(GOLDEN) as d:
        return {k: d[k] for k in d.files}


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (n if n > 0 else 1.0))


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a host without CUDA (run with -m 'not gpu')")
    from melvin import _native

    _native.load_library()  # fails loudly when the library is missing
    return torch.device("cuda", 0)
