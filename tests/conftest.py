import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def lib_built():
    """Builds libreprobus_gb300.so if needed (nvcc cross-compiles without a GPU)."""
    from reprobus_gb300 import build
    return build.build()


def relerr(a, b, floor=1e-300):
    """Elementwise |a-b| / max(|b|, floor); 0 where both are equal (incl. both 0)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.abs(a - b)
    d = np.where(a == b, 0.0, d)
    return d / np.maximum(np.abs(b), floor)
