import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session", autouse=True)
def _build_oracle():
    from tomosipo_gb300._build import build_oracle

    build_oracle()


@pytest.fixture(scope="session")
def native_lib():
    """Native library, built if needed (GPU tests only)."""
    from tomosipo_gb300._build import build_library
    from tomosipo_gb300 import _native

    build_library()
    return _native.load()


def rel_l2(a, b):
    import numpy as np

    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
