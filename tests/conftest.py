import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle"), GOLDEN):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build libmclg.so and the oracle once per session (in-tree, incremental)."""
    from mantle_convection_lab_gb300 import _build
    _build.build()
    import build_oracle
    build_oracle.build()


def golden(case):
    return np.load(os.path.join(GOLDEN, f"{case}.npz"))


def golden_input(case):
    return os.path.join(GOLDEN, f"{case}.input")


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)
