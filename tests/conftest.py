"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs
on a CPU-only machine."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libhzgb300.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    return O.Oracle()


@pytest.fixture(scope="session")
def hz():
    """The CUDA library; built on first use if needed."""
    import helmholtz_3d_torrone_gb300 as hz
    if not os.path.exists(hz.LIB_PATH):
        from helmholtz_3d_torrone_gb300 import _build
        _build.build()
    hz.load()
    return hz


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))
