import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libfuelg.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.load()
    return o


@pytest.fixture(scope="session")
def lib():
    """libfuelg.so, built in place if it is missing (nvcc cross-compiles here)."""
    from fuel_gb300 import _lib, build
    if not build.up_to_date():
        build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def gpu(lib):
    """Fails (never skips) when no GPU is visible: GPU tests must run the CUDA path."""
    from fuel_gb300 import _lib
    n = _lib.device_count()
    assert n >= 1, "no CUDA device visible: GPU tests need a GB300"
    return n


def threads():
    return max(1, min(16, os.cpu_count() or 1))


def f32_bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)
