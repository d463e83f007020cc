import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the kernels of libgbpt.so")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gb():
    """libgbpt.so built and loaded; the kernels must run on the device."""
    from cudapt_gb300 import build
    build.build()
    import cudapt_gb300
    cudapt_gb300._native.load()
    return cudapt_gb300


@pytest.fixture(scope="session")
def gbdev(gb):
    if not gb.device_available():
        pytest.fail("GPU test: no usable CUDA device for libgbpt.so")
    return gb
