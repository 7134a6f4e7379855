"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device and the built library."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libmesolf_lf.so")


@pytest.fixture(scope="session")
def lib():
    """The built C-ABI library (built on demand with nvcc; no GPU needed to build)."""
    from mesolf_gb300 import build, _lib
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mesolf_gb300 import build
    build.build()
    return torch.device("cuda:0")
