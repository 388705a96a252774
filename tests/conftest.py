import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """Build the CUDA library (cross-compiles without a GPU) and the oracle once."""
    from cudaprotoplanetarydisks_gb300 import build as pbuild
    from oracle import build as obuild
    pbuild.build()
    obuild.build()
    yield


def have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture
def gpu():
    if not have_gpu():
        pytest.fail("this test needs a GPU")
    return True
