import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpulib():
    """The CUDA library, built in-tree; GPU tests fail loudly if it cannot load."""
    if not gpu_available():
        pytest.skip("no CUDA device")
    from starfish_gb300 import build, abi
    build.build()
    return abi.load()
