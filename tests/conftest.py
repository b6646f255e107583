import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402

PKG = __graft_entry__.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def pkg():
    return PKG


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if stale) and load the CUDA library; skip-free: GPU tests fail
    loudly when the library cannot be built or no device exists."""
    PKG.build.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return PKG.load_library()
