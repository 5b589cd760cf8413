import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libpfg.so")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def cuda():
    """The GPU tests run only where a GPU exists; the library must be built
    there (no fallback: a missing libpfg.so is a failure, not a skip)."""
    import torch
    assert torch.cuda.is_available(), "GPU test selected but no CUDA device is visible"
    from plantfem_gb300 import _native
    _native.load()
    return torch.device("cuda:0")
