from __future__ import annotations

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built sm_103a library")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def built_library():
    """Build the CUDA library (nvcc cross-compiles without a GPU) and the oracle helper."""
    from d2ic_gb300 import build as b
    b.build()
    from oracle import fast
    fast.build()
    from d2ic_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from d2ic_gb300 import build as b
    b.build()
    return torch.device("cuda:0")
