import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def port():
    from oracle.cforacle import Port
    return Port()


@pytest.fixture(scope="session")
def cuda_lib():
    """The in-tree CUDA library, built for sm_103a if it is missing."""
    from channel_flow_gb300 import build
    build.build()
    from channel_flow_gb300 import _lib
    return _lib.load()
