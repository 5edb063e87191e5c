import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libemix_gb300.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle_py
    oracle_py.load()
    return oracle_py


@pytest.fixture(scope="session")
def emix():
    """The CUDA library; on a GPU machine a missing build is an error, not a skip."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from emix_gb300 import ops, _lib
    _lib.load()
    return ops
