import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through libnsg.so")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build(ref=None)
    return oracle


@pytest.fixture(scope="session")
def nsg():
    """libnsg.so built in-tree and loaded (CPU-safe: loading needs no GPU)."""
    from nscale_gb300 import build, _lib
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from nscale_gb300 import build
    build.build()
    return torch.device("cuda:0")
