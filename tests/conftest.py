import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: full-size cases")


@pytest.fixture(scope="session")
def lib():
    from blitzen_gb300 import build
    build.build()
    from blitzen_gb300 import abi
    return abi.load()


@pytest.fixture(scope="session")
def culler(lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from blitzen_gb300.culler import Culler
    c = Culler(0)
    yield c
    c.close()
