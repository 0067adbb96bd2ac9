import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs libmpcore.so kernels)")


@pytest.fixture(scope="session")
def built():
    """libmpcore.so and the oracle, built in tree (quick when up to date)."""
    from micropolis_gb300 import build as b
    b.build()
    from oracle import oracle
    oracle.build()
    return True


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch
