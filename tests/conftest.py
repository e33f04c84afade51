import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libxg.so")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def xg():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from ngsxfem_gb300 import build
    build.build()
    from ngsxfem_gb300 import xfem
    return xfem
