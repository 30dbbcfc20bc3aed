import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built libqkgw.so")


def _have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def ctx():
    """A qkgw context on cuda:0.  Skips on machines without a GPU; on a GPU machine a missing
    or broken library is an error, never a skip."""
    if not _have_gpu():
        pytest.skip("no CUDA device visible")
    from quack_gb300 import build
    build.build()
    from quack_gb300 import api
    c = api.Context(0)
    yield c
    c.close()
