import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA path through the C ABI)")


def _cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cuda_ok():
    if not _cuda_available():
        pytest.skip("no CUDA device")
    return True


@pytest.fixture(scope="session")
def gpu_lib():
    """The built CUDA library (fails loudly if it cannot be built or loaded)."""
    from footile_gb300 import _lib
    return _lib.load()


@pytest.fixture()
def ctx(cuda_ok, gpu_lib):
    from footile_gb300._lib import Context
    c = Context(0)
    yield c
    c.close()
