import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the native library")


@pytest.fixture(scope="session")
def native_lib():
    """Builds (if needed) and loads the native library."""
    from moljax_gb300 import build_native, _native
    build_native.build()
    return _native.load()


@pytest.fixture(scope="session")
def cuda(native_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda", 0)
