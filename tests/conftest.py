import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: long CPU-only checks")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds and loads libprgpu.so; GPU tests fail loudly if it is missing."""
    from playrho_gb300 import build, gpu

    build.build()
    return gpu.load_library()
