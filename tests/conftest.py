import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsgr.so")


@pytest.fixture(scope="session")
def sgr_lib():
    """The built CUDA library (built on first use)."""
    from partgs_gb300 import build, _lib
    build.build()
    return _lib.load()
