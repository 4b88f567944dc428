import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (runs through the C-ABI)")


@pytest.fixture(scope="session")
def native():
    """The CUDA engine library, built in-tree if needed."""
    from mbsolve_gb300 import build, _native
    build.build()
    return _native.load()


@pytest.fixture(autouse=True)
def _fresh_library():
    from mbsolve_gb300 import lib as mb
    mb.material.clear_library()
    yield
    mb.material.clear_library()
