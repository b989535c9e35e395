import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def native_lib():
    """lib_fftwpp.so, built in-tree if stale."""
    from fftwpp_gb300 import build, _native
    build.build()
    return _native.load()
