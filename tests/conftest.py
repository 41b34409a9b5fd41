import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)

import __graft_entry__ as ge  # noqa: E402

ge.load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def api():
    """The CUDA library's Python context (builds it if needed)."""
    from beachslope_gb300 import build
    build.build_library()
    from beachslope_gb300 import api as a
    return a


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.build()
    return o
