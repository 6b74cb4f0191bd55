import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import __graft_entry__  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


@pytest.fixture(scope="session")
def eb():
    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def O():
    return __graft_entry__.load_oracle()


@pytest.fixture(scope="session")
def scenes(eb):
    from endobeams_gb300 import scenes as s
    return s
