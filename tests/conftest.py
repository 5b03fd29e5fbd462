import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); run with -m gpu")
    config.addinivalue_line("markers", "slow: long CPU test")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    """Build the host libraries (case builder, oracle) in-tree once per session."""
    from eqdyna_gb300 import build
    build.build_case()
    build.build_oracle()
    yield


def golden_path(name):
    return os.path.join(GOLDEN, name + ".npz")


def nthreads():
    return max(1, min(16, os.cpu_count() or 1))
