import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 host)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the library and the oracle in-tree once per session (incremental)."""
    from trust_gb300 import build
    build.build_all()
