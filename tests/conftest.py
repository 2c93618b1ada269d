import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the oracle and the library once per session (both are incremental)."""
    from nbounce_gb300.build import build
    from oracle.build import build_oracle

    build_oracle()
    build()
