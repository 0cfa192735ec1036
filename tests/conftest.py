import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds libgg.so and the oracle once per session (no GPU needed)."""
    import __graft_entry__
    __graft_entry__.build()
    yield
