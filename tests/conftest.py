import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the engine's C ABI")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the engine and the oracle once per session (no-op when up to date)."""
    from briefmatch_gb300 import build as b

    b.build_engine()
    b.build_oracle()
    yield
