import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the library and the oracle once per session (no-op when fresh)."""
    from blobs_gb300 import build as b
    from oracle import build as ob
    b.build()
    ob.build()
