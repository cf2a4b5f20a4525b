import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU; runs the CUDA library")


@pytest.fixture(scope="session")
def xrt():
    """Builds (if stale) and loads libxrt.so."""
    from xrtailor_gb300 import build as xb
    xb.build()
    from xrtailor_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    return oracle.lib()
