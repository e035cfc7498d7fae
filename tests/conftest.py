import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); run with -m gpu")


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle (test infrastructure)."""
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def lgt():
    """The product package, with its CUDA library loaded (built if stale)."""
    import lgt_gb300
    from lgt_gb300 import _capi
    _capi.load()
    return lgt_gb300
