import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer-running case")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads the C-ABI library; only used by gpu tests."""
    from fv2d_gb300 import build as b
    b.build()
    import fv2d_gb300
    return fv2d_gb300.lib()
