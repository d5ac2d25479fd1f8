import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def built_lib():
    """Builds (if needed) and loads the in-tree library."""
    from cupss_gb300 import build
    build.build()
    import cupss_gb300.capi as capi
    return capi.load()
