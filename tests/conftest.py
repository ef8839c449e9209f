import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("simulation-server_gb300", "oracle"):
    p = os.path.join(REPO, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libbcs.so")


@pytest.fixture(scope="session")
def lib():
    """libbcs.so, built for sm_103a if it is missing or stale."""
    import bcs_build
    import bcs
    bcs_build.build()
    return bcs.load_library()
