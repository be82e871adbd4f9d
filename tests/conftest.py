import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def built_lib():
    """Build libdns3d_gpu.so in-tree (no-op when up to date) and load it."""
    from f90_dns_gb300 import build, capi
    build.build()
    return capi.load_library()
