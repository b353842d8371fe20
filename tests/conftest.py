import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "hydro-cl-lua_gb300")
ORACLE = os.path.join(ROOT, "oracle")
for p in (PKG, ORACLE, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs libhydrocuda kernels)")


@pytest.fixture(scope="session")
def hc():
    """The product library on GPU 0.  No silent skip: a GPU test without a
    working device or library fails."""
    import hydrocuda
    hydrocuda.load_library()
    n = hydrocuda.device_count()
    assert n > 0, "GPU tests need a CUDA device"
    return hydrocuda


@pytest.fixture(scope="session")
def ctx(hc):
    return hc.default_context()
