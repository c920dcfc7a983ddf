import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def gbrt_lib():
    """libgbrt.so, built in-tree if missing; raises (no fallback) when it
    cannot be loaded."""
    from libyafaray_gb300 import build, gbrt
    if not os.path.exists(gbrt.LIB_PATH):
        build.build()
    return gbrt.load()


@pytest.fixture(scope="session")
def cuda_device(gbrt_lib):
    import ctypes
    n = ctypes.c_int(0)
    rc = gbrt_lib.gbrt_device_count(ctypes.byref(n))
    if rc != 0 or n.value < 1:
        pytest.fail("no CUDA device visible to libgbrt.so")
    return 0
