import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libgrx.so")


@pytest.fixture(scope="session")
def grx_lib():
    """libgrx.so built and loaded; GPU tests fail (not skip) when it is missing."""
    from graspa_gb300 import grx
    from graspa_gb300 import build as b
    b.build()
    L = grx.load()
    import ctypes
    n = ctypes.c_int32()
    st = L.grx_device_count(ctypes.byref(n))
    assert st == 0 and n.value > 0, "no CUDA device visible to libgrx"
    return grx
