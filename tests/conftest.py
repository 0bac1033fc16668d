import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the native library and the oracle once per session if missing."""
    from xflat_gb300 import _abi
    if not os.path.exists(_abi.LIB_PATH):
        from xflat_gb300 import build
        build.build()
    from oracle import port
    if not os.path.exists(port.LIB):
        port.build()
    yield


@pytest.fixture(scope="session")
def gpu_available():
    import ctypes
    try:
        cudart = ctypes.CDLL("libcuda.so.1")
        n = ctypes.c_int()
        return cudart.cuInit(0) == 0 and cudart.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
    except OSError:
        return False
