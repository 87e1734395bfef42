import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built liblagrbf.so")


@pytest.fixture(scope="session")
def have_gpu():
    import ctypes
    try:
        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        import glob
        cands = glob.glob("/usr/local/cuda/lib64/libcudart.so*")
        if not cands:
            return False
        rt = ctypes.CDLL(cands[0])
    n = ctypes.c_int(0)
    return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
