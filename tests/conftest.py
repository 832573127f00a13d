"""Test configuration: the `gpu` marker and a session-start build check.

CPU tests (`-m "not gpu"`) exercise the oracle against the golden vectors,
the host logic of the library and its exported C ABI; GPU tests (`-m gpu`)
are the parity tests proper and call the CUDA library through the C ABI.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300)")


def pytest_sessionstart(session):
    # build what is stale: the oracle (gcc, seconds) and the CUDA library
    from oracle import oracle as O
    O.build()
    from weldformgpu_gb300 import build as B
    B.build()


@pytest.fixture(scope="session")
def has_gpu():
    import ctypes
    try:
        lib = ctypes.CDLL("libcuda.so.1")
        n = ctypes.c_int(0)
        if lib.cuInit(0) != 0 or lib.cuDeviceGetCount(ctypes.byref(n)) != 0:
            return False
        return n.value > 0
    except OSError:
        return False
