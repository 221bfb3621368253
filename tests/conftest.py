"""Shared test setup: the `gpu` marker, library / oracle builds."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity of the CUDA path against the oracle")
    config.addinivalue_line("markers", "slow: full-size workload")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def nbgb_lib():
    """The CUDA library, built in-tree for sm_103a (compiles here without a GPU)."""
    from nbodysimulation_gb300 import build
    build.build()
    import nbodysimulation_gb300 as nb
    nb.load()
    return nb


@pytest.fixture(scope="session")
def gpu(nbgb_lib):
    """Skip unless a CUDA device is visible; the library itself must load either way."""
    import ctypes
    try:
        cudart = ctypes.CDLL("libcuda.so.1")
        cnt = ctypes.c_int(0)
        if cudart.cuInit(0) != 0 or cudart.cuDeviceGetCount(ctypes.byref(cnt)) != 0 or cnt.value == 0:
            pytest.skip("no CUDA device")
    except OSError:
        pytest.skip("no CUDA driver")
    return nbgb_lib
