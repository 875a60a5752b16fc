import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libmddem_gb300.so")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if stale) and load the CUDA library; the GPU tests fail loudly without it."""
    from mddem_gb300 import build, capi

    build.build()
    lib = capi.load()
    import ctypes

    n = ctypes.c_int(0)
    lib.mdg_device_count(ctypes.byref(n))
    assert n.value >= 1, "no CUDA device visible"
    return lib


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle

    oracle.build()
    return oracle
