import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def sbs():
    """The GPU package. On a GPU machine a missing or unloadable libsbs fails the test."""
    import soap_bubble_simulation_gb300 as pkg

    lib = pkg._native.lib()
    import ctypes

    n = ctypes.c_int()
    rc = lib.sbs_device_count(ctypes.byref(n))
    if rc != 0 or n.value < 1:
        pytest.fail(f"no CUDA device visible to libsbs: {pkg._native.last_error()}")
    return pkg
