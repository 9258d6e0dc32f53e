import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libakaze_gb300.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle_ctypes as oc
    oc.build()
    return oc


@pytest.fixture(scope="session")
def gpu_lib():
    import akaze_gb300
    akaze_gb300.compile_library()
    return akaze_gb300
