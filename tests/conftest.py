import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs libvmp.so kernels)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    return oracle.load()


@pytest.fixture(scope="session")
def vmp_lib():
    from voxelmapplus_fastlio2_gb300 import _lib
    return _lib.load()
