import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libifemgpu.so")


@pytest.fixture(scope="session")
def gpulib():
    """The C-ABI library, built in-tree if missing."""
    from ifem_gb300 import build, ifemgpu
    build.ensure_built()
    return ifemgpu.load_library()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle
