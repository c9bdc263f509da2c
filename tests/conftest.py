import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libswc.so")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def lib():
    """libswc.so, built in-tree if missing. A GPU test fails (never skips) without it."""
    from smaiso_wcomp_gb300 import abi, build
    if not os.path.exists(abi.LIB_PATH):
        build.build()
    return abi.load_library()
