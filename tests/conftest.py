import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built CUDA library")


@pytest.fixture(scope="session")
def cuda_lib():
    """The CUDA library, built in-tree if needed (no fallback)."""
    from drd_application_gb300 import _lib, build

    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def oracle_build():
    from oracle import oracle

    oracle.build()
    return oracle
