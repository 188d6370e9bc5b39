import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    return oracle.load()


@pytest.fixture(scope="session")
def gpulib():
    from mctomo_gb300 import build
    build.build()
    import mctomo_gb300
    return mctomo_gb300.lib()
