import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def built_oracle():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def built_lib():
    from jurassic_gb300 import build, native
    build.build()
    return native.load()
