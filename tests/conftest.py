import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")


@pytest.fixture(scope="session")
def built_lib():
    from pincosimulator_gb300 import build_ext, twmc

    build_ext.build()
    return twmc.load()


@pytest.fixture(scope="session")
def oracle():
    from oracle import build_oracle, loader

    build_oracle.build()
    return loader
