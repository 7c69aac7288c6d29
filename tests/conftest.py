import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the library's device code")
    config.addinivalue_line("markers", "slow: long CPU test")


@pytest.fixture(scope="session")
def lib_path():
    from hofstadter_hubbard_tsc_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def device(lib_path):
    from hofstadter_hubbard_tsc_gb300.device import Device
    dev = Device(0)
    yield dev
    dev.close()
