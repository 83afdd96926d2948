import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def native():
    from lassie_gb300 import _native as nat
    L = nat.load()
    return L


@pytest.fixture(scope="session")
def gpu(native):
    if not native.lassie_device_ok():
        pytest.fail("GPU test without an sm_103 device: the native path must run")
    return native
