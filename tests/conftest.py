import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long CPU test")


@pytest.fixture(scope="session")
def native():
    from bubbles_gb300 import _native
    _native.load()
    return _native


@pytest.fixture(scope="session")
def gpu(native):
    if native.device_count() < 1:
        pytest.fail("no CUDA device visible to libbbg")
    return native
