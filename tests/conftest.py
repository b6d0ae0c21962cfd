import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)   # tests/mlp_ref.py


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


@pytest.fixture(scope="session")
def small():
    """Small PCISPH dam break (1,440 particles, box + sphere)."""
    from bubbles_gb300 import scenes
    return scenes.small_pcisph()


@pytest.fixture(scope="session")
def moved(gpu, small):
    """A state after 30 GPU substeps of the small dam break (particles in motion)."""
    import bubbles_gb300 as bb
    sc, pos = small
    with bb.Solver(sc, pos=pos) as g:
        for _ in range(30):
            g.advance_time_step(sc["dt"])
        p, v = g.download()
    return sc, p, v
