import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lla():
    """The package, loaded from linfa-linalg_gb300/ (the library must be built)."""
    import __graft_entry__
    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def gpu_lla(lla):
    if lla.device_count() == 0:
        pytest.fail("GPU test collected on a machine without a CUDA device")
    return lla
