import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def flake():
    from dynemol_gb300 import systems
    return systems.honeycomb_flake()


@pytest.fixture(scope="session")
def elhl():
    """The product library (built in-tree); GPU tests only."""
    from dynemol_gb300 import api, build
    build.build()
    api.load()
    if api.device_count() == 0:
        pytest.skip("no CUDA device")
    return api
