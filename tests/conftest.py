import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads the CUDA library; GPU tests fail loudly without it."""
    from simpimc_gb300 import build as B
    B.build()
    import simpimc_gb300
    return simpimc_gb300.load_library()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle
