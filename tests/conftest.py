import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 and the CUDA library")
    config.addinivalue_line("markers", "slow: longer CPU oracle runs")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def ug():
    """The CUDA library (built in-tree); GPU tests fail loudly without it."""
    import upcgen_gb300
    from upcgen_gb300 import build
    build.build()
    upcgen_gb300.load_library()
    return upcgen_gb300
