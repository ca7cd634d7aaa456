import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
# shared test helpers (shape_cases)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def si_tables():
    from montecarlocpp_gb300 import silicon_tables
    return silicon_tables()


@pytest.fixture(scope="session")
def omat(si_tables):
    from oracle import oracle as O
    return O.OMaterial(*si_tables, 300.0)


@pytest.fixture(scope="session")
def gmat():
    import montecarlocpp_gb300 as M
    return M.Material.silicon(300.0)
