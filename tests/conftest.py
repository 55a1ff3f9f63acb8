import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103) and the built CUDA library")


@pytest.fixture(scope="session")
def built():
    """Builds the oracle and the CUDA library once per session."""
    from oracle import build as ob
    from aurora_gb300 import build as ab
    ob.build_oracle()
    ab.build()
    return True


@pytest.fixture(scope="session")
def ctx(built):
    from aurora_gb300 import api
    c = api.Context(0)
    yield c
    c.close()
