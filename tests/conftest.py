import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def backend():
    """The GPU backend; built on demand.  Fails (does not skip) if the
    library cannot be built or loaded."""
    from simradar_gb300 import build as b
    from simradar_gb300 import rsc
    b.build()
    rsc.load_library()
    return rsc
