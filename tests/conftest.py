import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libmsl.so")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name))
    return load


@pytest.fixture(scope="session")
def fparams():
    from multislice_gb300 import fparams_table
    return fparams_table()


@pytest.fixture(scope="session")
def ctx():
    """A libmsl context on cuda:0; fails (never skips) when the library or GPU is missing."""
    from multislice_gb300 import Context
    c = Context(0)
    yield c
    c.close()
