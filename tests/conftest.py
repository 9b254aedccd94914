import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden(name):
    """Load a golden fixture made by tests/golden/make_golden.py."""
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def sub(d, prefix):
    """Entries of an .npz whose key starts with ``prefix + '__'``."""
    p = prefix + "__"
    return {k[len(p):]: d[k] for k in d.files if k.startswith(p)}


@pytest.fixture(scope="session")
def oracle_py():
    from oracle.oracle import Oracle
    return Oracle("py")


@pytest.fixture(scope="session")
def oracle_nb():
    from oracle.oracle import Oracle
    return Oracle("numba")


@pytest.fixture(scope="session")
def oracle_cr():
    from oracle.oracle import Oracle
    return Oracle("cr")
