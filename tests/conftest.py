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


def with_rain(st, per_cell, seed=1):
    """A few SIPs of every cell become drops of 80-400 um radius with small
    multiplicities, falling: most segments of the cloud rows against their
    blocks then have a bound above the thinning threshold (per-pair draws),
    and many pairs collect, as in a raining state."""
    rng = np.random.default_rng(seed)
    nz = st["grid_no_cells"][1]
    cid = st["cells"][0] * nz + st["cells"][1]
    for c in np.unique(cid):
        idx = np.flatnonzero(cid == c)
        sel = rng.choice(idx, size=min(per_cell, len(idx)), replace=False)
        R = rng.uniform(80.0, 400.0, size=len(sel))            # um
        st["m_w"][sel] = 4.18879e3 * R ** 3                     # fg (1000 kg/m^3)
        st["xi"][sel] = rng.uniform(1e2, 1e4, size=len(sel))
        st["vel"][1, sel] = -0.008 * R                          # m/s
    return st


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
