"""Batched ensemble: M members advanced by one launch per kernel must evolve
exactly like M single-member runs with the same Philox seeds.

Both modes are deterministic (in mixed precision the per-cell condensation
sums are exact integer sums), so batch and single runs agree bit for bit, and
so do two runs of the same ensemble.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from lacmopy_gb300 import build
    build.build()


def _members(M, nx=24, nz=20):
    from lacmopy_gb300 import synthetic
    return [synthetic.make_icmw_state(Nx=nx, Nz=nz, seed=100 + m, kernel_type="Hall_Bott",
                                      uneven=(32, 96), drizzle_fraction=0.15, r_tot=12.5E-3)
            for m in range(M)]


def _copy(st):
    return {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}


@pytest.mark.parametrize("precision,draws", [("fp64", "philox"), ("mixed", "philox"),
                                             ("mixed", "thinned"), ("fp64", "thinned")])
@pytest.mark.parametrize("graph", [False, True])
def test_batch_equals_single_members(precision, draws, graph):
    from lacmopy_gb300 import BatchState, DeviceState
    sts = _members(3)
    seeds = [11, 12, 13]
    assert len({st["xi"].size for st in sts}) == 3   # uneven member sizes
    b = BatchState([_copy(st) for st in sts], seeds, precision=precision, draws=draws)
    b.adv_step(3, graph=graph)
    for m, st in enumerate(sts):
        d = DeviceState(_copy(st), draws=draws, seed=seeds[m], precision=precision)
        d.adv_step(3)
        A, B = d.snapshot(), b.snapshot(m)
        assert np.array_equal(A["cells"], B["cells"])
        assert np.array_equal(A["no_cols"], B["no_cols"])
        for k in ("m_w", "xi", "pos", "vel", "grid_scalar_fields", "water_removed"):
            assert np.array_equal(A[k], B[k]), (precision, m, k)
    assert sum(int(b.snapshot(m)["no_cols"].sum()) for m in range(3)) > 0
    assert all(b.flags(m) == 0 for m in range(3))


def test_mixed_ensemble_is_reproducible():
    """Two runs of the same mixed-precision ensemble give the same bits."""
    from lacmopy_gb300 import BatchState
    sts = _members(2)
    out = []
    for _ in range(2):
        b = BatchState([_copy(st) for st in sts], [21, 22], precision="mixed", draws="thinned")
        b.adv_step(4, graph=True)
        out.append([b.snapshot(m) for m in range(2)])
    for A, B in zip(*out):
        for k in ("m_w", "xi", "pos", "vel", "grid_scalar_fields", "no_cols"):
            assert np.array_equal(A[k], B[k]), k
