"""Batched ensemble: M members advanced by one launch per kernel must evolve
exactly like M single-member runs with the same Philox seeds.

FP64 mode is deterministic, so batch and single runs agree bit for bit.  In
mixed precision the per-cell condensation sums are FP64 atomics in arbitrary
order, so values agree to 1e-12 relative and the discrete outcomes (cells,
collision counts) exactly.
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
            if precision == "fp64":
                assert np.array_equal(A[k], B[k]), (m, k)
            else:
                np.testing.assert_allclose(B[k], A[k], rtol=1e-12, atol=1e-14, err_msg=f"{m} {k}")
    assert sum(int(b.snapshot(m)["no_cols"].sum()) for m in range(3)) > 0
    assert all(b.flags(m) == 0 for m in range(3))
