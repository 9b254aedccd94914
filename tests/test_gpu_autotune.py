"""Launch shapes change the speed, not the results: an FP64 batch steps bit
for bit alike under every collision and cell-ordering shape, a mixed batch
under every particle-kernel shape to the tolerance of its any-order sums
(1e-12); and the autotuner picks listed options and reuses its cache."""
import copy

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
    yield
    from lacmopy_gb300 import autotune
    autotune.reset()


def _members():
    from lacmopy_gb300 import synthetic
    out = []
    for sd in (3, 4):
        st = synthetic.make_icmw_state(Nx=12, Nz=10, no_spcm=(10, 14), seed=sd,
                                       kernel_type="Hall_Bott", drizzle_fraction=0.3,
                                       r_tot=12.5E-3)
        st["dt_col_over_dV"] = st["dt_col_over_dV"] * 60.0
        out.append(st)
    return out


def _run(states, precision, choice, steps=3):
    from lacmopy_gb300 import BatchState, autotune
    autotune.reset()
    autotune.apply(choice)
    b = BatchState([copy.deepcopy(s) for s in states], [11, 12], precision=precision,
                   draws="thinned")
    b.adv_step(steps)
    out = [b.snapshot(m) for m in range(b.M)]
    autotune.reset()
    return out


def test_fp64_results_do_not_depend_on_collision_and_order_shapes():
    from lacmopy_gb300 import autotune
    st = _members()
    ref = _run(st, "fp64", {})
    assert sum(r["no_cols"].sum() for r in ref) > 0
    for col in autotune.options("collision_blocks_per_sm")[1:]:
        for order in autotune.options("order_blocks_per_sm")[1:2]:
            got = _run(st, "fp64", {"collision_blocks_per_sm": col, "order_blocks_per_sm": order})
            for g, r in zip(got, ref):
                for k in ("xi", "m_w", "m_s", "pos", "vel", "no_cols", "cells"):
                    assert np.array_equal(g[k], r[k]), (col, order, k)


def test_mixed_results_do_not_depend_on_particle_shape():
    from lacmopy_gb300 import autotune
    st = _members()
    ref = _run(st, "mixed", {})
    for pb in autotune.options("particle_blocks_per_sm")[1:]:
        got = _run(st, "mixed", {"particle_blocks_per_sm": pb})
        for g, r in zip(got, ref):
            np.testing.assert_allclose(g["m_w"], r["m_w"], rtol=1e-12, atol=0)
            np.testing.assert_allclose(g["grid_scalar_fields"], r["grid_scalar_fields"],
                                       rtol=1e-12)


def test_tune_batch_picks_options_and_reuses_the_cache(tmp_path):
    from lacmopy_gb300 import autotune
    st = _members()
    path = str(tmp_path / "shapes.json")
    choice = autotune.tune_batch(st, [11, 12], precision="mixed", draws="thinned",
                                 cache_path=path)
    for k, v in choice.items():
        assert v in autotune.options(k)
    assert autotune.current() == choice
    cache = autotune.load_cache(path)
    assert len(cache) == 1
    entry = next(iter(cache.values()))
    assert set(entry["ms_per_step"]) == set(autotune.KNOBS)
    autotune.reset()
    again = autotune.tune_batch(st, [11, 12], precision="mixed", draws="thinned",
                                cache_path=path)
    assert again == choice and autotune.current() == choice
    autotune.reset()
