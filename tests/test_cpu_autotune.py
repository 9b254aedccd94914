"""Host logic of the launch-shape autotuner: the knobs of the C ABI (no GPU
needed to set them), the workload key and the cache."""
import numpy as np
import pytest


def test_knobs_options_set_get():
    from lacmopy_gb300 import autotune
    from lacmopy_gb300 import build
    build.build()
    autotune.reset()
    for knob in autotune.KNOBS:
        opts = autotune.options(knob)
        assert len(opts) >= 2 and len(set(opts)) == len(opts)
        assert autotune.current()[knob] == opts[0]
        autotune.apply({knob: opts[-1]})
        assert autotune.current()[knob] == opts[-1]
    with pytest.raises(Exception):
        autotune.apply({"collision_blocks_per_sm": 7})
    autotune.reset()
    assert autotune.current() == {k: autotune.options(k)[0] for k in autotune.KNOBS}


def test_workload_key_and_cache(tmp_path):
    from lacmopy_gb300 import autotune, synthetic
    a = synthetic.make_icmw_state(Nx=8, Nz=6, no_spcm=(4, 6), seed=1)
    b = synthetic.make_icmw_state(Nx=8, Nz=6, no_spcm=(4, 6), seed=2)
    c = synthetic.make_icmw_state(Nx=8, Nz=6, no_spcm=(40, 60), seed=3)
    k1 = autotune.workload_key([a, b], "mixed", "thinned", "GPU")
    assert k1 == autotune.workload_key([b, a], "mixed", "thinned", "GPU")
    assert k1 != autotune.workload_key([a, b], "fp64", "thinned", "GPU")
    assert k1 != autotune.workload_key([a, b], "mixed", "philox", "GPU")
    assert k1 != autotune.workload_key([c, c], "mixed", "thinned", "GPU")
    # a raining ensemble (a drop of 1e8 fg = R ~ 290 um) is a different workload
    r = dict(a)
    r["m_w"] = np.asarray(a["m_w"]).copy()
    r["m_w"][np.flatnonzero(np.asarray(a["active_ids"]))[0]] = 1e8
    assert k1 != autotune.workload_key([r, b], "mixed", "thinned", "GPU")
    path = str(tmp_path / "shapes.json")
    assert autotune.load_cache(path) == {}
    autotune.save_cache(path, {k1: {"choice": {"particle_blocks_per_sm": 8}}})
    assert autotune.load_cache(path)[k1]["choice"]["particle_blocks_per_sm"] == 8
    np.testing.assert_equal(len(autotune.load_cache(path)), 1)
