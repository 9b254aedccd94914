"""Drop-in step functions called once per time step with Philox draws.

The reference draws fresh uniforms on every collision step
(collision/all_or_nothing.py:545, np.random.rand).  The drop-in functions
build a new device state on every call, so they carry the Philox
collision-step counter of each seed from one call to the next: two
consecutive ``integrate_adv_step_np`` calls equal two steps of one resident
``DeviceState`` bit for bit, and two calls on identical inputs draw
different uniforms.
"""
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


def _state(seed=41):
    from lacmopy_gb300 import synthetic
    st = synthetic.make_icmw_state(Nx=20, Nz=18, no_spcm=(10, 14), seed=seed,
                                   kernel_type="Hall_Bott", drizzle_fraction=0.3, r_tot=12.5E-3)
    st["dt_col_over_dV"] = st["dt_col_over_dV"] * 60.0   # collisions in every step
    return st


@pytest.mark.parametrize("draws", ["philox", "thinned"])
def test_consecutive_dropin_calls_continue_the_draws(draws):
    from lacmopy_gb300 import DeviceState
    from lacmopy_gb300 import integration as I
    from lacmopy_gb300.device import philox_counter, reset_philox_counters
    seed = 777
    st = _state()
    want_ds = DeviceState(copy.deepcopy(st), draws=draws, seed=seed)
    want_ds.adv_step(2)
    want = want_ds.snapshot()
    assert want_ds.col_step == 4      # two collision steps per advection step

    reset_philox_counters(seed)
    got = copy.deepcopy(st)
    for _ in range(2):
        I.integrate_adv_step_np(*[got[k] for k in I._STATE_KEYS], draws=draws, seed=seed)
    assert philox_counter(seed) == 4
    assert want["no_cols"].sum() > 0
    assert np.array_equal(got["no_cols"], want["no_cols"])
    for k in ("xi", "m_w", "m_s", "pos", "vel"):
        assert np.array_equal(got[k], want[k]), k
    assert np.array_equal(got["cells"], want["cells"])

    # a pinned counter reproduces the second call alone
    again = copy.deepcopy(st)
    I.integrate_adv_step_np(*[again[k] for k in I._STATE_KEYS], draws=draws, seed=seed,
                            col_step=0)
    I.integrate_adv_step_np(*[again[k] for k in I._STATE_KEYS], draws=draws, seed=seed,
                            col_step=2)
    for k in ("xi", "m_w", "m_s"):
        assert np.array_equal(again[k], want[k]), k
    reset_philox_counters(seed)


@pytest.mark.parametrize("draws", ["philox", "thinned"])
def test_repeated_collision_calls_draw_fresh_uniforms(draws):
    """The all-cells collision drop-in on the same input twice: the second
    call uses the next collision step's draws, so its outcome differs."""
    from lacmopy_gb300 import collision as C
    from lacmopy_gb300.device import reset_philox_counters
    st = _state(seed=43)
    seed = 5
    reset_philox_counters(seed)
    outs = []
    for _ in range(2):
        xi, mw, ms = st["xi"].copy(), st["m_w"].copy(), st["m_s"].copy()
        nc = np.zeros(2, np.int64)
        C.collision_step_Ecol_grid_R_all_cells_2D_multicomp_np(
            xi, mw, ms, st["vel"], st["grid_scalar_fields"][0], st["cells"], st["grid_no_cells"],
            st["dt_col_over_dV"], st["E_col_grid"], st["no_kernel_bins"], st["R_kernel_low_log"],
            st["bin_factor_R_log"], nc, "AS", draws=draws, seed=seed)
        outs.append((xi, mw, nc))
    assert outs[0][2].sum() > 0 and outs[1][2].sum() > 0
    assert not np.array_equal(outs[0][0], outs[1][0])
    reset_philox_counters(seed)


def test_resident_buffers_and_graph_between_calls():
    """integrate_adv_step_np keeps its device buffers (and the captured step
    graph) between calls of the same shape: three calls in mixed precision
    equal three steps of one resident DeviceState bit for bit; a call with
    changed parameters captures a new graph and equals a fresh state with
    those parameters; another shape in between leaves both intact."""
    from lacmopy_gb300 import DeviceState
    from lacmopy_gb300 import integration as I
    from lacmopy_gb300.device import reset_philox_counters
    seed = 913
    st = _state(seed=47)
    key = (st["pos"].shape[1], 20, 18)
    want_ds = DeviceState(copy.deepcopy(st), draws="thinned", seed=seed, precision="mixed")
    want_ds.adv_step(3)
    want = want_ds.snapshot()

    I.release_resident()
    reset_philox_counters(seed)
    got = copy.deepcopy(st)
    other = _state(seed=48)
    other["pos"] = other["pos"][:, :-5].copy()   # another SIP count
    for k in ("vel", "rel_pos"):
        other[k] = other[k][:, :-5].copy()
    for k in ("m_w", "m_s", "xi", "T_p", "active_ids"):
        other[k] = other[k][:-5].copy()
    other["cells"] = other["cells"][:, :-5].copy()
    plans = []
    for step in range(3):
        I.integrate_adv_step_np(*[got[k] for k in I._STATE_KEYS], draws="thinned", seed=seed,
                                precision="mixed")
        plans.append(I._resident[key]._plan_handle.value)
        if step == 0:
            I.integrate_adv_step_np(*[other[k] for k in I._STATE_KEYS], draws="thinned",
                                    seed=seed + 1, precision="mixed")
    assert plans[0] == plans[1] == plans[2]          # one graph, replayed
    assert want["no_cols"].sum() > 0
    for k in ("xi", "m_w", "m_s", "pos", "vel", "T_p", "grid_scalar_fields", "no_cols"):
        assert np.array_equal(got[k], want[k]), k
    assert np.array_equal(got["cells"], want["cells"])

    # changed parameters: a new graph, the results of a fresh state
    got2 = copy.deepcopy(got)
    got2["dt_col_over_dV"] = got2["dt_col_over_dV"] * 2.0
    fresh = DeviceState(copy.deepcopy(got2), draws="thinned", seed=seed, precision="mixed")
    fresh.continue_philox(6)
    fresh.adv_step(1)
    want2 = fresh.snapshot()
    reset_philox_counters(seed)
    I.integrate_adv_step_np(*[got2[k] for k in I._STATE_KEYS], draws="thinned", seed=seed,
                            precision="mixed", col_step=6)
    assert I._resident[key]._plan_handle.value != plans[0]
    for k in ("xi", "m_w", "m_s", "pos", "vel", "no_cols"):
        assert np.array_equal(got2[k], want2[k]), k
    I.release_resident()
    assert not I._resident
    reset_philox_counters(seed)
    reset_philox_counters(seed + 1)


def test_concurrent_dropin_calls_from_threads():
    """Two host threads, each on its own CUDA stream, step their own states
    through integrate_adv_step_np at the same time: each equals its own
    resident DeviceState bit for bit."""
    import threading
    from lacmopy_gb300 import DeviceState
    from lacmopy_gb300 import integration as I
    from lacmopy_gb300.device import reset_philox_counters
    states = [_state(seed=51), _state(seed=52)]
    states[1]["pos"] = states[1]["pos"][:, :-3].copy()
    for k in ("vel", "rel_pos"):
        states[1][k] = states[1][k][:, :-3].copy()
    for k in ("m_w", "m_s", "xi", "T_p", "active_ids"):
        states[1][k] = states[1][k][:-3].copy()
    states[1]["cells"] = states[1]["cells"][:, :-3].copy()
    seeds = [301, 302]
    want = []
    for st, sd in zip(states, seeds):
        ds = DeviceState(copy.deepcopy(st), draws="thinned", seed=sd, precision="mixed")
        ds.adv_step(3)
        want.append(ds.snapshot())
    for sd in seeds:
        reset_philox_counters(sd)
    I.release_resident()
    got = [copy.deepcopy(st) for st in states]
    errs = []

    def run(m):
        try:
            with torch.cuda.stream(torch.cuda.Stream()):
                for _ in range(3):
                    I.integrate_adv_step_np(*[got[m][k] for k in I._STATE_KEYS], draws="thinned",
                                            seed=seeds[m], precision="mixed")
        except BaseException as ex:
            errs.append(ex)

    ths = [threading.Thread(target=run, args=(m,)) for m in range(2)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()
    torch.cuda.synchronize()
    assert not errs, errs
    for m in range(2):
        assert want[m]["no_cols"].sum() > 0
        for k in ("xi", "m_w", "m_s", "pos", "vel", "no_cols"):
            assert np.array_equal(got[m][k], want[m][k]), (m, k)
    I.release_resident()
    for sd in seeds:
        reset_philox_counters(sd)


@pytest.mark.parametrize("mode", ["engine", "kernel"])
def test_dropin_copy_paths(mode):
    """The one-call drop-in step with its host copies by the copy engines
    (one cudaMemcpyAsync per array) and by the SMs reading and writing the
    host pages directly: both equal two steps of a resident DeviceState bit
    for bit."""
    from lacmopy_gb300 import DeviceState, _lib
    from lacmopy_gb300 import integration as I
    from lacmopy_gb300.device import reset_philox_counters
    seed = 401
    st = _state(seed=55)
    key = (st["pos"].shape[1], 20, 18)
    want_ds = DeviceState(copy.deepcopy(st), draws="thinned", seed=seed, precision="mixed")
    want_ds.adv_step(2)
    want = want_ds.snapshot()
    reset_philox_counters(seed)
    I.release_resident()
    got = copy.deepcopy(st)
    I.integrate_adv_step_np(*[got[k] for k in I._STATE_KEYS], draws="thinned", seed=seed,
                            precision="mixed")
    ds = I._resident[key]
    code = _lib.COPY_ENGINE if mode == "engine" else _lib.COPY_KERNEL
    try:
        ok = ds.dropin_step(dict(zip(I._STATE_KEYS, [got[k] for k in I._STATE_KEYS])), seed,
                            "thinned", "mixed", copy_mode=code)
    except _lib.LacmoError:
        if mode == "kernel":
            pytest.skip("the device does not access pageable host memory")
        raise
    assert ok
    assert want["no_cols"].sum() > 0
    for k in ("xi", "m_w", "m_s", "pos", "vel", "rel_pos", "T_p", "grid_scalar_fields",
              "no_cols", "cells", "active_ids"):
        assert np.array_equal(got[k], want[k]), k
    I.release_resident()
    reset_philox_counters(seed)
