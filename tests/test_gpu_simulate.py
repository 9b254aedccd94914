"""The simulation drivers on the GPU: simulate_interval (integration.py:1615)
against the step function called step by step, and the frame writer
(integration.py:2055-2110 frames) against snapshots of the same run."""
import copy

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
DT_COL = 60.0


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from lacmopy_gb300 import build
    build.build()


def _state(seed=51):
    from lacmopy_gb300 import synthetic
    st = synthetic.make_icmw_state(Nx=16, Nz=14, no_spcm=(8, 10), seed=seed,
                                   kernel_type="Hall_Bott", drizzle_fraction=0.3, r_tot=12.5E-3)
    # collision time step 60 s (dt_col / V exactly as simulate_interval forms it)
    st["dt_col_over_dV"] = DT_COL / st["grid_volume_cell"]
    return st


def test_simulate_interval_equals_stepwise_calls():
    from lacmopy_gb300 import integration as I
    from lacmopy_gb300.device import reset_philox_counters
    from lacmopy_gb300.simulate import simulate_interval
    seed, steps, dump_every = 313, 4, 2
    st = _state()
    trace = np.arange(5, st["xi"].size, 97)
    # step by step through the drop-in step function, tracers recorded by hand
    a = copy.deepcopy(st)
    reset_philox_counters(seed)
    rec = []
    for cnt in range(steps):
        if cnt % dump_every == 0:
            rec.append((a["pos"][:, trace].copy(), a["vel"][:, trace].copy(),
                        a["m_w"][trace].copy(), a["xi"][trace].copy(),
                        float(a["water_removed"][0])))
        I.integrate_adv_step_np(*[a[k] for k in I._STATE_KEYS], draws="philox", seed=seed)
    # the interval driver
    b = copy.deepcopy(st)
    reset_philox_counters(seed)
    nd = steps // dump_every
    tv = np.zeros((nd, 2, 2, trace.size)); ts = np.zeros((nd, 3, trace.size))
    tx = np.zeros((nd, trace.size)); tw = np.zeros(nd)
    args = [b[k] for k in I._STATE_KEYS]
    # simulate_interval takes dt_col (not dt_col / V) and the step count
    kw = dict(zip(I._STATE_KEYS, args))
    simulate_interval(
        kw["grid_scalar_fields"], kw["grid_mat_prop"], kw["grid_velocity"],
        kw["grid_mass_flux_air_dry"], kw["p_ref"], kw["p_ref_inv"], kw["grid_no_cells"],
        kw["grid_ranges"], kw["grid_steps"], kw["grid_volume_cell"], kw["pos"], kw["vel"],
        kw["cells"], kw["rel_pos"], kw["m_w"], kw["m_s"], kw["xi"], kw["solute_type"],
        kw["water_removed"], kw["id_list"], kw["active_ids"], kw["T_p"], kw["delta_m_l"],
        kw["dt"], kw["dt_sub"], kw["dt_sub_half"], DT_COL,
        kw["scale_dt_cond"], kw["no_col_per_adv"], steps, kw["act_collisions"],
        kw["act_relaxation"], kw["init_profile_r_v"], kw["init_profile_Theta"],
        kw["relaxation_time_profile"], kw["no_iter_impl_mass"], kw["g_set"], dump_every, trace,
        tv, ts, tx, tw, kw["E_col_grid"], kw["no_kernel_bins"], kw["R_kernel_low_log"],
        kw["bin_factor_R_log"], kw["no_cols"], draws="philox", seed=seed)
    reset_philox_counters(seed)
    assert a["no_cols"].sum() > 0
    assert np.array_equal(b["no_cols"], a["no_cols"])
    for k in ("pos", "vel", "m_w", "m_s", "xi", "cells", "water_removed"):
        assert np.array_equal(b[k], a[k]), k
    for d, (p, v, mw, x, w) in enumerate(rec):
        assert np.array_equal(tv[d, 0], p) and np.array_equal(tv[d, 1], v)
        assert np.array_equal(ts[d, 0], mw) and np.array_equal(tx[d], x)
        assert tw[d] == w


def test_frame_writer_matches_snapshots(tmp_path):
    from lacmopy_gb300 import DeviceState
    from lacmopy_gb300 import file_handling as fh
    from lacmopy_gb300.simulate import simulate_frames
    st = _state(seed=52)
    seed = 99
    ds = DeviceState(copy.deepcopy(st), draws="philox", seed=seed)
    path = str(tmp_path) + "/"
    times = simulate_frames(ds, 0, 2, 2, 1.0, path, graph=True)
    assert times == [0, 2, 4]
    ref = DeviceState(copy.deepcopy(st), draws="philox", seed=seed)
    snaps = []
    for f in range(3):
        ref.update_grid_r_l()
        snaps.append(ref.snapshot())
        if f < 2:
            ref.adv_step(2)
    vec, cells, scal, xi, act = fh.load_particle_data_all(path, times)
    fields = fh.load_grid_scalar_fields(path, times)
    for f, sn in enumerate(snaps):
        assert np.array_equal(vec[f, 0], sn["pos"]) and np.array_equal(vec[f, 1], sn["vel"])
        assert np.array_equal(cells[f], sn["cells"])
        assert np.array_equal(scal[f, 0], sn["m_w"]) and np.array_equal(scal[f, 1], sn["m_s"])
        assert np.array_equal(xi[f], sn["xi"]) and np.array_equal(act[f], sn["active_ids"])
        g = sn["grid_scalar_fields"]
        assert np.array_equal(fields[f], np.array([g[4], g[5], g[2], g[0], g[1], g[6]]))
        assert np.array_equal(np.load(path + f"no_cols_{times[f]}.npy"), sn["no_cols"])
    assert snaps[-1]["no_cols"].sum() > 0
