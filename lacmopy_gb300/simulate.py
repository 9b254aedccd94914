"""The reference's simulation drivers around the step function, on a state
kept resident on the GPU.

``simulate_interval`` keeps the argument list of integration.py:1615-1633:
one device state advances ``no_adv_steps`` advection steps, tracer particles
are recorded every ``dump_every`` steps from the device, and the caller's
arrays receive the final state.  ``simulate_frames`` is the frame loop of
integration.py:2055-2110 on a device state: each frame's r_l update, grid
fields, particle data and collision counters go to disk in the reference's
format through ``file_handling.FrameWriter`` while the steps go on.
"""
import numpy as np
import torch

from . import file_handling as fh
from .device import DeviceState
from .integration import _STATE_KEYS


def simulate_interval(grid_scalar_fields, grid_mat_prop, grid_velocity, grid_mass_flux_air_dry,
                      p_ref, p_ref_inv, grid_no_cells, grid_ranges, grid_steps, grid_volume_cell,
                      pos, vel, cells, rel_pos, m_w, m_s, xi, solute_type, water_removed, id_list,
                      active_ids, T_p, delta_m_l, dt, dt_sub, dt_sub_half, dt_col, scale_dt_cond,
                      no_col_per_adv, no_adv_steps, act_collisions, act_relaxation,
                      init_profile_r_v, init_profile_Theta, relaxation_time_profile,
                      no_iter_impl_mass, g_set, dump_every, trace_ids, traced_vectors,
                      traced_scalars, traced_xi, traced_water, E_col_grid, no_kernel_bins,
                      R_kernel_low_log, bin_factor_R_log, no_cols, *, draws="numpy", seed=1001,
                      precision="fp64", col_step=None):
    """integration.py:1615-1768 on the GPU, in place: the state is copied to
    the device once, advanced ``no_adv_steps`` steps and written back; the
    tracer records are gathered on the device before every ``dump_every``-th
    step.  ``draws``, ``seed``, ``precision`` and ``col_step`` as in
    ``integration.integrate_adv_step_np``."""
    dt_col_over_dV = dt_col / grid_volume_cell
    vals = (grid_scalar_fields, grid_mat_prop, grid_velocity, grid_mass_flux_air_dry, p_ref,
            p_ref_inv, grid_no_cells, grid_ranges, grid_steps, grid_volume_cell, pos, vel, cells,
            rel_pos, m_w, m_s, xi, solute_type, water_removed, id_list, active_ids, T_p,
            delta_m_l, dt, dt_sub, dt_sub_half, dt_col_over_dV, scale_dt_cond, no_col_per_adv,
            act_collisions, act_relaxation, init_profile_r_v, init_profile_Theta,
            relaxation_time_profile, no_iter_impl_mass, g_set, E_col_grid, no_kernel_bins,
            R_kernel_low_log, bin_factor_R_log, no_cols)
    st = dict(zip(_STATE_KEYS, vals))
    ds = DeviceState(st, draws=draws, seed=seed, precision=precision)
    philox = isinstance(draws, str) and draws in ("philox", "thinned")
    if philox:
        ds.continue_philox(col_step)
    tid = torch.as_tensor(np.asarray(trace_ids, dtype=np.int64), device=ds.device)
    dump_n = 0
    for cnt in range(int(no_adv_steps)):
        if cnt % dump_every == 0:
            tv = torch.stack([ds.pos.index_select(1, tid), ds.vel.index_select(1, tid)])
            ts = torch.stack([ds.m_w.index_select(0, tid), ds.m_s.index_select(0, tid),
                              ds.T_p.index_select(0, tid)])
            traced_vectors[dump_n] = tv.cpu().numpy()
            traced_scalars[dump_n] = ts.cpu().numpy()
            traced_xi[dump_n] = ds.xi.index_select(0, tid).cpu().numpy()
            traced_water[dump_n] = float(ds.water_removed[0])
            dump_n += 1
        ds.adv_step(1)
    if philox:
        ds.record_philox()
    ds.export_to(st)


def simulate_frames(ds, t_start, no_frames, frame_every, dt, path, graph=True, writer=None):
    """Frames of a device-resident state (integration.py:2055-2110): before
    each of ``no_frames`` intervals of ``frame_every`` steps and after the
    last one, r_l is updated and the frame is written to ``path`` (grid
    scalar fields, all particle data, collision counters) in the reference's
    format, while the steps continue on the GPU.  Returns the frame times."""
    own = writer is None
    w = fh.FrameWriter(path) if own else writer
    times = []
    try:
        for f in range(int(no_frames) + 1):
            t = t_start + f * frame_every * dt
            w.dump(ds, t)
            times.append(int(t))
            if f < no_frames:
                ds.adv_step(int(frame_every), graph=graph)
    finally:
        if own:
            w.close()
    return times
