"""Drop-in replacements for the reference's time-integration step functions.

Same names, argument lists and in-place semantics as LacmoPy's integration.py
(and grid.py / microphysics.py for the helpers), running on the GPU through
the C ABI.  NumPy arguments are copied to the device, advanced, and written
back in place; CUDA tensors stay on the device.  Extra keyword-only arguments
select the collision draw source (see lacmopy_gb300.device):

    draws="numpy"   NumPy's global generator, the reference's count and order
    draws="philox"  device Philox4x32-10 with ``seed``, one uniform per pair
    draws="thinned" the same generator, thinned draws (csrc/lacmo_thin.h)
    draws=<array>   injected uniforms

With the Philox modes, consecutive calls with the same ``seed`` continue one
stream of draws: each call starts at the collision-step counter where the
previous call with that seed stopped (``lacmopy_gb300.device.philox_counter``),
so every call draws fresh uniforms as the reference does.  ``col_step=k``
pins the counter; ``lacmopy_gb300.device.reset_philox_counters`` restarts it.

``integrate_adv_step_np`` keeps the device buffers of its last call per state
shape (SIP count and grid) and reuses them, with the captured step graph when
the parameters and draw source are the same, for the next call with NumPy
arrays of that shape: the call then copies the arrays in, steps and copies
them back without allocating.  ``release_resident()`` frees those buffers.
Calls for different states may come from several host threads, each with its
own current CUDA stream (``torch.cuda.stream``): they overlap on the GPU.

For repeated stepping keep the state on the device with
``lacmopy_gb300.DeviceState`` instead of calling these per step.
"""
import ctypes
import threading
from collections import OrderedDict

import numpy as np
import torch

from . import _lib
from .constants import solute_code
from .device import DeviceState, _ptr, _stream, to_device

_STATE_KEYS = ("grid_scalar_fields", "grid_mat_prop", "grid_velocity", "grid_mass_flux_air_dry",
               "p_ref", "p_ref_inv", "grid_no_cells", "grid_ranges", "grid_steps",
               "grid_volume_cell", "pos", "vel", "cells", "rel_pos", "m_w", "m_s", "xi",
               "solute_type", "water_removed", "id_list", "active_ids", "T_p", "delta_m_l", "dt",
               "dt_sub", "dt_sub_half", "dt_col_over_dV", "scale_dt_cond", "no_col_per_adv",
               "act_collisions", "act_relaxation", "init_profile_r_v", "init_profile_Theta",
               "relaxation_time_profile", "no_iter_impl_mass", "g_set", "E_col_grid",
               "no_kernel_bins", "R_kernel_low_log", "bin_factor_R_log", "no_cols")


def integrate_adv_step_np(grid_scalar_fields, grid_mat_prop, grid_velocity,
                          grid_mass_flux_air_dry, p_ref, p_ref_inv, grid_no_cells, grid_ranges,
                          grid_steps, grid_volume_cell, pos, vel, cells, rel_pos, m_w, m_s, xi,
                          solute_type, water_removed, id_list, active_ids, T_p, delta_m_l, dt,
                          dt_sub, dt_sub_half, dt_col_over_dV, scale_dt_cond, no_col_per_adv,
                          act_collisions, act_relaxation, init_profile_r_v, init_profile_Theta,
                          relaxation_time_profile, no_iter_impl_mass, g_set, E_col_grid,
                          no_kernel_bins, R_kernel_low_log, bin_factor_R_log, no_cols, *,
                          draws="numpy", seed=1001, precision="fp64", col_step=None):
    """One advection step dt on the GPU (integration.py:1298-1611), in place.
    ``precision="mixed"`` runs the mixed-precision sub-steps
    (lacmopy_gb300.device); with Philox draws the call continues the seed's
    stream of draws (module docstring)."""
    st = dict(zip(_STATE_KEYS, (
        grid_scalar_fields, grid_mat_prop, grid_velocity, grid_mass_flux_air_dry, p_ref,
        p_ref_inv, grid_no_cells, grid_ranges, grid_steps, grid_volume_cell, pos, vel, cells,
        rel_pos, m_w, m_s, xi, solute_type, water_removed, id_list, active_ids, T_p, delta_m_l,
        dt, dt_sub, dt_sub_half, dt_col_over_dV, scale_dt_cond, no_col_per_adv, act_collisions,
        act_relaxation, init_profile_r_v, init_profile_Theta, relaxation_time_profile,
        no_iter_impl_mass, g_set, E_col_grid, no_kernel_bins, R_kernel_low_log,
        bin_factor_R_log, no_cols)))
    # NumPy arrays only: CUDA tensors passed in are the device state itself
    host = not any(isinstance(v, torch.Tensor) for v in st.values())
    key = (np.shape(pos)[1], int(grid_no_cells[0]), int(grid_no_cells[1]))
    old = None
    if host:
        with _resident_lock:
            old = _resident.pop(key, None)
        # the state of the last call of this shape: copies in, the graph step
        # and the copies back in one native call
        if (old is not None and isinstance(draws, str)
                and old.dropin_step(st, seed, draws, precision, col_step)):
            with _resident_lock:
                _resident[key] = old
            return
    ds = DeviceState(st, draws=draws, seed=seed, precision=precision, reuse=old)
    philox = isinstance(draws, str) and draws in ("philox", "thinned")
    if philox:
        ds.continue_philox(col_step)
    ds.adv_step(1, graph=philox)
    if philox:
        ds.record_philox()
    ds.export_to(st)
    if host:
        with _resident_lock:
            _resident[key] = ds
            while len(_resident) > _RESIDENT_MAX:
                _resident.popitem(last=False)


# the device states of the last integrate_adv_step_np calls with NumPy arrays,
# by (SIP count, nx, nz), oldest first; their buffers serve the next call of
# the same shape.  Calls from several host threads (each on its own current
# CUDA stream) run concurrently: a call takes its shape's state out of the
# table for its duration.
_resident = OrderedDict()
_resident_lock = threading.Lock()
_RESIDENT_MAX = 8


def release_resident():
    """Free the device buffers integrate_adv_step_np keeps between calls."""
    with _resident_lock:
        _resident.clear()


def propagate_particles_subloop_step_np(grid_scalar_fields, grid_mat_prop, grid_velocity,
                                        grid_no_cells, grid_ranges, grid_steps, pos, vel, cells,
                                        rel_pos, m_w, m_s, xi, water_removed, id_list, active_ids,
                                        T_p, solute_type, delta_m_l, dt_sub, dt_sub_pos,
                                        no_iter_impl_mass, g_set):
    """One particle sub-step on the GPU (integration.py:944-1091), in place."""
    Nx, Nz = int(grid_no_cells[0]), int(grid_no_cells[1])
    st = dict(grid_scalar_fields=grid_scalar_fields, grid_mat_prop=grid_mat_prop,
              grid_velocity=grid_velocity,
              grid_mass_flux_air_dry=np.zeros((2, Nx + 1, Nz + 1)), p_ref=1e5, p_ref_inv=1e-5,
              grid_no_cells=grid_no_cells, grid_ranges=grid_ranges, grid_steps=grid_steps,
              grid_volume_cell=float(grid_steps[0]) * float(grid_steps[1]), pos=pos, vel=vel,
              cells=cells, rel_pos=rel_pos, m_w=m_w, m_s=m_s, xi=xi, solute_type=solute_type,
              water_removed=water_removed, active_ids=active_ids, T_p=T_p, delta_m_l=delta_m_l,
              dt=1.0, dt_sub=dt_sub, dt_sub_half=0.5 * dt_sub, dt_col_over_dV=0.0,
              scale_dt_cond=1, no_col_per_adv=2, act_collisions=False, act_relaxation=False,
              init_profile_r_v=None, init_profile_Theta=None, relaxation_time_profile=None,
              no_iter_impl_mass=no_iter_impl_mass, g_set=g_set, E_col_grid=0.5,
              no_kernel_bins=None, R_kernel_low_log=None, bin_factor_R_log=None)
    ds = DeviceState(st, draws="philox")
    ds.particles_substep(dt_sub, dt_sub_pos)
    ds.export_to(st)


def propagate_grid_subloop_step_np(grid_scalar_fields, grid_mat_prop, p_ref, p_ref_inv,
                                   delta_Theta_ad, delta_r_v_ad, delta_m_l, grid_volume_cell):
    """One grid sub-step on the GPU (integration.py:402-484), in place."""
    lib = _lib.load()
    Nx, Nz = np.shape(grid_scalar_fields)[1:]
    gsf = to_device(grid_scalar_fields)
    gmp = to_device(grid_mat_prop)
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    g = _lib.Grid(Nx, Nz, gsf.data_ptr(), gmp.data_ptr(), dummy.data_ptr(), dummy.data_ptr(),
                  dummy.data_ptr(), 0.0, 1.0, 0.0, 1.0, 1.0, 1.0, float(grid_volume_cell),
                  float(p_ref), float(p_ref_inv))
    a, b, c = (to_device(x) for x in (delta_Theta_ad, delta_r_v_ad, delta_m_l))
    _lib.check(lib.lacmo_propagate_grid_subloop_step(ctypes.byref(g), _ptr(a), _ptr(b), _ptr(c),
                                                     _stream()), "propagate_grid_subloop_step")
    _writeback(grid_scalar_fields, gsf)
    _writeback(grid_mat_prop, gmp)


def compute_divergence_upwind_np(field, flux_field, grid_no_cells, grid_steps,
                                 boundary_conditions=np.array([0, 1])):
    """integration.py:150-287 on the GPU; returns a new [Nx, Nz] array."""
    lib = _lib.load()
    Nx, Nz = int(grid_no_cells[0]), int(grid_no_cells[1])
    f, fl = to_device(field), to_device(flux_field)
    out = torch.empty((Nx, Nz), dtype=torch.float64, device="cuda")
    _lib.check(lib.lacmo_divergence_upwind(_ptr(f), _ptr(fl), Nx, Nz, float(grid_steps[0]),
                                           float(grid_steps[1]), int(boundary_conditions[0]),
                                           int(boundary_conditions[1]), _ptr(out), _stream()),
               "divergence_upwind")
    return _result(field, out)


def compute_relaxation_term(field, profile0, t_relax, dt):
    """integration.py:325-354 on the GPU; returns a new [Nz] array."""
    lib = _lib.load()
    Nx, Nz = np.shape(field)
    f, p, t = to_device(field), to_device(profile0), to_device(t_relax)
    out = torch.empty(Nz, dtype=torch.float64, device="cuda")
    _lib.check(lib.lacmo_relaxation_term(_ptr(f), Nx, Nz, _ptr(p), _ptr(t), float(dt), _ptr(out),
                                         _stream()), "relaxation_term")
    return _result(field, out)


def interpolate_velocity_from_cell_bilinear(cells, rel_pos, grid_vel, grid_no_cells):
    """grid.py:257-323 on the GPU (active cells, j >= 0); returns [2, n]."""
    lib = _lib.load()
    Nx, Nz = int(grid_no_cells[0]), int(grid_no_cells[1])
    cells_np = np.asarray(cells)
    n = cells_np.shape[1]
    cell = to_device(np.where(cells_np[1] >= 0, cells_np[0] * Nz + cells_np[1], -1 - cells_np[0]),
                     torch.int32)
    rel, gv = to_device(rel_pos), to_device(grid_vel)
    out = torch.empty((2, n), dtype=torch.float64, device="cuda")
    _lib.check(lib.lacmo_interpolate_velocity(_ptr(cell), _ptr(rel), _ptr(gv), n, Nx, Nz,
                                              _ptr(out), _stream()), "interpolate_velocity")
    return _result(rel_pos, out)


def _mass_rate_args(m_w, m_s, w_s, R_p, T_p, rho_p, T_amb, p_amb, S_amb, e_s_amb, L_v, K, D_v,
                    sigma_p):
    arrs = [to_device(np.atleast_1d(a)) for a in
            (m_w, m_s, w_s, R_p, T_p, rho_p, T_amb, p_amb, S_amb, e_s_amb, L_v, K, D_v, sigma_p)]
    n = max(a.numel() for a in arrs)
    arrs = [a.expand(n).contiguous() if a.numel() == 1 and n > 1 else a for a in arrs]
    return n, arrs


def compute_mass_rate_and_derivative_np(solute_type, m_w, m_s, w_s, R_p, T_p, rho_p, T_amb,
                                        p_amb, S_amb, e_s_amb, L_v, K, D_v, sigma_p):
    """microphysics.py:1359 (AS) / :1239 (NaCl), elementwise on the GPU."""
    lib = _lib.load()
    n, arrs = _mass_rate_args(m_w, m_s, w_s, R_p, T_p, rho_p, T_amb, p_amb, S_amb, e_s_amb, L_v,
                              K, D_v, sigma_p)
    g = torch.empty(n, dtype=torch.float64, device="cuda")
    dg = torch.empty_like(g)
    _lib.check(lib.lacmo_mass_rate_and_derivative(solute_code(solute_type), n,
                                                  *[_ptr(a) for a in arrs], _ptr(g), _ptr(dg),
                                                  _stream()), "mass_rate_and_derivative")
    return g.cpu().numpy(), dg.cpu().numpy()


def compute_mass_rate_and_derivative_AS_np(*args):
    return compute_mass_rate_and_derivative_np("AS", *args)


def compute_mass_rate_and_derivative_NaCl_np(*args):
    return compute_mass_rate_and_derivative_np("NaCl", *args)


def compute_dml_and_gamma_impl_Newton_full_np(dt_sub, no_iter_impl_mass, m_w, m_s, w_s, R_p, T_p,
                                              rho_p, T_amb, p_amb, S_amb, e_s_amb, L_v, K, D_v,
                                              sigma_p, solute_type):
    """integration.py:728-836, elementwise on the GPU; returns (dm, gamma0)."""
    lib = _lib.load()
    n, arrs = _mass_rate_args(m_w, m_s, w_s, R_p, T_p, rho_p, T_amb, p_amb, S_amb, e_s_amb, L_v,
                              K, D_v, sigma_p)
    dm = torch.empty(n, dtype=torch.float64, device="cuda")
    g0 = torch.empty_like(dm)
    _lib.check(lib.lacmo_newton_full(solute_code(solute_type), n, float(dt_sub),
                                     int(no_iter_impl_mass), *[_ptr(a) for a in arrs], _ptr(dm),
                                     _ptr(g0), _stream()), "newton_full")
    return dm.cpu().numpy(), g0.cpu().numpy()


def update_grid_r_l_np(m_w, xi, cells, grid_r_l, grid_mass_dry_inv, active_ids, id_list=None):
    """grid.py:370-412 on the GPU, in place on ``grid_r_l``."""
    Nx, Nz = np.shape(grid_r_l)
    n = np.shape(m_w)[0]
    gsf = np.zeros((10, Nx, Nz))
    gsf[8] = grid_mass_dry_inv
    st = _minimal_state(Nx, Nz, n, m_w=m_w, xi=xi, cells=cells, active_ids=active_ids, gsf=gsf)
    ds = DeviceState(st, draws="philox")
    ds.update_grid_r_l()
    np.copyto(grid_r_l, ds.gsf[5].cpu().numpy())


def _minimal_state(Nx, Nz, n, m_w, xi, cells, active_ids, gsf=None, m_s=None, vel=None):
    return dict(grid_scalar_fields=np.zeros((10, Nx, Nz)) if gsf is None else gsf,
                grid_mat_prop=np.zeros((7, Nx, Nz)), grid_velocity=np.zeros((2, Nx + 1, Nz + 1)),
                grid_mass_flux_air_dry=np.zeros((2, Nx + 1, Nz + 1)), p_ref=1e5, p_ref_inv=1e-5,
                grid_no_cells=np.array([Nx, Nz]), grid_ranges=np.array([[0., 1.], [0., 1.]]),
                grid_steps=np.array([1.0, 1.0]), grid_volume_cell=1.0,
                pos=np.zeros((2, n)), vel=np.zeros((2, n)) if vel is None else vel,
                cells=cells, rel_pos=np.zeros((2, n)), m_w=m_w,
                m_s=np.zeros(n) if m_s is None else m_s, xi=xi, solute_type="AS",
                water_removed=np.zeros(1), active_ids=active_ids, T_p=np.zeros(n),
                delta_m_l=np.zeros((Nx, Nz)), dt=1.0, dt_sub=0.1, dt_sub_half=0.05,
                dt_col_over_dV=1.0, scale_dt_cond=1, no_col_per_adv=2, act_collisions=True,
                act_relaxation=False, init_profile_r_v=None, init_profile_Theta=None,
                relaxation_time_profile=None, no_iter_impl_mass=3, g_set=0.0, E_col_grid=0.5,
                no_kernel_bins=None, R_kernel_low_log=None, bin_factor_R_log=None)


def _writeback(dst, t):
    if isinstance(dst, torch.Tensor):
        if dst.data_ptr() != t.data_ptr():
            dst.copy_(t.reshape(dst.shape))
    else:
        np.copyto(dst, t.cpu().numpy().reshape(np.shape(dst)))


def _result(like, t):
    return t if isinstance(like, torch.Tensor) else t.cpu().numpy()
