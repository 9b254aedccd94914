"""Drop-in replacements for collision/all_or_nothing.py and the box-model
collision driver, running the all-or-nothing step on the GPU.

Same names, arguments and in-place semantics as the reference; keyword-only
``draws`` selects the uniform draws ("numpy": NumPy's global generator with
the reference's count and order, "philox": device Philox with ``seed`` and
``step``, or an explicit array).  Collision decisions and multiplicity/mass
updates are bit-exact with the reference given the same draws (see the
kernel file k_collision.cu for how).
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib
from .device import DeviceState, _ptr, _stream, to_device
from .integration import _minimal_state, _writeback


def _box_draws(draws, n):
    need = n * (n - 1) // 2
    if isinstance(draws, str):
        if draws == "numpy":
            return to_device(np.random.rand(need) if need else np.zeros(1))
        if draws == "philox":
            return None
        raise ValueError(f"unknown draw source {draws!r}")
    t = to_device(draws)
    if t.numel() < need:
        raise ValueError(f"need {need} draws, got {t.numel()}")
    return t


def collision_step_Golovin_np(xis, masses, dt_over_dV, no_cols, *, draws="numpy", seed=0,
                              step=0):
    """collision/all_or_nothing.py:109-185 (Golovin kernel, box model)."""
    lib = _lib.load()
    n = int(np.shape(xis)[0])
    x, m, nc = to_device(xis), to_device(masses), to_device(no_cols, torch.int64)
    r = _box_draws(draws, n)
    _lib.check(lib.lacmo_collision_step_golovin(_ptr(x), _ptr(m), n, float(dt_over_dV), _ptr(nc),
                                                _ptr(r), int(seed), int(step), _stream()),
               "collision_step_golovin")
    for dst, t in ((xis, x), (masses, m), (no_cols, nc)):
        _writeback(dst, t)


def collision_step_kernel_grid_m_np(xis, masses, dt_over_dV, kernel_grid, no_kernel_bins,
                                    m_kernel_low_log, bin_factor_m_log, no_cols, *,
                                    draws="numpy", seed=0, step=0):
    """collision/all_or_nothing.py:392-491 (kernel K(m1, m2) on a logarithmic
    mass grid, box model)."""
    lib = _lib.load()
    n = int(np.shape(xis)[0])
    x, m, nc = to_device(xis), to_device(masses), to_device(no_cols, torch.int64)
    K = to_device(kernel_grid)
    r = _box_draws(draws, n)
    _lib.check(lib.lacmo_collision_step_kernel_grid_m(
        _ptr(x), _ptr(m), n, float(dt_over_dV), _ptr(K), int(no_kernel_bins),
        float(m_kernel_low_log), float(bin_factor_m_log), _ptr(nc), _ptr(r), int(seed), int(step),
        _stream()), "collision_step_kernel_grid_m")
    for dst, t in ((xis, x), (masses, m), (no_cols, nc)):
        _writeback(dst, t)


def collision_step_Ecol_grid_R_np(xis, masses, radii, vel, mass_densities, dt_over_dV,
                                  E_col_grid, no_kernel_bins, R_kernel_low_log, bin_factor_R_log,
                                  no_cols, *, draws="numpy", seed=0, step=0):
    """collision/all_or_nothing.py:269-390 (E_col(R1,R2) table, box model)."""
    lib = _lib.load()
    n = int(np.shape(xis)[0])
    x, m, R = to_device(xis), to_device(masses), to_device(radii)
    v, rho, E = to_device(vel), to_device(mass_densities), to_device(E_col_grid)
    nc = to_device(no_cols, torch.int64)
    r = _box_draws(draws, n)
    _lib.check(lib.lacmo_collision_step_ecol_grid_r_box(
        _ptr(x), _ptr(m), _ptr(R), _ptr(v), _ptr(rho), n, float(dt_over_dV), _ptr(E),
        int(no_kernel_bins), float(R_kernel_low_log), float(bin_factor_R_log), _ptr(nc), _ptr(r),
        int(seed), int(step), _stream()), "collision_step_ecol_grid_r_box")
    for dst, t in ((xis, x), (masses, m), (radii, R), (no_cols, nc)):
        _writeback(dst, t)


def update_velocity_Beard(vel, R):
    """collision/kernel.py:193-210 (Beard terminal velocity), in place."""
    lib = _lib.load()
    v, r = to_device(vel), to_device(R)
    _lib.check(lib.lacmo_update_velocity_beard(_ptr(v), _ptr(r), v.numel(), _stream()),
               "update_velocity_beard")
    _writeback(vel, v)


def collision_step_Ecol_grid_R_all_cells_2D_multicomp_np(
        xis, m_w, m_s, vel, grid_temperature, cells, no_cells, dt_over_dV, E_col_grid,
        no_kernel_bins, R_kernel_low_log, bin_factor_R_log, no_cols, solute_type, *,
        draws="numpy", seed=0, col_step=None):
    """collision/all_or_nothing.py:754-846: one AON step in every grid cell.

    With ``draws="philox"`` or ``"thinned"`` consecutive calls with the same
    ``seed`` continue one stream of draws (lacmopy_gb300.integration);
    ``col_step`` pins the collision-step counter."""
    Nx, Nz = int(no_cells[0]), int(no_cells[1])
    n = int(np.shape(xis)[0])
    cells_np = np.asarray(cells)
    act = (cells_np[1] >= 0) & (cells_np[1] < Nz) & (cells_np[0] >= 0) & (cells_np[0] < Nx)
    gsf = np.zeros((10, Nx, Nz))
    gsf[0] = np.asarray(grid_temperature)
    st = _minimal_state(Nx, Nz, n, m_w=m_w, xi=xis, cells=np.where(act, cells_np, 0),
                        active_ids=act, gsf=gsf, m_s=m_s, vel=vel)
    st.update(dt_col_over_dV=dt_over_dV, E_col_grid=E_col_grid, no_kernel_bins=no_kernel_bins,
              R_kernel_low_log=R_kernel_low_log, bin_factor_R_log=bin_factor_R_log,
              solute_type=solute_type, no_cols=no_cols)
    mode = draws if isinstance(draws, str) else "philox"
    ds = DeviceState(st, draws=mode, seed=seed)
    philox = isinstance(draws, str) and draws in ("philox", "thinned")
    if philox:
        ds.continue_philox(col_step)
    ds.collision_step(None if isinstance(draws, str) else draws)
    if philox:
        ds.record_philox()
    torch.cuda.current_stream().synchronize()
    for dst, t in ((xis, ds.xi), (m_w, ds.m_w), (m_s, ds.m_s), (no_cols, ds.no_cols)):
        _writeback(dst, t)


def compute_radius_and_kernel_index(masses, mass_densities, R_kernel_low_log, bin_factor_R_log,
                                    no_kernel_bins):
    """Collision-path radius (microphysics.py:83-100) and kernel bin
    (collision/all_or_nothing.py:35-67), correctly rounded; returns (R, bin)."""
    lib = _lib.load()
    m, rho = to_device(masses), to_device(mass_densities)
    R = torch.empty_like(m)
    k = torch.empty(m.numel(), dtype=torch.int64, device=m.device)
    _lib.check(lib.lacmo_radius_and_bin(_ptr(m), _ptr(rho), m.numel(), float(R_kernel_low_log),
                                        float(bin_factor_R_log), int(no_kernel_bins), _ptr(R),
                                        _ptr(k), _stream()), "radius_and_bin")
    return R.cpu().numpy(), k.cpu().numpy()


def simulate_collisions(SIP_quantities, kernel_quantities, kernel_name, kernel_method, dV, dt,
                        t_end, dt_save, no_cols, seed, save_dir=None, *, draws="numpy"):
    """Box-model time loop (collision/box_model.py:44-205) on the GPU.

    The state stays on the device between steps; the saved (xis, masses)
    snapshots and save times are returned (and written to ``save_dir`` with the
    reference's file names when it is given).  ``draws="numpy"`` seeds NumPy's
    global generator with ``seed`` like the reference; ``"philox"`` uses the
    device generator keyed by ``seed``.
    """
    lib = _lib.load()
    if draws == "numpy":
        np.random.seed(seed)
    # box_model.py:135-145 picks the step by kernel_name first, then loops by
    # kernel_method (:160-194); the Golovin kernel runs with any method but the
    # two tabulated ones
    if kernel_name == "Golovin" and kernel_method not in ("Ecol_grid_R", "kernel_grid_m"):
        method = "golovin"
        xis, masses = SIP_quantities
    elif kernel_method == "Ecol_grid_R":
        method = "ecol"
        xis, masses, radii, vel, mass_densities = SIP_quantities
        E_col_grid, no_kernel_bins, R_kernel_low_log, bin_factor_R_log = kernel_quantities
    elif kernel_method == "kernel_grid_m":
        method = "kgrid"
        xis, masses = SIP_quantities
        kernel_grid, no_kernel_bins, m_kernel_low_log, bin_factor_m_log = kernel_quantities
    else:
        raise ValueError(f"kernel_name {kernel_name!r} with kernel_method {kernel_method!r}")
    n = int(np.shape(xis)[0])
    no_steps = int(math.ceil(t_end / dt))
    no_saves = int(t_end / dt_save - 0.001) + 2
    dn_save = int(math.ceil(dt_save / dt))
    dt_over_dV = dt / dV
    x, m, nc = to_device(xis), to_device(masses), to_device(no_cols, torch.int64)
    if method == "ecol":
        R, v, rho, E = (to_device(a) for a in (radii, vel, mass_densities, E_col_grid))
    elif method == "kgrid":
        K = to_device(kernel_grid)
    xis_vs_time = np.zeros((no_saves, n))
    masses_vs_time = np.zeros((no_saves, n))
    save_times = np.zeros(no_saves)
    save_n = 0
    s = _stream()
    for step_n in range(no_steps):
        if step_n % dn_save == 0:
            xis_vs_time[save_n] = x.cpu().numpy()
            masses_vs_time[save_n] = m.cpu().numpy()
            save_times[save_n] = step_n * dt
            save_n += 1
        r = _box_draws(draws, n)
        if method == "golovin":
            _lib.check(lib.lacmo_collision_step_golovin(_ptr(x), _ptr(m), n, dt_over_dV, _ptr(nc),
                                                        _ptr(r), int(seed), step_n, s), "golovin")
        elif method == "kgrid":
            # no velocity update: the kernel table holds the whole K(m1, m2)
            _lib.check(lib.lacmo_collision_step_kernel_grid_m(
                _ptr(x), _ptr(m), n, dt_over_dV, _ptr(K), int(no_kernel_bins),
                float(m_kernel_low_log), float(bin_factor_m_log), _ptr(nc), _ptr(r), int(seed),
                step_n, s), "kernel_grid_m")
        else:
            _lib.check(lib.lacmo_collision_step_ecol_grid_r_box(
                _ptr(x), _ptr(m), _ptr(R), _ptr(v), _ptr(rho), n, dt_over_dV, _ptr(E),
                int(no_kernel_bins), float(R_kernel_low_log), float(bin_factor_R_log), _ptr(nc),
                _ptr(r), int(seed), step_n, s), "ecol_box")
            _lib.check(lib.lacmo_update_velocity_beard(_ptr(v), _ptr(R), n, s), "beard")
    xis_vs_time[save_n] = x.cpu().numpy()
    masses_vs_time[save_n] = m.cpu().numpy()
    save_times[save_n] = no_steps * dt
    _writeback(xis, x)
    _writeback(masses, m)
    _writeback(no_cols, nc)
    if method == "ecol":
        _writeback(radii, R)
        _writeback(vel, v)
    if save_dir is not None:
        np.save(save_dir + f"xis_vs_time_{seed}", xis_vs_time)
        np.save(save_dir + f"masses_vs_time_{seed}", masses_vs_time)
        np.save(save_dir + f"save_times_{seed}", save_times)
    return xis_vs_time, masses_vs_time, save_times
