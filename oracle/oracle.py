"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
use this module, as the checker.  Functions mirror the reference's step
functions and mutate their NumPy arguments in place like the reference does;
where the reference draws uniforms from NumPy's global generator, the oracle
takes the draw buffer explicitly (``draws``) plus a one-element int64 cursor
``pos`` that it advances.

Variants (see oracle/Makefile): ``"numba"`` (x**2 as x*x, glibc libm),
``"py"`` (x**2 as pow(x, 2) like the Numba-stubbed reference that made the
golden fixtures), ``"cr"`` (Numba semantics with the correctly-rounded
pow/log on the collision path, the GPU's math).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS = {"numba": "liblacmo_oracle.so", "py": "liblacmo_oracle_py.so",
         "cr": "liblacmo_oracle_cr.so"}
_cache = {}

D = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
I64 = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
U8 = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
i64 = ctypes.c_int64
dbl = ctypes.c_double
cint = ctypes.c_int


def build(quiet=True):
    """Compile the oracle variants with the Makefile (gcc, no GPU needed)."""
    out = subprocess.run(["make", "-C", HERE, "-s", "-j3"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


F32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")


def _lib(variant):
    if variant in _cache:
        return _cache[variant]
    path = os.path.join(HERE, _LIBS[variant])
    if not os.path.exists(path):
        build()
    lib = ctypes.CDLL(path)
    lib.orc_mass_rate_and_derivative.argtypes = [cint, i64] + [D] * 16
    lib.orc_newton_full.argtypes = [cint, i64, dbl, cint] + [D] * 16
    lib.orc_R_ws_rho.argtypes = [cint, i64, D, D, D, D, D, D]
    lib.orc_surface_tension.argtypes = [cint, i64, D, D, D]
    lib.orc_interpolate_velocity.argtypes = [I64, D, D, i64, i64, i64, D]
    lib.orc_update_velocity_Beard.argtypes = [D, D, i64]
    lib.orc_kernel_index.argtypes = [D, i64, dbl, dbl, i64, I64]
    lib.orc_radius_from_mass_col.argtypes = [D, D, i64, D]
    lib.orc_collision_step_Golovin.argtypes = [D, D, i64, dbl, I64, D]
    lib.orc_collision_step_kernel_grid_m.argtypes = [D, D, i64, dbl, D, i64, dbl, dbl, I64, D]
    lib.orc_collision_step_Ecol_grid_R.argtypes = [D, D, D, D, D, i64, dbl, D, i64, dbl, dbl, I64, D]
    lib.orc_collision_step_all_cells_2d.argtypes = [
        D, D, D, D, D, I64, i64, i64, i64, dbl, ctypes.c_void_p, dbl, i64, dbl, dbl, I64, cint,
        D, i64, I64]
    lib.orc_collision_step_all_cells_2d.restype = cint
    lib.orc_collision_pair_count.argtypes = [I64, i64, i64, i64]
    lib.orc_collision_pair_count.restype = i64
    lib.orc_propagate_particles_subloop_step.argtypes = [
        D, D, D, i64, i64, D, D, D, D, I64, D, D, D, D, D, U8, D, cint, D, i64, dbl, dbl, cint, dbl]
    lib.orc_propagate_grid_subloop_step.argtypes = [D, D, i64, i64, dbl, dbl, D, D, D, dbl]
    lib.orc_divergence_upwind.argtypes = [D, D, i64, i64, D, cint, cint, D]
    lib.orc_relaxation_term.argtypes = [D, i64, i64, D, D, dbl, D]
    lib.orc_update_grid_r_l.argtypes = [D, D, I64, D, D, U8, i64, i64, i64]
    lib.orc_integrate_adv_step.argtypes = [
        D, D, D, D, dbl, dbl, i64, i64, D, D, dbl, D, D, I64, D, D, D, D, cint, D, U8, D, D,
        dbl, dbl, dbl, dbl, cint, cint, cint, cint, D, D, D, cint, dbl, ctypes.c_void_p, dbl,
        i64, dbl, dbl, I64, ctypes.c_void_p, i64, ctypes.c_void_p, i64, ctypes.c_uint64,
        ctypes.c_void_p, cint]
    lib.orc_collision_step_all_cells_2d_philox.argtypes = [
        D, D, D, D, D, I64, i64, i64, i64, dbl, ctypes.c_void_p, dbl, i64, dbl, dbl, I64, cint,
        ctypes.c_uint64, I64, cint]
    lib.orc_collision_step_all_cells_2d_philox.restype = cint
    U64 = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
    lib.orc_philox_uniform.argtypes = [ctypes.c_uint64, U64, U64, i64, D]
    U8P = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
    lib.orc_update_cell_sum.argtypes = [cint, D, D, D, I64, i64, i64, i64, D, U8P]
    lib.orc_compute_moment_R_grid.argtypes = [i64, D, D, dbl, I64, U8P, i64, i64, i64, D]
    lib.orc_segment_bound.argtypes = [F32] * 4 + [i64, i64, i64, ctypes.c_float, ctypes.c_float]
    lib.orc_segment_bound.restype = ctypes.c_float
    lib.orc_lt_cbrtf.argtypes = [F32, i64, F32]
    lib.orc_philox_block.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                     np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")]
    lib.orc_integrate_adv_step.restype = cint
    lib.orc_set_threads.argtypes = [cint]
    lib.orc_get_threads.restype = cint
    if variant == "cr":
        I32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        lib.orc_cr_pow_array.argtypes = [D, D, i64, D, I32]
        lib.orc_cr_log_array.argtypes = [D, i64, D, I32]
    _cache[variant] = lib
    return lib


def _sol(solute_type):
    if isinstance(solute_type, (int, np.integer)):
        return int(solute_type)
    return {"AS": 0, "NaCl": 1}[str(solute_type)]


def _c(a, dt=np.float64):
    a = np.asarray(a)
    if a.dtype != dt or not a.flags.c_contiguous:
        raise TypeError(f"expected C-contiguous {dt}, got {a.dtype}")
    return a


def _E(E_col_grid):
    if isinstance(E_col_grid, (float, np.floating)):
        return None, float(E_col_grid)
    E = np.ascontiguousarray(E_col_grid, dtype=np.float64)
    return E, 0.0


class Oracle:
    def __init__(self, variant="numba"):
        self.variant = variant
        self.lib = _lib(variant)

    def set_threads(self, n):
        self.lib.orc_set_threads(int(n))

    def threads(self):
        return self.lib.orc_get_threads()

    # -- microphysics -------------------------------------------------------
    def mass_rate_and_derivative(self, sol, m_w, m_s, w_s, R_p, T_p, rho_p, T_amb, p_amb, S_amb,
                                 e_s_amb, L_v, K, D_v, sigma_p):
        n = len(m_w)
        g, dg = np.empty(n), np.empty(n)
        args = [np.ascontiguousarray(a, dtype=np.float64) for a in
                (m_w, m_s, w_s, R_p, T_p, rho_p, T_amb, p_amb, S_amb, e_s_amb, L_v, K, D_v, sigma_p)]
        self.lib.orc_mass_rate_and_derivative(_sol(sol), n, *args, g, dg)
        return g, dg

    def newton_full(self, sol, dt_sub, no_iter, m_w, m_s, w_s, R_p, T_p, rho_p, T_amb, p_amb,
                    S_amb, e_s_amb, L_v, K, D_v, sigma_p):
        n = len(m_w)
        dm, g0 = np.empty(n), np.empty(n)
        args = [np.ascontiguousarray(a, dtype=np.float64) for a in
                (m_w, m_s, w_s, R_p, T_p, rho_p, T_amb, p_amb, S_amb, e_s_amb, L_v, K, D_v, sigma_p)]
        self.lib.orc_newton_full(_sol(sol), n, float(dt_sub), int(no_iter), *args, dm, g0)
        return dm, g0

    def R_ws_rho(self, sol, m_w, m_s, T_p):
        n = len(m_w)
        R, w, r = np.empty(n), np.empty(n), np.empty(n)
        self.lib.orc_R_ws_rho(_sol(sol), n, np.ascontiguousarray(m_w, dtype=np.float64),
                              np.ascontiguousarray(m_s, dtype=np.float64),
                              np.ascontiguousarray(T_p, dtype=np.float64), R, w, r)
        return R, w, r

    def surface_tension(self, sol, w_s, T_p):
        out = np.empty(len(w_s))
        self.lib.orc_surface_tension(_sol(sol), len(w_s), np.ascontiguousarray(w_s, dtype=np.float64),
                                     np.ascontiguousarray(T_p, dtype=np.float64), out)
        return out

    def interpolate_velocity(self, cells, rel_pos, grid_vel):
        n = cells.shape[1]
        Nx, Nz = grid_vel.shape[1] - 1, grid_vel.shape[2] - 1
        out = np.empty((2, n))
        self.lib.orc_interpolate_velocity(np.ascontiguousarray(cells, dtype=np.int64),
                                          np.ascontiguousarray(rel_pos, dtype=np.float64),
                                          np.ascontiguousarray(grid_vel, dtype=np.float64),
                                          Nx, Nz, n, out)
        return out

    # -- collisions ---------------------------------------------------------
    def collision_step_Golovin_np(self, xis, masses, dt_over_dV, no_cols, draws):
        n = len(xis)
        need = n * (n - 1) // 2
        assert len(draws) >= need
        self.lib.orc_collision_step_Golovin(_c(xis), _c(masses), n, float(dt_over_dV),
                                            _c(no_cols, np.int64), _c(draws))

    def collision_step_kernel_grid_m_np(self, xis, masses, dt_over_dV, kernel_grid,
                                        no_kernel_bins, m_kernel_low_log, bin_factor_m_log,
                                        no_cols, draws):
        n = len(xis)
        assert len(draws) >= n * (n - 1) // 2
        self.lib.orc_collision_step_kernel_grid_m(
            _c(xis), _c(masses), n, float(dt_over_dV),
            np.ascontiguousarray(kernel_grid, dtype=np.float64), int(no_kernel_bins),
            float(m_kernel_low_log), float(bin_factor_m_log), _c(no_cols, np.int64), _c(draws))

    def update_velocity_Beard(self, vel, R):
        self.lib.orc_update_velocity_Beard(_c(vel), _c(R), len(vel))

    def collision_step_Ecol_grid_R_np(self, xis, masses, radii, vel, mass_densities, dt_over_dV,
                                      E_col_grid, no_kernel_bins, R_kernel_low_log,
                                      bin_factor_R_log, no_cols, draws):
        n = len(xis)
        assert len(draws) >= n * (n - 1) // 2
        self.lib.orc_collision_step_Ecol_grid_R(
            _c(xis), _c(masses), _c(radii), _c(vel), _c(mass_densities), n, float(dt_over_dV),
            np.ascontiguousarray(E_col_grid, dtype=np.float64), int(no_kernel_bins),
            float(R_kernel_low_log), float(bin_factor_R_log), _c(no_cols, np.int64), _c(draws))

    def collision_pair_count(self, cells, no_cells):
        return self.lib.orc_collision_pair_count(_c(cells, np.int64), cells.shape[1],
                                                 int(no_cells[0]), int(no_cells[1]))

    def collision_step_Ecol_grid_R_all_cells_2D_multicomp_np(
            self, xis, m_w, m_s, vel, grid_temperature, cells, no_cells, dt_over_dV, E_col_grid,
            no_kernel_bins, R_kernel_low_log, bin_factor_R_log, no_cols, solute_type, draws,
            pos=None):
        E, Ec = _E(E_col_grid)
        if pos is None:
            pos = np.zeros(1, dtype=np.int64)
        rc = self.lib.orc_collision_step_all_cells_2d(
            _c(xis), _c(m_w), _c(m_s), _c(vel), np.ascontiguousarray(grid_temperature, dtype=np.float64),
            _c(cells, np.int64), len(xis), int(no_cells[0]), int(no_cells[1]), float(dt_over_dV),
            None if E is None else E.ctypes.data, Ec, int(no_kernel_bins or 0),
            float(R_kernel_low_log or 0.0), float(bin_factor_R_log or 1.0), _c(no_cols, np.int64),
            _sol(solute_type), _c(draws), len(draws), pos)
        if rc != 0:
            raise ValueError("not enough draws for the collision step")
        return pos

    # -- particles and grid ---------------------------------------------------
    def propagate_particles_subloop_step_np(
            self, grid_scalar_fields, grid_mat_prop, grid_velocity, grid_no_cells, grid_ranges,
            grid_steps, pos, vel, cells, rel_pos, m_w, m_s, xi, water_removed, id_list,
            active_ids, T_p, solute_type, delta_m_l, dt_sub, dt_sub_pos, no_iter_impl_mass,
            g_set):
        act = active_ids.view(np.uint8)
        self.lib.orc_propagate_particles_subloop_step(
            _c(grid_scalar_fields), _c(grid_mat_prop), _c(grid_velocity), int(grid_no_cells[0]),
            int(grid_no_cells[1]), _c(np.asarray(grid_ranges, dtype=np.float64)),
            _c(np.asarray(grid_steps, dtype=np.float64)), _c(pos), _c(vel), _c(cells, np.int64),
            _c(rel_pos), _c(m_w), _c(m_s), _c(xi), _c(water_removed), act, _c(T_p),
            _sol(solute_type), _c(delta_m_l), len(xi), float(dt_sub), float(dt_sub_pos),
            int(no_iter_impl_mass), float(g_set))

    def propagate_grid_subloop_step_np(self, grid_scalar_fields, grid_mat_prop, p_ref, p_ref_inv,
                                       delta_Theta_ad, delta_r_v_ad, delta_m_l, grid_volume_cell):
        Nx, Nz = grid_scalar_fields.shape[1:]
        self.lib.orc_propagate_grid_subloop_step(
            _c(grid_scalar_fields), _c(grid_mat_prop), Nx, Nz, float(p_ref), float(p_ref_inv),
            np.ascontiguousarray(delta_Theta_ad, dtype=np.float64),
            np.ascontiguousarray(delta_r_v_ad, dtype=np.float64),
            np.ascontiguousarray(delta_m_l, dtype=np.float64), float(grid_volume_cell))

    def compute_divergence_upwind_np(self, field, flux_field, grid_no_cells, grid_steps,
                                     boundary_conditions=(0, 1)):
        Nx, Nz = int(grid_no_cells[0]), int(grid_no_cells[1])
        out = np.empty((Nx, Nz))
        self.lib.orc_divergence_upwind(np.ascontiguousarray(field, dtype=np.float64),
                                       np.ascontiguousarray(flux_field, dtype=np.float64), Nx, Nz,
                                       np.ascontiguousarray(grid_steps, dtype=np.float64),
                                       int(boundary_conditions[0]), int(boundary_conditions[1]),
                                       out)
        return out

    def compute_relaxation_term(self, field, profile0, t_relax, dt):
        Nx, Nz = field.shape
        out = np.empty(Nz)
        self.lib.orc_relaxation_term(np.ascontiguousarray(field, dtype=np.float64), Nx, Nz,
                                     np.ascontiguousarray(profile0, dtype=np.float64),
                                     np.ascontiguousarray(t_relax, dtype=np.float64), float(dt), out)
        return out

    def update_grid_r_l(self, m_w, xi, cells, grid_r_l, grid_mass_dry_inv, active_ids):
        Nx, Nz = grid_r_l.shape
        self.lib.orc_update_grid_r_l(_c(m_w), _c(xi), _c(cells, np.int64), _c(grid_r_l),
                                     np.ascontiguousarray(grid_mass_dry_inv, dtype=np.float64),
                                     active_ids.view(np.uint8), len(xi), Nx, Nz)

    def integrate_adv_step_np(
            self, grid_scalar_fields, grid_mat_prop, grid_velocity, grid_mass_flux_air_dry,
            p_ref, p_ref_inv, grid_no_cells, grid_ranges, grid_steps, grid_volume_cell, pos, vel,
            cells, rel_pos, m_w, m_s, xi, solute_type, water_removed, id_list, active_ids, T_p,
            delta_m_l, dt, dt_sub, dt_sub_half, dt_col_over_dV, scale_dt_cond, no_col_per_adv,
            act_collisions, act_relaxation, init_profile_r_v, init_profile_Theta,
            relaxation_time_profile, no_iter_impl_mass, g_set, E_col_grid, no_kernel_bins,
            R_kernel_low_log, bin_factor_R_log, no_cols, draws, draw_pos=None, seed=0,
            col_step=None, thin=False):
        """``draws``: uniform buffer consumed from ``draw_pos``, or None for
        Philox draws keyed by ``seed`` and the counter ``col_step`` (int64[1])."""
        E, Ec = _E(E_col_grid)
        Nz = int(grid_no_cells[1])
        if draw_pos is None:
            draw_pos = np.zeros(1, dtype=np.int64)
        if draws is None and col_step is None:
            col_step = np.zeros(1, dtype=np.int64)
        prof = lambda a: (np.zeros(Nz) if a is None else np.ascontiguousarray(a, dtype=np.float64))
        rc = self.lib.orc_integrate_adv_step(
            _c(grid_scalar_fields), _c(grid_mat_prop), _c(grid_velocity),
            _c(grid_mass_flux_air_dry), float(p_ref), float(p_ref_inv), int(grid_no_cells[0]), Nz,
            _c(np.asarray(grid_ranges, dtype=np.float64)), _c(np.asarray(grid_steps, dtype=np.float64)),
            float(grid_volume_cell), _c(pos), _c(vel), _c(cells, np.int64), _c(rel_pos), _c(m_w),
            _c(m_s), _c(xi), _sol(solute_type), _c(water_removed), active_ids.view(np.uint8),
            _c(T_p), _c(delta_m_l), float(dt), float(dt_sub), float(dt_sub_half),
            float(dt_col_over_dV), int(scale_dt_cond), int(no_col_per_adv), int(bool(act_collisions)),
            int(bool(act_relaxation)), prof(init_profile_r_v), prof(init_profile_Theta),
            prof(relaxation_time_profile), int(no_iter_impl_mass), float(g_set),
            None if E is None else E.ctypes.data, Ec, int(no_kernel_bins or 0),
            float(R_kernel_low_log or 0.0), float(bin_factor_R_log or 1.0), _c(no_cols, np.int64),
            None if draws is None else _c(draws).ctypes.data, 0 if draws is None else len(draws),
            draw_pos.ctypes.data, len(xi), int(seed),
            None if col_step is None else _c(col_step, np.int64).ctypes.data, int(bool(thin)))
        if rc != 0:
            raise ValueError("not enough draws for the advection step")
        return draw_pos

    def collision_step_all_cells_philox(self, xis, m_w, m_s, vel, grid_temperature, cells,
                                        no_cells, dt_over_dV, E_col_grid, no_kernel_bins,
                                        R_kernel_low_log, bin_factor_R_log, no_cols, solute_type,
                                        seed, col_step, thin=False):
        E, Ec = _E(E_col_grid)
        self.lib.orc_collision_step_all_cells_2d_philox(
            _c(xis), _c(m_w), _c(m_s), _c(vel), np.ascontiguousarray(grid_temperature, dtype=np.float64),
            _c(cells, np.int64), len(xis), int(no_cells[0]), int(no_cells[1]), float(dt_over_dV),
            None if E is None else E.ctypes.data, Ec, int(no_kernel_bins or 0),
            float(R_kernel_low_log or 0.0), float(bin_factor_R_log or 1.0), _c(no_cols, np.int64),
            _sol(solute_type), int(seed), _c(col_step, np.int64), int(bool(thin)))

    def philox_uniform(self, key, k, c1):
        """Uniforms of pair ranks ``k`` (block k >> 1, half k & 1) under
        counter word ``c1`` (collision step << 32 | cell)."""
        k = np.ascontiguousarray(k, dtype=np.uint64)
        c1 = np.ascontiguousarray(c1, dtype=np.uint64)
        out = np.empty(k.size)
        self.lib.orc_philox_uniform(int(key), k, c1, k.size, out)
        return out

    # -- diagnostics (evaluation.py) -------------------------------------------
    def update_cell_sum(self, kind, m_w, xi, cells, no_cells, mass_dry_inv, mask):
        """kind 0: update_mixing_ratio (evaluation.py:93-133); kind 1:
        update_number_concentration_per_dry_mass (:136-174); id_list = 0..N-1."""
        Nx, Nz = int(no_cells[0]), int(no_cells[1])
        out = np.empty(Nx * Nz)
        self.lib.orc_update_cell_sum(int(kind), out, _c(m_w), _c(xi), _c(cells, np.int64), len(xi),
                                     Nx, Nz, np.ascontiguousarray(mass_dry_inv, dtype=np.float64),
                                     np.ascontiguousarray(mask, dtype=np.uint8))
        return out.reshape(Nx, Nz)

    def compute_moment_R_grid(self, n, R_p, xi, V0, cells, active_ids, no_cells):
        """evaluation.py:1392-1445 with id_list = 0..N-1."""
        Nx, Nz = int(no_cells[0]), int(no_cells[1])
        out = np.empty(Nx * Nz)
        self.lib.orc_compute_moment_R_grid(int(n), _c(R_p), _c(xi), float(V0),
                                           _c(cells, np.int64),
                                           np.ascontiguousarray(active_ids, dtype=np.uint8),
                                           len(xi), Nx, Nz, out)
        return out.reshape(Nx, Nz)

    def segment_bound(self, x, R, u, w, a, lo, hi, er, dtdv):
        """lt_segment_bound of SIP a against the block [lo, hi) of the FP32
        copies x, R, u, w (lacmopy_gb300/csrc/lacmo_thin.h)."""
        f = lambda v: np.ascontiguousarray(v, dtype=np.float32)
        return float(self.lib.orc_segment_bound(f(x), f(R), f(u), f(w), int(a), int(lo), int(hi),
                                                float(er), float(dtdv)))

    def lt_cbrtf(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.empty_like(x)
        self.lib.orc_lt_cbrtf(x, x.size, out)
        return out

    def philox_block(self, key, c0, c1):
        """The raw Philox4x32-10 output block (x0, x1, x2, x3) for key and the
        128-bit counter (c0 low 64 bits, c1 high 64 bits)."""
        out = np.zeros(4, dtype=np.uint32)
        self.lib.orc_philox_block(int(key), int(c0), int(c1), out)
        return out

    # -- correctly-rounded routines (variant 'cr') -----------------------------
    def cr_pow(self, x, y):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.ascontiguousarray(np.broadcast_to(y, x.shape), dtype=np.float64)
        out = np.empty(len(x))
        hard = np.zeros(len(x), dtype=np.int32)
        self.lib.orc_cr_pow_array(x, y, len(x), out, hard)
        return out, hard

    def cr_log(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.empty(len(x))
        hard = np.zeros(len(x), dtype=np.int32)
        self.lib.orc_cr_log_array(x, len(x), out, hard)
        return out, hard
