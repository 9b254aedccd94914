"""ctypes binding of liblacmo_gb300.so (the C ABI in include/lacmo_gb300.h).

Loading fails loudly: there is no CPU fallback for any entry point.  The
structs mirror the header; every pointer is a device address.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblacmo_gb300.so")

OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA runtime error", -3: "injected draw buffer too short",
          -4: "workspace missing or too small", -5: "size above the fixed capacity"}
FLAG_DRAWS_SHORT = 0x1
FLAG_CELL_CLAMPED = 0x2
FLAG_NONFINITE = 0x4
FLAG_CELL_TOO_BIG = 0x8
FLAG_CELL_RANGE = 0x10
FLAG_SYNC_TIMEOUT = 0x20
FLAG_ACC_RANGE = 0x40
NOALLOC_MAX_SIPS = 524288
NOALLOC_MAX_CELLS = 16384
BOX_MAX_SIPS = 8192
ECOL_BOX_MAX_SIPS = 4096

vp = ctypes.c_void_p
i64 = ctypes.c_int64
i32 = ctypes.c_int32
dbl = ctypes.c_double
u64 = ctypes.c_uint64
sz = ctypes.c_size_t


class Sips(ctypes.Structure):
    _fields_ = [("n", i64), ("pos", vp), ("vel", vp), ("rel_pos", vp), ("m_w", vp), ("m_s", vp),
                ("xi", vp), ("T_p", vp), ("cell", vp), ("water_removed", vp), ("no_cols", vp)]


class Grid(ctypes.Structure):
    _fields_ = [("nx", i64), ("nz", i64), ("scalar_fields", vp), ("mat_prop", vp),
                ("velocity", vp), ("mass_flux_air_dry", vp), ("delta_m_l", vp),
                ("x_min", dbl), ("x_max", dbl), ("z_min", dbl), ("z_max", dbl), ("dx", dbl),
                ("dz", dbl), ("volume_cell", dbl), ("p_ref", dbl), ("p_ref_inv", dbl)]


class Params(ctypes.Structure):
    _fields_ = [("dt", dbl), ("dt_sub", dbl), ("dt_sub_half", dbl), ("dt_col_over_dV", dbl),
                ("g_set", dbl), ("scale_dt_cond", i32), ("no_col_per_adv", i32),
                ("act_collisions", i32), ("act_relaxation", i32), ("no_iter_impl_mass", i32),
                ("solute", i32), ("init_profile_r_v", vp), ("init_profile_Theta", vp),
                ("relaxation_time_profile", vp), ("E_col_grid", vp), ("E_col_const", dbl),
                ("no_kernel_bins", i64), ("R_kernel_low_log", dbl), ("bin_factor_R_log", dbl),
                ("precision", i32), ("thin_draws", i32)]


TUNE_PARTICLE_BLOCKS = 0
TUNE_COLLISION_BLOCKS = 1
TUNE_ORDER_CTAS = 2
PRECISION_FP64 = 0
PRECISION_MIXED = 1


class Draws(ctypes.Structure):
    _fields_ = [("draws", vp), ("n_draws", i64), ("seed", u64)]


class Copy(ctypes.Structure):
    _fields_ = [("dst", vp), ("src", vp), ("bytes", i64)]


class Dropin(ctypes.Structure):
    _fields_ = [("in_", ctypes.POINTER(Copy)), ("n_in", i32), ("out", ctypes.POINTER(Copy)),
                ("n_out", i32), ("sips", ctypes.POINTER(Sips)), ("grid", ctypes.POINTER(Grid)),
                ("prm", ctypes.POINTER(Params)), ("draws", ctypes.POINTER(Draws)), ("ws", vp),
                ("ws_bytes", ctypes.c_size_t), ("cells_in", vp), ("active_in", vp),
                ("cells_out", vp), ("active_out", vp), ("plan", vp), ("col_step", i64),
                ("col_step_out", ctypes.POINTER(i64)), ("copy_mode", i32)]


COPY_AUTO, COPY_ENGINE, COPY_KERNEL = 0, 1, 2


P = ctypes.POINTER
# name -> (restype, argtypes)
PROTOTYPES = {
    "lacmo_abi_version": (ctypes.c_int, []),
    "lacmo_kernel_launches": (ctypes.c_uint64, []),
    "lacmo_tune_options": (ctypes.c_int, [ctypes.c_int, P(ctypes.c_int), ctypes.c_int]),
    "lacmo_tune_set": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "lacmo_tune_get": (ctypes.c_int, [ctypes.c_int]),
    "lacmo_particles_only": (ctypes.c_int, [P(Sips), P(Grid), P(Params), dbl, dbl, vp, sz, vp]),
    "lacmo_bin": (ctypes.c_int, [P(Sips), P(Grid), vp, sz, vp]),
    "lacmo_error_string": (ctypes.c_char_p, [ctypes.c_int]),
    "lacmo_workspace_bytes": (sz, [i64, i64, i64]),
    "lacmo_workspace_reset": (ctypes.c_int, [vp, sz, i64, i64, i64, vp]),
    "lacmo_read_flags": (ctypes.c_int, [vp, i64, i64, i64, P(ctypes.c_uint32), vp]),
    "lacmo_get_collision_step": (ctypes.c_int, [vp, i64, i64, i64, P(i64), vp]),
    "lacmo_set_collision_step": (ctypes.c_int, [vp, i64, i64, i64, i64, vp]),
    "lacmo_read_fallbacks": (ctypes.c_int, [vp, i64, i64, i64, P(ctypes.c_uint64), vp]),
    "lacmo_cells_import": (ctypes.c_int, [vp, vp, vp, i64, i64, i64, vp]),
    "lacmo_cells_export": (ctypes.c_int, [vp, vp, vp, vp, vp, i64, i64, i64, dbl, dbl, dbl, dbl,
                                          vp]),
    "lacmo_prepare": (ctypes.c_int, [P(Sips), P(Grid), P(Params), vp, sz, vp]),
    "lacmo_integrate_adv_step": (ctypes.c_int, [P(Sips), P(Grid), P(Params), P(Draws), vp, sz,
                                                vp]),
    "lacmo_plan_create": (ctypes.c_int, [P(Sips), P(Grid), P(Params), P(Draws), vp, sz,
                                         ctypes.c_int, vp, P(vp)]),
    "lacmo_plan_launch": (ctypes.c_int, [vp, vp]),
    "lacmo_plan_destroy": (ctypes.c_int, [vp]),
    "lacmo_plan_kernel_nodes": (i64, [vp]),
    "lacmo_dropin_adv_step": (ctypes.c_int, [P(Dropin), vp]),
    "lacmo_batch_workspace_bytes": (sz, [ctypes.c_int, P(i64), i64, i64]),
    "lacmo_batch_create": (ctypes.c_int, [ctypes.c_int, P(Sips), P(Grid), P(Params), P(u64), vp,
                                          sz, P(vp)]),
    "lacmo_batch_prepare": (ctypes.c_int, [vp, P(Params), vp]),
    "lacmo_batch_adv_step": (ctypes.c_int, [vp, P(Params), vp]),
    "lacmo_batch_plan_create": (ctypes.c_int, [vp, P(Params), ctypes.c_int, vp, P(vp)]),
    "lacmo_batch_particles_only": (ctypes.c_int, [vp, P(Params), vp]),
    "lacmo_batch_member_workspace": (ctypes.c_int, [vp, ctypes.c_int, P(vp), P(sz)]),
    "lacmo_batch_destroy": (ctypes.c_int, [vp]),
    "lacmo_adv_step_begin": (ctypes.c_int, [P(Sips), P(Grid), P(Params), vp, sz, vp]),
    "lacmo_adv_step_second_half": (ctypes.c_int, [P(Sips), P(Grid), P(Params), vp, sz, vp]),
    "lacmo_adv_substep": (ctypes.c_int, [P(Sips), P(Grid), P(Params), dbl, ctypes.c_int, vp, sz,
                                         vp]),
    "lacmo_propagate_particles_subloop_step": (ctypes.c_int, [P(Sips), P(Grid), P(Params), dbl,
                                                              dbl, vp, sz, vp]),
    "lacmo_propagate_grid_subloop_step": (ctypes.c_int, [P(Grid), vp, vp, vp, vp]),
    "lacmo_divergence_upwind": (ctypes.c_int, [vp, vp, i64, i64, dbl, dbl, ctypes.c_int,
                                               ctypes.c_int, vp, vp]),
    "lacmo_relaxation_term": (ctypes.c_int, [vp, i64, i64, vp, vp, dbl, vp, vp]),
    "lacmo_update_grid_r_l": (ctypes.c_int, [P(Sips), P(Grid), vp, sz, vp]),
    "lacmo_update_cell_sum": (ctypes.c_int, [ctypes.c_int, vp, vp, vp, vp, vp, i64, i64, i64, vp,
                                             vp, sz, vp]),
    "lacmo_compute_moment_R_grid": (ctypes.c_int, [i64, vp, vp, dbl, vp, i64, i64, i64, vp, vp,
                                                   sz, vp]),
    "lacmo_compute_R_p_w_s_rho_p": (ctypes.c_int, [ctypes.c_int, i64, vp, vp, vp, vp, vp, vp,
                                                   vp]),
    "lacmo_radius_from_mass": (ctypes.c_int, [i64, vp, dbl, vp, vp]),
    "lacmo_histogram_weighted": (ctypes.c_int, [vp, vp, i64, vp, i64, vp, vp]),
    "lacmo_sinsip_generate": (ctypes.c_int, [vp, vp, vp, i64, ctypes.c_int, vp, vp, dbl,
                                             ctypes.c_int, i64, vp, vp, vp, vp]),
    "lacmo_sinsip_gather": (ctypes.c_int, [vp, vp, vp, vp, i64, i64, vp, vp, vp, i64, vp]),
    "lacmo_init_mass_fraction": (ctypes.c_int, [ctypes.c_int, i64, vp, dbl, dbl, dbl, dbl, dbl,
                                                vp, vp]),
    "lacmo_saturation_adjust_level": (ctypes.c_int, [ctypes.c_int, i64, vp, i64, vp, vp, vp, vp,
                                                     vp, dbl, dbl, dbl, dbl, dbl, dbl,
                                                     ctypes.c_int, vp, vp, vp]),
    "lacmo_collision_step_cells": (ctypes.c_int, [P(Sips), P(Grid), P(Params), P(Draws), vp, sz,
                                                  vp]),
    "lacmo_collision_pair_count": (ctypes.c_int, [vp, i64, i64, i64, P(i64), vp]),
    "lacmo_collision_step_cells_noalloc": (ctypes.c_int, [vp, vp, vp, vp, vp, vp, i64, i64, i64,
                                                          P(Params), P(Draws), u64, vp, vp]),
    "lacmo_noalloc_status": (ctypes.c_int, [P(ctypes.c_uint32), P(i64), vp]),
    "lacmo_collision_step_golovin": (ctypes.c_int, [vp, vp, i64, dbl, vp, vp, u64, u64, vp]),
    "lacmo_collision_step_kernel_grid_m": (ctypes.c_int, [vp, vp, i64, dbl, vp, i64, dbl, dbl, vp,
                                                          vp, u64, u64, vp]),
    "lacmo_collision_step_ecol_grid_r_box": (ctypes.c_int, [vp, vp, vp, vp, vp, i64, dbl, vp, i64,
                                                            dbl, dbl, vp, vp, u64, u64, vp]),
    "lacmo_update_velocity_beard": (ctypes.c_int, [vp, vp, i64, vp]),
    "lacmo_mass_rate_and_derivative": (ctypes.c_int, [ctypes.c_int, i64] + [vp] * 16 + [vp]),
    "lacmo_newton_full": (ctypes.c_int, [ctypes.c_int, i64, dbl, ctypes.c_int] + [vp] * 16 + [vp]),
    "lacmo_interpolate_velocity": (ctypes.c_int, [vp, vp, vp, i64, i64, i64, vp, vp]),
    "lacmo_radius_and_bin": (ctypes.c_int, [vp, vp, i64, dbl, dbl, i64, vp, vp, vp]),
    "lacmo_adj_forward": (ctypes.c_int, [i64, i64, vp, vp, vp, vp, i64] + [vp] * 7 + [
        dbl, dbl, dbl, dbl, ctypes.c_int, ctypes.c_int, vp, vp, vp]),
    "lacmo_adj_backward": (ctypes.c_int, [i64, i64, vp, vp, vp, i64] + [vp] * 5 + [
        dbl, dbl, dbl, dbl, ctypes.c_int, ctypes.c_int] + [vp] * 10),
    "lacmo_collision_event_log": (ctypes.c_int, [vp, i64, vp]),
    "lacmo_batch_rebin": (ctypes.c_int, [vp, vp]),
    "lacmo_adj_collisions_forward": (ctypes.c_int, [vp, vp, i64, vp, vp, vp, vp]),
    "lacmo_adj_collisions_backward": (ctypes.c_int, [vp, vp, i64, vp, vp, vp]),
    "lacmo_adj_increments": (ctypes.c_int, [vp] * 4 + [i64, i64, dbl, dbl, dbl] + [vp] * 3 + [
        ctypes.c_int, vp, vp, vp]),
    "lacmo_adj_increments_vjp": (ctypes.c_int, [vp] * 4 + [i64, i64, dbl, dbl, dbl] + [vp] * 3 + [
        dbl, dbl] + [vp] * 5),
}

_lib = None


class LacmoError(RuntimeError):
    pass


def load():
    """Load the CUDA library (raises if it is missing: no fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise LacmoError(
            f"{LIB_PATH} is missing; build it with `python -m lacmopy_gb300.build` "
            "(nvcc, sm_103a). The SIP hot path has no CPU fallback.")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in PROTOTYPES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if lib.lacmo_abi_version() != 1:
        raise LacmoError("liblacmo_gb300.so ABI version mismatch")
    _lib = lib
    return lib


def check(status, what=""):
    if status != OK:
        raise LacmoError(f"{what}: {ERRORS.get(status, status)} (status {status})")
    return status
