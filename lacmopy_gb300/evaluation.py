"""Drop-in replacements for the reference's per-cell diagnostics
(evaluation.py), computed on the GPU through the C ABI.

Same names, argument lists and results as LacmoPy's evaluation.py: per-cell
sums over the SIPs in ascending ID order, bit for bit the reference's loops
(``id_list`` must be 0 .. N-1, the reference's convention).  A SIP removed at
the ground (``cells[1] = -1``) counts where the reference's index -1 lands,
in the top row of its column.  NumPy arguments are copied to the device and
the results back; CUDA tensors stay on the device.
"""
import numpy as np
import torch

from . import _lib
from .device import _ptr, _stream, to_device


def _prepare(cells, n, no_cells, xi_dev):
    lib = _lib.load()
    nx, nz = int(no_cells[0]), int(no_cells[1])
    dev = xi_dev.device
    c = to_device(cells, torch.int64, dev)
    act = (c[1] >= 0).to(torch.uint8).contiguous()
    cell = torch.empty(n, dtype=torch.int32, device=dev)
    _lib.check(lib.lacmo_cells_import(_ptr(c), _ptr(act), _ptr(cell), n, nx, nz, _stream()),
               "cells_import")
    ws_bytes = int(lib.lacmo_workspace_bytes(n, nx, nz))
    ws = torch.zeros(ws_bytes, dtype=torch.uint8, device=dev)
    return lib, nx, nz, cell, ws, ws_bytes


def _check_ids(id_list, n):
    if id_list is not None and not np.array_equal(np.asarray(id_list), np.arange(n)):
        raise ValueError("id_list must be 0 .. N-1 (the reference's particle ID list)")


def _cell_sum(kind, out, m_w, xi, cells, mass_dry_inv, id_list, mask):
    n = int(np.shape(xi)[0])
    _check_ids(id_list, n)
    xi_d = to_device(xi)
    lib, nx, nz, cell, ws, ws_bytes = _prepare(cells, n, (np.shape(out)[0], np.shape(out)[1]),
                                               xi_d)
    mw_d = to_device(m_w) if kind == 0 else None
    mask_d = to_device(mask, torch.uint8)
    mdi = to_device(mass_dry_inv)
    res = torch.empty(nx * nz, dtype=torch.float64, device=xi_d.device)
    _lib.check(lib.lacmo_update_cell_sum(kind, _ptr(mw_d), _ptr(xi_d), _ptr(cell), _ptr(mask_d),
                                         _ptr(mdi), n, nx, nz, _ptr(res), _ptr(ws), ws_bytes,
                                         _stream()), "update_cell_sum")
    if isinstance(out, torch.Tensor):
        out.copy_(res.view(nx, nz))
    else:
        np.copyto(out, res.view(nx, nz).cpu().numpy())


def update_mixing_ratio(mixing_ratio, m_w, xi, cells, mass_dry_inv, id_list, mask):
    """evaluation.py:93-133: water mixing ratio of the masked SIPs per cell,
    in place."""
    _cell_sum(0, mixing_ratio, m_w, xi, cells, mass_dry_inv, id_list, mask)


def update_number_concentration_per_dry_mass(conc, xi, cells, mass_dry_inv, id_list, mask):
    """evaluation.py:136-174: number concentration per dry air mass of the
    masked SIPs per cell, in place."""
    _cell_sum(1, conc, None, xi, cells, mass_dry_inv, id_list, mask)


def compute_moment_R_grid(n, R_p, xi, V0, cells, active_ids, id_list, no_cells):
    """evaluation.py:1392-1445: the n-th moment of the radius distribution per
    cell from the active SIPs (mu^n / m^3); R_p^n by repeated squaring, as
    Numba's integer power."""
    N = int(np.shape(xi)[0])
    _check_ids(id_list, N)
    xi_d = to_device(xi)
    cells_eff = np.array(cells, dtype=np.int64, copy=True) if not isinstance(cells, torch.Tensor) \
        else cells.clone()
    act = np.asarray(active_ids, dtype=bool) if not isinstance(active_ids, torch.Tensor) \
        else active_ids.bool().cpu().numpy()
    cells_eff[1][~act] = -1   # only the active SIPs count
    lib, nx, nz, cell, ws, ws_bytes = _prepare(cells_eff, N, no_cells, xi_d)
    R_d = to_device(R_p)
    res = torch.empty(nx * nz, dtype=torch.float64, device=xi_d.device)
    _lib.check(lib.lacmo_compute_moment_R_grid(int(n), _ptr(R_d), _ptr(xi_d), float(V0),
                                               _ptr(cell), N, nx, nz, _ptr(res), _ptr(ws),
                                               ws_bytes, _stream()), "compute_moment_R_grid")
    return res.view(nx, nz).cpu().numpy()


# ---- radii, size spectra and moments of saved simulations --------------------------
def compute_R_p_w_s_rho_p(m_w, m_s, T_p, solute_type):
    """microphysics.py:208-266 on the GPU: (R_p, w_s, rho_p) per SIP."""
    from .constants import solute_code
    lib = _lib.load()
    mw, ms, tp = to_device(m_w), to_device(m_s), to_device(T_p)
    R, w, rho = (torch.empty_like(mw) for _ in range(3))
    _lib.check(lib.lacmo_compute_R_p_w_s_rho_p(solute_code(solute_type), mw.numel(), _ptr(mw),
                                               _ptr(ms), _ptr(tp), _ptr(R), _ptr(w), _ptr(rho),
                                               _stream()), "compute_R_p_w_s_rho_p")
    return R.cpu().numpy(), w.cpu().numpy(), rho.cpu().numpy()


def compute_radius_from_mass(mass, density):
    """microphysics.py:83-100 on the GPU for one density."""
    lib = _lib.load()
    m = to_device(mass)
    R = torch.empty_like(m)
    _lib.check(lib.lacmo_radius_from_mass(m.numel(), _ptr(m), float(density), _ptr(R),
                                          _stream()), "radius_from_mass")
    return R.cpu().numpy()


def histogram_weighted(x, bins, weights=None):
    """numpy.histogram(x, bins, weights=weights)[0] on the GPU (the weights of
    a bin add up in any order)."""
    lib = _lib.load()
    xd, e = to_device(x), to_device(bins)
    wd = to_device(weights) if weights is not None else None
    out = torch.empty(e.numel() - 1, dtype=torch.float64, device=xd.device)
    _lib.check(lib.lacmo_histogram_weighted(_ptr(xd), _ptr(wd), xd.numel(), _ptr(e),
                                            e.numel() - 1, _ptr(out), _stream()),
               "histogram_weighted")
    return out.cpu().numpy()


def update_T_p(grid_temp, cells, T_p):
    """evaluation.py:177-200: the cell temperature of every SIP (the row
    index -1 of a removed SIP wraps like NumPy indexing)."""
    T_p[:] = np.asarray(grid_temp)[cells[0], cells[1]]


def sample_masses_per_m_dry(m_w, m_s, xi, cells, id_list, grid_temperature, grid_mass_dry_inv,
                            target_cell, no_cells_x, no_cells_z):
    """evaluation.py:987-1083: the SIPs of the no_cells_x x no_cells_z box
    around target_cell, in ascending ID order, with their weights
    xi / m_dry of their cell and cell temperatures; (m_w, m_s, xi, weights,
    T_p, number of cells of the box)."""
    dx, dz = no_cells_x // 2, no_cells_z // 2
    i_lo, i_hi = target_cell[0] - dx, target_cell[0] + dx
    j_lo, j_hi = target_cell[1] - dz, target_cell[1] + dz
    no_cells_eval = (dx * 2 + 1) * (dz * 2 + 1)
    mask = (cells[0] >= i_lo) & (cells[0] <= i_hi) & (cells[1] >= j_lo) & (cells[1] <= j_hi)
    ids = np.asarray(id_list)[mask]
    ci, cj = cells[0, ids], cells[1, ids]
    return (np.array(m_w[ids]), np.array(m_s[ids]), np.array(xi[ids]),
            xi[ids] * grid_mass_dry_inv[ci, cj], np.array(grid_temperature[ci, cj]),
            no_cells_eval)


def sample_radii_per_m_dry(m_w, m_s, xi, cells, solute_type, id_list, grid_temperature,
                           grid_mass_dry_inv, target_cell, no_cells_x, no_cells_z):
    """evaluation.py:1085-1170: wet and dry radii (GPU) of the box's SIPs;
    (R_p, R_s, xi, weights, number of cells of the box)."""
    from . import constants as c
    m_w_o, m_s_o, xi_o, w_o, T_p, n_eval = sample_masses_per_m_dry(
        m_w, m_s, xi, cells, id_list, grid_temperature, grid_mass_dry_inv, target_cell,
        no_cells_x, no_cells_z)
    rho_dry = c.mass_density_AS_dry if solute_type == "AS" else c.mass_density_NaCl_dry
    R_s = compute_radius_from_mass(m_s_o, rho_dry)
    R_p = compute_R_p_w_s_rho_p(m_w_o, m_s_o, T_p, solute_type)[0]
    return R_p, R_s, xi_o, w_o, n_eval


def generate_size_spectra_R(load_path_list, ind_time, grid_mass_dry_inv, grid_no_cells,
                            solute_type, target_cell_list, no_cells_x, no_cells_z, no_bins_R_p,
                            no_bins_R_s):
    """evaluation.py:1172-1390: wet and dry radius spectra around target
    cells over the seeds' saved frames (file_handling formats), histograms on
    the GPU; (f_R_p, f_R_s, bins_R_p, bins_R_s, save_times, r_l averaged over
    the seeds, R_p minima, R_p maxima)."""
    from . import file_handling as fh
    no_seeds, no_tg = len(load_path_list), len(target_cell_list[0])
    grid_save_times = np.load(load_path_list[0] + "grid_save_times.npy")
    save_times_out = np.array([grid_save_times[ind_time[n]] for n in range(no_tg)],
                              dtype=np.int64)
    Rp, Rs, W = ([[] for _ in range(no_tg)] for _ in range(3))
    r_l = np.zeros((len(ind_time), grid_no_cells[0], grid_no_cells[1]))
    n_eval = 1
    for path in load_path_list:
        fields = fh.load_grid_scalar_fields(path, grid_save_times)
        _, cells_t, scal_t, xi_t, _ = fh.load_particle_data_all(path, grid_save_times)
        for n in range(no_tg):
            it = ind_time[n]
            R_p, R_s, _, w, n_eval = sample_radii_per_m_dry(
                scal_t[it, 0], scal_t[it, 1], xi_t[it], cells_t[it], solute_type,
                np.arange(len(xi_t[it])), fields[it, 3], grid_mass_dry_inv,
                target_cell_list[:, n], no_cells_x, no_cells_z)
            Rp[n].append(R_p); Rs[n].append(R_s); W[n].append(w)
            r_l[n] += fields[it, 1]
    r_l /= no_seeds
    f_p = np.zeros((no_tg, no_seeds, no_bins_R_p))
    f_s = np.zeros((no_tg, no_seeds, no_bins_R_s))
    b_p = np.zeros((no_tg, no_bins_R_p + 1))
    b_s = np.zeros((no_tg, no_bins_R_s + 1))
    R_min, R_max = [], []
    for n in range(no_tg):
        p_all, s_all = np.concatenate(Rp[n]), np.concatenate(Rs[n])
        R_min.append(np.amin(p_all)); R_max.append(np.amax(p_all))
        b_p[n] = np.logspace(np.log10(np.amin(p_all) * 0.5), np.log10(np.amax(p_all) * 2.),
                             no_bins_R_p + 1)
        b_s[n] = np.logspace(np.log10(np.amin(s_all) * 0.5), np.log10(np.amax(s_all) * 2.),
                             no_bins_R_s + 1)
        for k in range(no_seeds):
            f_p[n, k] = (1E-6 * histogram_weighted(Rp[n][k], b_p[n], W[n][k])
                         / (b_p[n][1:] - b_p[n][:-1]) / n_eval)
            f_s[n, k] = (1E-6 * histogram_weighted(Rs[n][k], b_s[n], W[n][k])
                         / (b_s[n][1:] - b_s[n][:-1]) / n_eval)
    return f_p, f_s, b_p, b_s, save_times_out, r_l, R_min, R_max


def generate_moments_all_seeds(load_path_list, no_moments, time_indices, grid_volume_cell,
                               no_cells, solute_type):
    """evaluation.py:1447-1549: the moments 0 .. no_moments - 1 of the radius
    distribution in every cell, for every seed and chosen save time, from the
    saved frames; radii and per-cell moments on the GPU.
    (moments[seed, time, moment, x, z], save times)."""
    from . import file_handling as fh
    grid_save_times = np.load(load_path_list[0] + "grid_save_times.npy")
    save_times_out = np.array([grid_save_times[i] for i in time_indices], dtype=np.int64)
    out = np.zeros((len(load_path_list), len(time_indices), no_moments, no_cells[0],
                    no_cells[1]))
    for k, path in enumerate(load_path_list):
        fields = fh.load_grid_scalar_fields(path, grid_save_times)
        _, cells_t, scal_t, xi_t, act_t = fh.load_particle_data_all(path, grid_save_times)
        for tn, it in enumerate(time_indices):
            n = len(xi_t[it])
            T_p = np.zeros(n)
            update_T_p(fields[it, 3], cells_t[it], T_p)
            R_p = compute_R_p_w_s_rho_p(scal_t[it, 0], scal_t[it, 1], T_p, solute_type)[0]
            for mom in range(no_moments):
                out[k, tn, mom] = compute_moment_R_grid(mom, R_p, xi_t[it], grid_volume_cell,
                                                        cells_t[it], act_t[it], np.arange(n),
                                                        no_cells)
    return out, save_times_out


def avg_moments_over_boxes(moments_vs_time_all_seeds, no_seeds, idx_t, no_moments,
                           target_cells_x, target_cells_z, no_cells_per_box_x,
                           no_cells_per_box_z):
    """evaluation.py:1551-1660: moments averaged over boxes of
    no_cells_per_box_x x no_cells_per_box_z cells centred at the target cells;
    [seed, time, moment, box x, box z]."""
    di, dj = no_cells_per_box_x // 2, no_cells_per_box_z // 2
    out = np.zeros((no_seeds, len(idx_t), no_moments, len(target_cells_x), len(target_cells_z)))
    for a, tx in enumerate(target_cells_x):
        for b, tz in enumerate(target_cells_z):
            # the box's cells in the order numpy.meshgrid lists them
            cz, cx = np.meshgrid(np.arange(tz - dj, tz - dj + no_cells_per_box_z),
                                 np.arange(tx - di, tx - di + no_cells_per_box_x), indexing="ij")
            cx, cz = cx.flatten(), cz.flatten()
            for k in range(no_seeds):
                for tn, it in enumerate(idx_t):
                    for mom in range(no_moments):
                        out[k, tn, mom, a, b] = np.average(
                            moments_vs_time_all_seeds[k, it, mom, cx, cz])
    return out
