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
