"""Collision-efficiency tables E_col(R1, R2) on a logarithmic radius grid.

Host-side, one-time set-up of the collision kernel input (not on the per-step
path).  The generators restate the reference's table construction with the
same floating-point operations, so the tables equal the ones the reference ships
in ``Ecol_grid_data/`` bit for bit:

* ``generate_E_col_grid_R_Long_Bott_np`` follows collision/kernel.py:512-569
  with the efficiency of collision/kernel.py:350-373 (Long kernel, Bott 1998);
* ``generate_E_col_grid_R_Hall_Bott_np`` follows collision/kernel.py:581-696,
  bilinear interpolation of the Hall (1980) table as corrected by Bott (1998).
  The 15 x 21 raw table ships as ``data/hall_bott_1998_raw.npz``.

``load_kernel_data_Ecol`` mirrors file_handling.py:764-804: it returns the table
and the binning parameters (low-radius log, log bin factor, bin count).
"""
import math
import os
from functools import lru_cache

import numpy as np

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")


def _radius_grid(R_low, R_high, no_bins_10):
    bin_factor = 10 ** (1.0 / no_bins_10)
    no_bins = int(math.ceil(no_bins_10 * math.log10(R_high / R_low))) + 1
    radius_grid = np.zeros(no_bins, dtype=np.float64)
    r = float(R_low)
    radius_grid[0] = r
    for n in range(1, no_bins):
        r = r * bin_factor
        radius_grid[n] = r
    return radius_grid


def compute_E_col_Long_Bott(R_i, R_j):
    """Long (1974) collection efficiency as modified by Bott (1998)."""
    if R_j >= R_i:
        R_max, R_min = R_j, R_i
    else:
        R_max, R_min = R_i, R_j
    if R_max <= 50:
        return 4.5E-4 * R_max * R_max * (1.0 - 3.0 / (max(3.0, R_min) + 1.0E-2))
    return 1.0


def generate_E_col_grid_R_Long_Bott_np(R_low, R_high, no_bins_10,
                                       radius_grid_in=None):
    if radius_grid_in is None:
        radius_grid = _radius_grid(R_low, R_high, no_bins_10)
    else:
        radius_grid = np.asarray(radius_grid_in, dtype=np.float64)
    nb = radius_grid.shape[0]
    rg = [float(v) for v in radius_grid]
    E = np.zeros((nb, nb), dtype=np.float64)
    for j in range(nb):
        R_j = rg[j]
        for i in range(j + 1):
            E[j, i] = compute_E_col_Long_Bott(rg[i], R_j)
            E[i, j] = E[j, i]
    return E, radius_grid


def _hall_bott_raw():
    d = np.load(os.path.join(_DATA, "hall_bott_1998_raw.npz"))
    return d["E_col"], d["R_col"], d["R_ratio"]


def generate_E_col_grid_R_Hall_Bott_np(R_low, R_high, no_bins_10,
                                       radius_grid_in=None):
    E_raw, R_raw, q_raw = _hall_bott_raw()
    E_raw = [[float(v) for v in row] for row in E_raw]
    R_raw = [float(v) for v in R_raw]
    q_raw = [float(v) for v in q_raw]
    n_R, n_q = len(R_raw), len(q_raw)
    if radius_grid_in is None:
        radius_grid = _radius_grid(R_low, R_high, no_bins_10)
    else:
        radius_grid = np.asarray(radius_grid_in, dtype=np.float64)
    rg = [float(v) for v in radius_grid]
    nb = len(rg)
    E = np.zeros((nb, nb), dtype=np.float64)
    for iR, R_col in enumerate(rg):
        if R_col <= R_raw[0]:
            iRt = -1
        elif R_col > R_raw[-1]:
            iRt = n_R - 1
        else:
            for k in range(n_R - 1):
                if R_raw[k] < R_col <= R_raw[k + 1]:
                    iRt = k
                    break
        for ir in range(iR + 1):
            ratio = rg[ir] / R_col
            if ratio >= 1.0:
                iq = n_q - 2
            else:
                for k in range(n_q - 1):
                    if q_raw[k] <= ratio < q_raw[k + 1]:
                        iq = k
                        break
            if iRt == n_R - 1:
                q = (ratio - q_raw[iq]) / (q_raw[iq + 1] - q_raw[iq])
                e = (1. - q) * E_raw[iRt][iq] + q * E_raw[iRt][iq + 1]
                E[iR, ir] = e if e <= 1.0 else 1.0
            elif iRt == -1:
                q = (ratio - q_raw[iq]) / (q_raw[iq + 1] - q_raw[iq])
                E[iR, ir] = (1. - q) * E_raw[0][iq] + q * E_raw[0][iq + 1]
            else:
                p = (R_col - R_raw[iRt]) / (R_raw[iRt + 1] - R_raw[iRt])
                q = (ratio - q_raw[iq]) / (q_raw[iq + 1] - q_raw[iq])
                f = E_raw
                E[iR, ir] = ((1. - p) * (1. - q) * f[iRt][iq]
                             + (1. - p) * q * f[iRt][iq + 1]
                             + p * (1. - q) * f[iRt + 1][iq]
                             + p * q * f[iRt + 1][iq + 1])
            E[ir, iR] = E[iR, ir]
    return E, radius_grid


def generate_E_col_grid_R_np(R_low, R_high, no_bins_10, kernel_name):
    """collision/kernel.py:697-741: the efficiency table of 'Hall_Bott' or
    'Long_Bott' on the logarithmic radius grid; (E_col_grid, radius_grid)."""
    if kernel_name == "Hall_Bott":
        return generate_E_col_grid_R_Hall_Bott_np(R_low, R_high, no_bins_10, None)
    if kernel_name == "Long_Bott":
        return generate_E_col_grid_R_Long_Bott_np(R_low, R_high, no_bins_10, None)
    raise ValueError(f"kernel_name {kernel_name!r}")


def generate_and_save_E_col_grid_R(R_low, R_high, no_bins_10, kernel_name, save_dir):
    """collision/kernel.py:745-790: as generate_E_col_grid_R_np, and the
    grids written to save_dir as radius_grid_out.npy and E_col_grid.npy."""
    E, rg = generate_E_col_grid_R_np(R_low, R_high, no_bins_10, kernel_name)
    np.save(save_dir + "radius_grid_out.npy", rg)
    np.save(save_dir + "E_col_grid.npy", E)
    return E, rg


# ---- collection kernel K(R1, R2) tables for the kernel-grid-m box model ----
# Beard (1976) terminal velocity as collision/kernel.py:107-167 evaluates it
# (standard-atmosphere constants, radii in micrometres), one scalar call per
# radius; polynomial coefficients highest order first
_BEARD_P1 = (-0.327815e-5, 0.855176e-4, -0.578878e-3, -0.987059e-3, -0.153193e-2, 0.992696,
             -0.318657e1)
_BEARD_P2 = (0.238449e-2, -0.542819e-1, 0.475294, -0.204914e1, 0.523778e1, -0.500015e1)
_V_MAX_BEARD = 9.04929248
_G = 9.80665   # constants.py earth_gravity


def _horner(par, x):
    res = par[0] * x + par[1]
    for a in par[2:]:
        res = res * x + a
    return res


def terminal_velocity_Beard(R):
    """Sedimentation velocity (m/s) of a water drop of radius R (um)."""
    rho_w, rho_a, mu, sig = 1.0E3, 1.225, 1.818E-5, 73.0E-3
    drho = rho_w - rho_a
    if R < 10.0:
        C1 = drho * _G / (4.5 * mu)
        C_sc = 1.0 + 1.257 * 6.62E-2 / R
        return C1 * C_sc * R * R * 1.0E-12
    if R < 535.0:
        N_Da = 32.0E-18 * R * R * R * rho_a * drho * _G / (3.0 * mu * mu)
        Y = _horner(_BEARD_P1, math.log(N_Da))
        C_sc = 1.0 + 1.257 * 6.62E-2 / R
        return mu * C_sc * math.exp(Y) / (rho_a * R * 2.0E-6)
    if R < 3500.0:
        N_Bo = 16.0E-12 * R * R * drho * _G / (3.0 * sig)
        N_P16 = math.pow(sig * sig * sig * rho_a * rho_a / (math.pow(mu, 4) * drho * _G),
                         1.0 / 6.0)
        Y = _horner(_BEARD_P2, math.log(N_Bo * N_P16))
        return mu * N_P16 * math.exp(Y) / (rho_a * R * 2.0E-6)
    return _V_MAX_BEARD


def _kernel_grid(radius_grid, E_of, mass_density):
    rg = [float(v) for v in radius_grid]
    nb = len(rg)
    vel = [terminal_velocity_Beard(r) for r in rg]
    K = np.zeros((nb, nb), dtype=np.float64)
    for j in range(1, nb):
        R_j, v_j = rg[j], vel[j]
        for i in range(j):
            R_i = rg[i]
            K[j, i] = (1.0E-12 * math.pi * (R_i + R_j) * (R_i + R_j) * E_of(i, j)
                       * abs(v_j - vel[i]))
            K[i, j] = K[j, i]
    c_radius_to_mass = 4.0E-18 * math.pi * mass_density / 3.0
    mass_grid = np.array([c_radius_to_mass * math.pow(r, 3) for r in rg])
    return K, np.array(vel), mass_grid, np.array(radius_grid, dtype=np.float64)


def generate_kernel_grid_Long_Bott_np(R_low, R_high, no_bins_10, mass_density):
    """collision/kernel.py:793-867: K = 1e-12 pi (R_i + R_j)^2 E_Long |v_j -
    v_i| (m^3/s) on the logarithmic radius grid, with the Beard velocities;
    returns (kernel_grid, vel_grid, mass_grid (1e-18 kg), radius_grid)."""
    rg = _radius_grid(R_low, R_high, no_bins_10)
    r = [float(v) for v in rg]

    def E(i, j):   # the larger radius is R_j
        if r[j] <= 50.0:
            return 4.5E-4 * r[j] * r[j] * (1.0 - 3.0 / (max(3.0, r[i]) + 1.0E-2))
        return 1.0
    return _kernel_grid(rg, E, mass_density)


def generate_kernel_grid_Hall_Bott_np(R_low, R_high, no_bins_10, mass_density):
    """collision/kernel.py:869-942: as the Long kernel with the Hall/Bott
    efficiency table on the same radius grid."""
    rg = _radius_grid(R_low, R_high, no_bins_10)
    Eg, _ = generate_E_col_grid_R_Hall_Bott_np(R_low, R_high, no_bins_10, radius_grid_in=rg)
    return _kernel_grid(rg, lambda i, j: float(Eg[j, i]), mass_density)


def generate_and_save_kernel_grid(R_low, R_high, no_bins_10, mass_density, kernel_name,
                                  save_dir):
    """collision/kernel.py:944-1005: the kernel grid of 'Long_Bott' or
    'Hall_Bott', written as radius_grid_out.npy, mass_grid_out.npy,
    kernel_grid.npy and velocity_grid.npy."""
    gen = {"Long_Bott": generate_kernel_grid_Long_Bott_np,
           "Hall_Bott": generate_kernel_grid_Hall_Bott_np}[kernel_name]
    K, vel, mass, rg = gen(R_low, R_high, no_bins_10, mass_density)
    np.save(save_dir + "radius_grid_out.npy", rg)
    np.save(save_dir + "mass_grid_out.npy", mass)
    np.save(save_dir + "kernel_grid.npy", K)
    np.save(save_dir + "velocity_grid.npy", vel)
    return K, vel, mass, rg


def kernel_grid_m_parameters(mass_grid):
    """The binning parameters of the kernel-grid-m box model from a mass grid
    (logarithmic) in the SIPs' mass unit, fg: the generators' grids are in kg,
    so pass 1e18 times them, as run_box_model.py:379-389 does;
    (no_kernel_bins, m_kernel_low_log, bin_factor_m_log)."""
    return len(mass_grid), math.log(mass_grid[0]), math.log(mass_grid[1] / mass_grid[0])


# The reference's shipped tables were made with these arguments.
TABLE_ARGS = {"Long_Bott": (0.01, 51., 100), "Hall_Bott": (0.01, 301., 100)}


@lru_cache(maxsize=4)
def _cached(kernel_type):
    R_low, R_high, n10 = TABLE_ARGS[kernel_type]
    if kernel_type == "Long_Bott":
        E, rg = generate_E_col_grid_R_Long_Bott_np(R_low, R_high, n10)
    elif kernel_type == "Hall_Bott":
        E, rg = generate_E_col_grid_R_Hall_Bott_np(R_low, R_high, n10)
    else:
        raise ValueError(kernel_type)
    E.setflags(write=False)
    rg.setflags(write=False)
    return E, rg


def load_kernel_data_Ecol(kernel_type, E_col_const=0.5):
    """Return ``(E_col_grid, radius_grid, R_low, bin_factor, R_low_log,
    bin_factor_log, no_kernel_bins)`` like file_handling.py:764-804.

    ``kernel_type`` is 'Long_Bott', 'Hall_Bott' (kernel method 'Ecol_grid_R')
    or 'Hydro_E_const' (kernel method 'Ecol_const', constant efficiency).
    """
    if kernel_type == "Hydro_E_const":
        return float(E_col_const), None, None, None, None, None, None
    E, rg = _cached(kernel_type)
    R_low = rg[0]
    bin_factor = rg[1] / rg[0]
    return (E, rg, R_low, bin_factor, np.log(R_low), np.log(bin_factor),
            len(rg))
