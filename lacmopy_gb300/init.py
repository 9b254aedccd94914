"""Initialisation of the 2-D kinematic case (ICMW 2012 test case 1) with the
SIP work on the GPU: init.py:439-1236 of the reference.

``initialize_grid_and_particles_SinSIP(config)`` takes the reference's
configuration dict (after its ``set_config(config, 'generation')``) and
returns ``(grid, pos, cells, vel, m_w, m_s, xi, active_ids)`` like the
reference, writing the full state of t = 0 (file_handling formats) and the
mode labels to ``config['paths']['grid']``.

The level loop and its scalar thermodynamics run on the host in the
reference's order and arithmetic.  The SIP work runs on the GPU
(csrc/k_init.cu): the SinSIP ensembles of all levels in one launch from the
uniforms the reference draws (NumPy's global generator, seeded as the
reference seeds it, so the ensembles are the reference's), the equilibrium
solute mass fraction of every SIP (the reference's fminbound / brentq per SIP
becomes a bounded Brent maximisation and a bisection on the device), and each
saturation-adjustment iteration of a level (the Newton condensation of the
time step and the per-cell sums).  The generator's bin count uses
l_max + 1 slots where the reference's Python loop could overrun its l_max
bins (generation_SIP_ensemble.py:105-121); the lognormal generator needs no
extra bin.
"""
import ctypes
import math

import numpy as np
import torch

from . import _lib
from . import constants as c
from . import file_handling as fh
from .constants import solute_code
from .device import _ptr, _stream, to_device

EARTH_G = 9.80665
EPSILON_GC = c.specific_gas_constant_air_dry / c.specific_gas_constant_water_vapor
KAPPA_AIR_DRY = c.specific_gas_constant_air_dry / c.specific_heat_capacity_air_dry_NTP
VOLUME_TO_RADIUS = (c.four_pi_over_three_inv) ** (1.0 / 3.0)
TWO_PI_SQRT = math.sqrt(2.0 * math.pi)
W_S_MAX = {"AS": 0.78, "NaCl": 0.45}


# ---- scalar thermodynamics of the level loop (atmosphere.py,
# material_properties.py), in the reference's operation order -------------------
def kappa_air_moist(r_v):
    return KAPPA_AIR_DRY * (1 - 0.289 * r_v)


def beta_without_liquid(r_tot, Theta_l):
    return (EARTH_G * kappa_air_moist(r_tot) * (1 + r_tot)
            / (c.specific_gas_constant_air_dry * Theta_l * (1 + r_tot / EPSILON_GC)))


def saturation_pressure(T):
    return 2.53E11 * math.exp(-5420.0 / T)


def pressure_vapor(rho_v, T):
    return rho_v * T * c.specific_gas_constant_water_vapor


def heat_of_vaporization(T):
    return 1.0E3 * (2500.82 - 2.358 * (T - 273.0))


def diffusion_constant(T, p):
    return 4.01218E-5 * math.pow(T, 1.94) / p


def thermal_conductivity(T):
    return 4.1868E-3 * (5.69 + 0.017 * (T - 273.15))


def solubility(T, solute):
    if solute == "AS":
        return 0.15767235 + 0.00092684 * T
    return 3.77253081e-01 + -8.68998172e-04 * T + 1.64705858e-06 * T * T


def profiles_T_p_rhod_S_without_liquid(z, z_0, p_0, p_ref, Theta_l, r_tot):
    """init.py:384-437: T, p, rho_dry, S at height z of the liquid-free
    adiabatic profile."""
    kappa_tot = kappa_air_moist(r_tot)
    kappa_tot_inv = 1.0 / kappa_tot
    p_0_over_p_ref_to_kappa_tot = math.pow(p_0 / p_ref, kappa_tot)
    beta_tot = beta_without_liquid(r_tot, Theta_l)
    T_over_Theta_l = p_0_over_p_ref_to_kappa_tot - beta_tot * (z - z_0)
    T = T_over_Theta_l * Theta_l
    p = math.pow(T_over_Theta_l, kappa_tot_inv) * p_ref
    rho_dry = p * beta_tot / (T_over_Theta_l * EARTH_G * kappa_tot)
    S = pressure_vapor(rho_dry * r_tot, T) / saturation_pressure(T)
    return T, p, rho_dry, S


def _mass_from_radius(R, rho):
    return c.four_pi_over_three * rho * R * R * R


def set_config_generation(config):
    """init.py:59-108 (set_config in 'generation' mode): the modes with SIPs,
    their lognormal parameters (mu_m_log from the NaCl dry density for either
    solute, as the reference computes it) and the grid path, in place."""
    config["no_spcm"] = np.array(config["no_spcm"])
    no_spcm = config["no_spcm"]
    no_cells = np.asarray(config["no_cells"])
    grid_path = (config["paths"]["simdata"]
                 + f"{config['solute_type']}/grid_{no_cells[0]}_{no_cells[1]}_"
                 + f"spcm_{no_spcm[0]}_{no_spcm[1]}/{config['seed_SIP_gen']}/")
    config["paths"]["grid"] = grid_path
    import os
    os.makedirs(grid_path, exist_ok=True)
    config["weak_threshold"] = config["eta_threshold"] == "weak"
    idx = np.nonzero(no_spcm)[0]
    config["idx_mode_nonzero"] = idx
    config["no_modes"] = no_modes = len(idx)
    config["no_spcm"] = no_spcm[idx][0] if no_modes == 1 else no_spcm[idx]
    if config["dist"] == "lognormal":
        pick = (lambda a: np.asarray(a)[idx][0]) if no_modes == 1 \
            else (lambda a: np.asarray(a)[idx])
        sigma_R, mu_R = pick(config["sigma_R"]), pick(config["mu_R"])
        config["r_critmin"] = pick(config["r_critmin"])
        config["DNC0"] = pick(config["DNC0"])
        mu_m_log = np.log(c.four_pi_over_three * c.mass_density_NaCl_dry * mu_R * mu_R * mu_R)
        config["dist_par"] = (mu_m_log, 3.0 * np.log(sigma_R))
    return config


# ---- GPU steps ---------------------------------------------------------------------
def _modes(config):
    """Per-mode arrays of the lognormal distribution (set_config's 'generation'
    branch, init.py:59-108)."""
    no_modes = int(config["no_modes"])
    mu, sig = config["dist_par"]
    as_arr = lambda v: np.atleast_1d(np.asarray(v, dtype=np.float64))
    no_spcm = np.atleast_1d(np.asarray(config["no_spcm"]))
    if no_modes == 1:
        kappa = np.atleast_1d(max(math.ceil(float(no_spcm[0]) / 20 * 28) * 0.1, 0.1))
    elif no_modes == 2:
        kappa = np.maximum(np.ceil(no_spcm / 20 * np.array([33, 25])) * 0.1, 0.1)
    else:
        kappa = np.maximum(np.ceil(no_spcm / 20 * 28) * 0.1, 0.1)
    return no_modes, as_arr(mu), as_arr(sig), as_arr(kappa), as_arr(config["r_critmin"]), \
        as_arr(config["DNC0"]), kappa


def generate_sinsip_levels(config, no_cells, volume_cell):
    """The SinSIP mass ensembles of every (level, cell, mode), generated on
    the GPU from the uniforms the reference draws, in its order: per level,
    per cell, per mode l_max draws (and l_max more with the weak threshold).
    Returns per-segment masses, weights and counts as host arrays plus the
    segment layout."""
    lib = _lib.load()
    no_modes, mu, sig, kappa, r_crit, DNC0, kappa_raw = _modes(config)
    solute = config["solute_type"]
    rho_dry_mat = c.mass_density_AS_dry if solute == "AS" else c.mass_density_NaCl_dry
    weak = config["eta_threshold"] == "weak"
    m_hi_lo = float(config["m_high_over_m_low"])
    l_max = np.array([int(math.ceil(k * np.log10(m_hi_lo))) for k in kappa], dtype=np.int32)
    bin_factor = np.array([10 ** (1.0 / k) for k in kappa])
    m_low = np.array([_mass_from_radius(r, rho_dry_mat) for r in r_crit])
    nx, nz = int(no_cells[0]), int(no_cells[1])
    seg_mode = np.tile(np.arange(no_modes, dtype=np.int32), nx * nz)
    per_seg = l_max[seg_mode].astype(np.int64) * (2 if weak else 1)
    rnd_off = np.concatenate([[0], np.cumsum(per_seg)[:-1]]).astype(np.int64)
    n_rnd = int(per_seg.sum())
    # the reference seeds once before its level loop (and again per level
    # with reseed); the draws of a level are contiguous
    np.random.seed(int(config["seed_SIP_gen"]))
    if config.get("reseed", False):
        lvl = int(per_seg[: nx * no_modes].sum())
        rnd = np.concatenate([(np.random.seed(int(config["seed_SIP_gen"])),
                               np.random.rand(lvl))[1] for _ in range(nz)])
    else:
        rnd = np.random.rand(n_rnd)
    S = nx * nz * no_modes
    cap = int(l_max.max()) + 1
    dev = "cuda"
    masses = torch.empty((S, cap), dtype=torch.float64, device=dev)
    weights = torch.empty_like(masses)
    count = torch.empty(S, dtype=torch.int32, device=dev)
    par = to_device(np.concatenate([mu, sig, bin_factor, m_low, [TWO_PI_SQRT]]))
    rnd_d, off_d = to_device(rnd), to_device(rnd_off, torch.int64)
    mode_d, lmax_d = to_device(seg_mode, torch.int32), to_device(l_max, torch.int32)
    _lib.check(lib.lacmo_sinsip_generate(_ptr(rnd_d), _ptr(off_d), _ptr(mode_d), S, no_modes,
                                         _ptr(par), _ptr(lmax_d), float(config["eta"]),
                                         int(weak), cap, _ptr(masses), _ptr(weights),
                                         _ptr(count), _stream()), "sinsip_generate")
    return dict(masses=masses, weights=weights, count=count, cap=cap, no_modes=no_modes,
                DNC0=DNC0, kappa=kappa_raw if no_modes > 1 else float(kappa[0]))


def initialize_grid_and_particles_SinSIP(config, write_files=True):
    """init.py:439-1236 with the SIP work on the GPU (module docstring)."""
    lib = _lib.load()
    s = _stream()
    solute = config["solute_type"]
    sol = solute_code(solute)
    grid_ranges = np.asarray(config["grid_ranges"], dtype=np.float64)
    grid_steps = np.asarray(config["grid_steps"], dtype=np.float64)
    dx, dz = float(grid_steps[0]), float(grid_steps[1])
    dy = float(config["dy"])
    p_0, p_ref = float(config["p_0"]), float(config["p_ref"])
    r_tot_0, Theta_l = float(config["r_tot_0"]), float(config["Theta_l"])
    S_init_max, dt_init = float(config["S_init_max"]), float(config["dt_init"])
    newton_it, iter_limit = int(config["Newton_iterations"]), int(config["iter_cnt_limit"])
    grid = fh.GridData(grid_ranges, grid_steps, dy)
    nx, nz = int(grid.no_cells[0]), int(grid.no_cells[1])
    levels_z = grid.ranges[1, 0] + np.linspace(0.0, grid.sizes[1], nz + 1)
    gen = generate_sinsip_levels(config, grid.no_cells, grid.volume_cell)
    no_modes = gen["no_modes"]
    counts = gen["count"].cpu().numpy().reshape(nz, nx, no_modes)
    V0 = grid.volume_cell
    no_rpcm_0 = np.ceil(V0 * gen["DNC0"]).astype(int)
    rho_dry_0 = p_0 / (c.specific_gas_constant_air_dry * 293.0)
    w_max = W_S_MAX[solute]
    sol_T = None
    kappa_tot = kappa_air_moist(r_tot_0)
    kappa_tot_inv = 1.0 / kappa_tot
    # per-level outputs
    p_bottom = np.zeros(nz + 1)
    p_bottom[0] = p_0
    p_c, T_c, rho_c, rv_c, rl_c, S_c = (np.zeros(nz) for _ in range(6))
    m_w_all, m_s_all, xi_all, modes_all, cx_all = [], [], [], [], []
    no_spc = np.zeros((nx, nz), dtype=np.int64)
    scale_factors = np.zeros(nz)
    dev = "cuda"
    mass_dens_cells = None
    for j in range(nz):
        z_bot, z_top = levels_z[j], levels_z[j + 1]
        r_tot = r_tot_0
        p_bot = p_bottom[j]
        T_bot, p_bot, rho_bot, S_bot = profiles_T_p_rhod_S_without_liquid(
            z_bot, z_bot, p_bot, p_ref, Theta_l, r_tot)
        T_top, p_top, rho_top, S_top = profiles_T_p_rhod_S_without_liquid(
            z_top, z_bot, p_bot, p_ref, Theta_l, r_tot)
        p_avg = (p_bot + p_top) * 0.5
        T_avg = (T_bot + T_top) * 0.5
        rho_dry_avg = (rho_bot + rho_top) * 0.5
        S_avg = (S_bot + S_top) * 0.5
        r_v_avg = r_tot
        m_air_lvl = grid.sizes[0] * dy * (p_bot - p_top) / (EARTH_G * (1 + r_tot))
        m_vap_lvl = r_v_avg * m_air_lvl
        m_liq_lvl = 0.0
        m_par_lvl = 0.0
        scale = rho_dry_avg / rho_dry_0
        no_rpcm = np.rint(no_rpcm_0 * scale).astype(int)
        scale_factors[j] = scale
        # the level's SIPs: segments of this level, cell-major, mode-minor
        seg0 = j * nx * no_modes
        cnt = counts[j].reshape(-1)
        off = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int64)
        n_lvl = int(off[-1])
        seg_scale = np.tile(no_rpcm.astype(np.float64), nx)
        m_s_d = torch.empty(n_lvl, dtype=torch.float64, device=dev)
        xi_d = torch.empty_like(m_s_d)
        # device copies bound to names: a temporary freed while the call's
        # arguments are formed would hand its block to the next one
        off_seg_d = to_device(off[:-1], torch.int64)
        seg_scale_d = to_device(seg_scale)
        _lib.check(lib.lacmo_sinsip_gather(
            _ptr(gen["masses"][seg0:]), _ptr(gen["weights"][seg0:]), _ptr(gen["count"][seg0:]),
            _ptr(off_seg_d), nx * no_modes, gen["cap"], _ptr(seg_scale_d), _ptr(m_s_d),
            _ptr(xi_d), n_lvl, s), "sinsip_gather")
        no_spc[:, j] = cnt.reshape(nx, no_modes).sum(axis=1)
        cell_off = np.concatenate([[0], np.cumsum(no_spc[:, j])]).astype(np.int64)
        # equilibrium solute mass fraction at the level's mean state
        w_s_d = torch.empty_like(m_s_d)
        _lib.check(lib.lacmo_init_mass_fraction(sol, n_lvl, _ptr(m_s_d), float(S_avg),
                                                float(T_avg), VOLUME_TO_RADIUS, w_max,
                                                solubility(T_avg, solute), _ptr(w_s_d), s),
                   "init_mass_fraction")
        m_p_d = m_s_d / w_s_d
        m_w_d = m_p_d - m_s_d
        dm_l = float((m_w_d * xi_d).sum()) * 1.0E-18
        dm_p = float((m_p_d * xi_d).sum()) * 1.0E-18
        m_liq_lvl += dm_l
        m_par_lvl += dm_p
        m_vap_lvl -= dm_l
        heat_cap = (m_air_lvl * c.specific_heat_capacity_air_dry_NTP
                    + m_vap_lvl * c.specific_heat_capacity_water_vapor_20C
                    + m_par_lvl * c.specific_heat_capacity_water_NTP)
        dT = dm_l * heat_of_vaporization(T_avg) / heat_cap
        T_avg += dT; T_bot += dT; T_top += dT
        r_v_avg = m_vap_lvl / m_air_lvl
        p_top = p_bot * math.pow(T_top / T_bot, ((1 + r_tot) * EARTH_G * dz)
                                 / ((1 + r_v_avg / EPSILON_GC) * c.specific_gas_constant_air_dry
                                    * (T_bot - T_top)))
        p_avg = 0.5 * (p_bot + p_top)
        rho_dry_avg = (p_bot - p_top) / (dz * (1 + r_tot) * EARTH_G)
        m_air_lvl = grid.sizes[0] * dy * dz * rho_dry_avg
        r_l_avg = m_liq_lvl / m_air_lvl
        r_v_avg = r_tot - r_l_avg
        m_vap_lvl = r_v_avg * m_air_lvl
        e_s_avg = saturation_pressure(T_avg)
        S_avg = pressure_vapor(rho_dry_avg * r_v_avg, T_avg) / e_s_avg
        e_s_cells = np.full(nx, e_s_avg)
        S_cells = np.full(nx, S_avg)
        dm_l_level = m_liq_lvl
        it = 0
        off_d = to_device(cell_off, torch.int64)
        dml_c = torch.empty(nx, dtype=torch.float64, device=dev)
        mwxi_c = torch.empty_like(dml_c)
        while m_liq_lvl != 0.0 and abs(dm_l_level / m_liq_lvl) > 1e-5 and it < iter_limit:
            D_v = diffusion_constant(T_avg, p_avg)
            K = thermal_conductivity(T_avg)
            L_v = heat_of_vaporization(T_avg)
            S2_d = to_device(np.minimum(S_cells, S_init_max))
            e_s_d = to_device(e_s_cells)
            _lib.check(lib.lacmo_saturation_adjust_level(
                sol, nx, _ptr(off_d), n_lvl, _ptr(m_w_d), _ptr(m_s_d), _ptr(xi_d), _ptr(S2_d),
                _ptr(e_s_d), float(T_avg), float(p_avg), float(L_v), float(K),
                float(D_v), dt_init, newton_it, _ptr(dml_c), _ptr(mwxi_c), s),
                "saturation_adjust_level")
            dml_cells = dml_c.cpu().numpy()
            mwxi = mwxi_c.cpu().numpy()
            dm_l_level = 0.0
            dm_p_level = 0.0
            for i in range(nx):
                dm_l_level += dml_cells[i]
                dm_p_level += dml_cells[i]
            dm_l_level *= 1.0E-18
            dm_p_level *= 1.0E-18
            m_liq_lvl += dm_l_level
            m_par_lvl += dm_p_level
            m_vap_lvl -= dm_l_level
            heat_cap = (m_air_lvl * c.specific_heat_capacity_air_dry_NTP
                        + m_vap_lvl * c.specific_heat_capacity_water_vapor_20C
                        + m_par_lvl * c.specific_heat_capacity_water_NTP)
            dT = dm_l_level * heat_of_vaporization(T_avg) / heat_cap
            T_avg += dT; T_bot += dT; T_top += dT
            r_v_avg = m_vap_lvl / m_air_lvl
            p_top = p_bot * math.pow(T_top / T_bot, kappa_tot_inv * (EPSILON_GC + r_tot)
                                     / (EPSILON_GC + r_v_avg))
            p_avg = 0.5 * (p_bot + p_top)
            rho_dry_avg = (p_bot - p_top) / (dz * (1 + r_tot) * EARTH_G)
            m_air_lvl = grid.sizes[0] * dy * dz * rho_dry_avg
            m_air_cell = dx * dy * dz * rho_dry_avg
            r_l_avg = m_liq_lvl / m_air_lvl
            r_v_avg = r_tot - r_l_avg
            r_l_cells = mwxi * (1.0E-18 / m_air_cell)
            r_v_cells = r_tot - r_l_cells
            e_s_cells = np.full(nx, saturation_pressure(T_avg))
            S_cells = np.array([pressure_vapor(rho_dry_avg * rv, T_avg) for rv in r_v_cells]) \
                / e_s_cells
            m_vap_lvl = r_v_avg * m_air_lvl
            e_s_avg = saturation_pressure(T_avg)
            S_avg = pressure_vapor(rho_dry_avg * r_v_avg, T_avg) / e_s_avg
            it += 1
        grid.mixing_ratio_water_vapor[:, j] = r_v_cells if it else r_v_avg
        grid.mixing_ratio_water_liquid[:, j] = r_l_cells if it else r_l_avg
        grid.saturation_pressure[:, j] = e_s_cells
        grid.saturation[:, j] = S_cells
        p_bottom[j + 1] = p_top
        p_c[j], T_c[j], rv_c[j], rl_c[j], rho_c[j], S_c[j] = (p_avg, T_avg, r_v_avg, r_l_avg,
                                                              rho_dry_avg, S_avg)
        m_w_all.append(m_w_d.cpu().numpy())
        m_s_all.append(m_s_d.cpu().numpy())
        xi_all.append(xi_d.cpu().numpy())
        modes_all.append(np.concatenate([np.repeat(np.arange(no_modes), cnt.reshape(nx, no_modes)[i])
                                         for i in range(nx)]))
    m_w = np.concatenate(m_w_all)
    m_s = np.concatenate(m_s_all)
    xi = np.concatenate(xi_all)
    modes = np.concatenate(modes_all)
    # grid fields (init.py:1086-1171)
    for i in range(nx):
        grid.pressure[i] = p_c
        grid.temperature[i] = T_c
        grid.mass_density_air_dry[i] = rho_c
    p_dry = grid.mass_density_air_dry * c.specific_gas_constant_air_dry * grid.temperature
    grid.potential_temperature = grid.temperature * np.vectorize(math.pow)(1.0E5 / p_dry,
                                                                         KAPPA_AIR_DRY)
    grid.saturation_pressure = np.vectorize(saturation_pressure)(grid.temperature)
    rho_bottom = 0.5 * (rho_c[0:-1] + rho_c[1:])
    rho_bottom = np.insert(rho_bottom, 0, 0.5 * (3.0 * rho_c[0] - rho_c[1]))
    rho_bottom = np.append(rho_bottom, 0.5 * (3.0 * rho_c[-1] - rho_c[-2]))
    j_max = (0.6 * math.sqrt(grid.sizes[0] * grid.sizes[0] + grid.sizes[1] * grid.sizes[1])
             / math.sqrt(2.0 * 1500.0 * 1500.0))
    grid.mass_flux_air_dry = mass_flux_icmw(grid, j_max)
    grid.velocity[0] = grid.mass_flux_air_dry[0] / rho_bottom
    grid.velocity[1] = grid.mass_flux_air_dry[1] / np.append(rho_c, rho_c[-1])
    grid.update_material_properties()
    grid.rho_dry_inv = np.ones_like(grid.mass_density_air_dry) / grid.mass_density_air_dry
    grid.mass_dry_inv = (1.0 / grid.volume_cell) * grid.rho_dry_inv
    pos, rel_pos, cells = generate_random_positions(grid, no_spc)
    vel = _interpolate_velocity(cells, rel_pos, grid.velocity, grid.no_cells)
    active_ids = np.full(len(m_s), True)
    if write_files:
        path = config["paths"]["grid"]
        fh.save_grid_and_particles_full(0, grid, pos, cells, vel, m_w, m_s, xi, active_ids, path)
        np.save(path + "modes_0", modes)
        np.save(path + "no_rpcm_scale_factors_lvl_wise", scale_factors)
    return grid, pos, cells, vel, m_w, m_s, xi, active_ids


def mass_flux_icmw(grid, j_max):
    """init.py:239-320: the ICMW stream-function mass flux at the staggered
    velocity points."""
    X, Z = grid.sizes[0], grid.sizes[1]
    k_x, k_z = 2.0 * np.pi / X, np.pi / Z
    X_over_Z = X / Z
    cx = grid.ranges[0, 0] + np.linspace(0.0, grid.sizes[0], grid.no_cells[0] + 1)
    cz = grid.ranges[1, 0] + np.linspace(0.0, grid.sizes[1], grid.no_cells[1] + 1)
    CX, CZ = np.meshgrid(cx, cz, indexing="ij")
    xu, zu = CX, CZ + 0.5 * grid.steps[1]
    xw, zw = CX + 0.5 * grid.steps[0], CZ
    j_x = j_max * X_over_Z * np.cos(k_x * xu) * np.cos(k_z * zu)
    j_z = 2 * j_max * np.sin(k_x * xw) * np.sin(k_z * zw)
    return np.array([j_x, j_z])


def generate_random_positions(grid, no_spc):
    """init.py:322-382 (the draws continue NumPy's global stream)."""
    no_spt = int(np.sum(no_spc))
    rnd_x = np.random.rand(no_spt)
    rnd_z = np.random.rand(no_spt)
    nx, nz = int(grid.no_cells[0]), int(grid.no_cells[1])
    cx = grid.ranges[0, 0] + np.linspace(0.0, grid.sizes[0], nx + 1)
    cz = grid.ranges[1, 0] + np.linspace(0.0, grid.sizes[1], nz + 1)
    ci = np.concatenate([np.repeat(np.arange(nx), no_spc[:, j]) for j in range(nz)])
    cj = np.concatenate([np.full(int(no_spc[:, j].sum()), j) for j in range(nz)])
    x = cx[ci] + grid.steps[0] * rnd_x
    z = cz[cj] + grid.steps[1] * rnd_z
    return np.array([x, z]), np.array([rnd_x, rnd_z]), np.array([ci, cj])


def _interpolate_velocity(cells, rel_pos, grid_vel, no_cells):
    from .integration import interpolate_velocity_from_cell_bilinear
    return interpolate_velocity_from_cell_bilinear(cells, rel_pos, grid_vel, no_cells)
