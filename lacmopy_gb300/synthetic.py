"""Seeded synthetic SIP/grid states with the shapes and value ranges of the
ICMW 2012 test case 1 (kinematic drizzling stratocumulus) and of the Golovin
collision box model.

These stand in for the reference's initialisation output (init.py:439-1236,
generation_SIP_ensemble.py), which is one-time set-up outside the per-step hot
path.  The grid follows the reference case definition: 75 x 75 cells of 20 m,
Theta_l = 289 K, r_tot = 7.5 g/kg, p_0 = 1015 hPa (config.py:76-89), the ICMW
stream-function mass flux with j_max = 0.6 kg m^-2 s^-1 (init.py:250-314,
1146-1182) and a bimodal lognormal ammonium-sulfate aerosol (60 + 40 cm^-3,
mu_R = 0.02 / 0.075 um, sigma_R = 1.4 / 1.6, config.py:100-114).  Wet masses
are put near equilibrium with the cell saturation; cloudy cells get activated
droplets that carry the cloud liquid water, and a small fraction of drizzle
drops so that collisions happen.  All arrays use the reference's layout:
particle arrays are indexed by SIP ID, grid arrays are [Nx, Nz].
"""
import math

import numpy as np

from . import constants as c

GRID_FIELD_NAMES = ("temperature", "pressure", "potential_temperature",
                    "mass_density_air_dry", "mixing_ratio_water_vapor",
                    "mixing_ratio_water_liquid", "saturation",
                    "saturation_pressure", "mass_dry_inv", "rho_dry_inv")
MAT_PROP_NAMES = ("thermal_conductivity", "diffusion_constant",
                  "heat_of_vaporization", "surface_tension",
                  "specific_heat_capacity", "viscosity", "mass_density_fluid")


# elementwise libm pow (the reference's material functions are scalar
# functions vectorized over the grid, so each power is one scalar pow call;
# NumPy's array power may take a vectorized routine that rounds differently)
_pow = np.vectorize(math.pow, otypes=[np.float64])


def _sigma_w(T):
    tau = 1 - T / 647.096
    return 0.2358 * _pow(tau, 1.256) * (1 - 0.625 * tau)


def material_properties(gsf):
    """Material-property grids from the scalar fields (grid.py:713-727,
    material_properties.py:224-544, atmosphere.py)."""
    T, p, r_v, rho_d = gsf[0], gsf[1], gsf[4], gsf[3]
    mp = np.empty((7,) + T.shape)
    mp[0] = 4.1868E-3 * (5.69 + 0.017 * (T - 273.15))
    mp[1] = 4.01218E-5 * _pow(T, 1.94) / p
    mp[2] = 1.0E3 * (2500.82 - 2.358 * (T - 273.0))
    mp[3] = _sigma_w(T)
    mp[4] = c.specific_heat_capacity_air_dry_NTP * (1 + 0.897 * r_v)
    mp[5] = 1.458E-6 * _pow(T, 1.5) / (T + 110.4)
    mp[6] = rho_d * (1.0 + r_v)
    return mp


def _thermo(rho_d, Theta, r_v, p_ref):
    pdr = (rho_d * Theta * c.specific_gas_constant_air_dry / p_ref) ** c.kappa_factor
    T = Theta * pdr ** c.kappa_air_dry
    p = pdr * p_ref * (1 + r_v / c.epsilon_gc)
    e_s = 2.53E11 * np.exp(-5420.0 / T)
    S = rho_d * r_v * T * c.specific_gas_constant_water_vapor / e_s
    return T, p, e_s, S


def _mass_flux_icmw(Nx, Nz, dx, dz, j_max):
    X, Z = Nx * dx, Nz * dz
    k_x, k_z = 2.0 * np.pi / X, np.pi / Z
    xc = np.arange(Nx + 1) * dx
    zc = np.arange(Nz + 1) * dz
    xu, zu = np.meshgrid(xc, zc + 0.5 * dz, indexing="ij")
    xw, zw = np.meshgrid(xc + 0.5 * dx, zc, indexing="ij")
    j_x = j_max * (X / Z) * np.cos(k_x * xu) * np.cos(k_z * zu)
    j_z = 2 * j_max * np.sin(k_x * xw) * np.sin(k_z * zw)
    return np.array([j_x, j_z])


def _water_activity_AS(w_s):
    a = c.par_wat_act_AS
    r = a[0] * w_s + a[1]
    for k in a[2:]:
        r = r * w_s + k
    return r


def _w_s_for_activity(S):
    """Solution mass fraction with a_w(w_s) = S (bisection; a_w decreases)."""
    S = np.clip(S, 0.35, 0.9995)
    lo = np.zeros_like(S)
    hi = np.full_like(S, c.w_s_max_AS)
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        f = _water_activity_AS(mid) - S
        lo = np.where(f > 0, mid, lo)
        hi = np.where(f > 0, hi, mid)
    return np.clip(0.5 * (lo + hi), 0.02, c.w_s_max_AS * 0.98)


def make_icmw_state(Nx=75, Nz=75, no_spcm=(26, 38), seed=1001,
                    dx=20.0, dz=20.0, kernel_type="Long_Bott",
                    drizzle_fraction=0.03, Theta_l=289.0, r_tot=7.5E-3,
                    p_0=1015E2, p_ref=1E5, uneven=None):
    """Build one 2-D ICMW-like state.

    ``no_spcm`` gives SIPs per cell per aerosol mode.  ``uneven=(lo, hi)``
    instead draws the SIP count of every cell uniformly in [lo, hi] (split
    between the two modes in the 26:38 ratio), as in a batched ensemble whose
    members have uneven cell populations.
    Returns a dict of NumPy arrays and scalars in the reference's layout.
    """
    rng = np.random.default_rng(seed)
    V = dx * dz * 1.0
    zc = (np.arange(Nz) + 0.5) * dz
    # hydrostatic column of dry density / Theta / r_v, cloud above the LCL
    rho_d_z = np.empty(Nz)
    Theta_z = np.empty(Nz)
    r_v_z = np.empty(Nz)
    r_l_z = np.empty(Nz)
    p = p_0
    z_prev = 0.0
    for j in range(Nz):
        # integrate dp/dz = -rho g from z_prev to zc[j] in small steps
        n_sub = 8
        hz = (zc[j] - z_prev) / n_sub
        for _ in range(n_sub):
            T_guess = Theta_l * (p / p_ref) ** c.kappa_air_dry
            rho = p / (c.specific_gas_constant_air_dry * T_guess * (1 + 0.61 * r_tot))
            p -= rho * c.earth_gravity * hz
        z_prev = zc[j]
        T = Theta_l * (p / p_ref) ** c.kappa_air_dry
        e_s = 2.53E11 * math.exp(-5420.0 / T)
        r_s = c.epsilon_gc * e_s / (p - e_s)
        if r_tot > r_s:
            r_v = r_s * 1.0015
            r_l = r_tot - r_v
        else:
            r_v = r_tot
            r_l = 0.0
        L_v = 1.0E3 * (2500.82 - 2.358 * (T - 273.0))
        Theta = Theta_l + L_v / c.specific_heat_capacity_air_dry_NTP * (p_ref / p) ** c.kappa_air_dry * r_l
        p_d = p / (1 + r_v / c.epsilon_gc)
        T = Theta * (p_d / p_ref) ** c.kappa_air_dry
        rho_d_z[j] = p_d / (c.specific_gas_constant_air_dry * T)
        Theta_z[j] = Theta
        r_v_z[j] = r_v
        r_l_z[j] = r_l
    rho_d = np.tile(rho_d_z, (Nx, 1)) * (1.0 + 1e-4 * rng.standard_normal((Nx, Nz)))
    Theta = np.tile(Theta_z, (Nx, 1)) + 0.02 * rng.standard_normal((Nx, Nz))
    r_v = np.tile(r_v_z, (Nx, 1)) * (1.0 + 2e-4 * rng.standard_normal((Nx, Nz)))
    T, p, e_s, S = _thermo(rho_d, Theta, r_v, p_ref)
    # pin the cloud layer at a small supersaturation (S = 1.001)
    cloud = np.tile(r_l_z > 0, (Nx, 1))
    r_v = np.where(cloud | (S > 1.001), r_v * (1.001 / S), r_v)
    T, p, e_s, S = _thermo(rho_d, Theta, r_v, p_ref)
    gsf = np.empty((10, Nx, Nz))
    gsf[0], gsf[1], gsf[2], gsf[3], gsf[4] = T, p, Theta, rho_d, r_v
    gsf[5] = 0.0
    gsf[6], gsf[7] = S, e_s
    gsf[9] = 1.0 / rho_d
    gsf[8] = (1.0 / V) * gsf[9]
    gmp = material_properties(gsf)

    # mass flux and velocity at the staggered faces
    j_max = 0.6 * np.sqrt((Nx * dx) ** 2 + (Nz * dz) ** 2) / np.sqrt(2.0 * 1500.0 * 1500.0)
    flux = _mass_flux_icmw(Nx, Nz, dx, dz, j_max)
    rho_bottom = np.empty(Nz + 1)
    rho_bottom[0] = rho_d_z[0]
    rho_bottom[1:Nz] = 0.5 * (rho_d_z[:-1] + rho_d_z[1:])
    rho_bottom[Nz] = rho_d_z[-1]
    vel_grid = np.empty_like(flux)
    vel_grid[0] = flux[0] / np.append(rho_d_z, rho_d_z[-1])
    vel_grid[1] = flux[1] / rho_bottom

    # particles: per cell, per mode, stratified log-radius sampling
    mu_R = np.array([0.02, 0.075])
    sigma_R = np.array([1.4, 1.6])
    DNC = np.array([60.0E6, 40.0E6])
    if uneven is None:
        counts = np.empty((Nx, Nz, 2), dtype=np.int64)
        counts[..., 0] = no_spcm[0]
        counts[..., 1] = no_spcm[1]
    else:
        tot = rng.integers(uneven[0], uneven[1] + 1, size=(Nx, Nz))
        m0 = np.maximum(1, np.rint(tot * 26.0 / 64.0).astype(np.int64))
        counts = np.stack([m0, np.maximum(1, tot - m0)], axis=-1)
    n_cell = counts.sum(axis=-1)
    N = int(n_cell.sum())
    ci = np.repeat(np.arange(Nx), Nz)
    cj = np.tile(np.arange(Nz), Nx)
    cell_x = np.repeat(ci, n_cell.ravel())
    cell_z = np.repeat(cj, n_cell.ravel())
    R_s = np.empty(N)
    xi = np.empty(N)
    mode = np.empty(N, dtype=np.int64)
    off = 0
    flat_counts = counts.reshape(-1, 2)
    starts = np.concatenate([[0], np.cumsum(n_cell.ravel())[:-1]])
    for k in range(2):
        n_k = flat_counts[:, k]
        tot_k = int(n_k.sum())
        # position of each SIP of mode k inside its cell block
        cell_of = np.repeat(np.arange(Nx * Nz), n_k)
        rank = np.arange(tot_k) - np.repeat(np.cumsum(n_k) - n_k, n_k)
        base = starts[cell_of] + (0 if k == 0 else flat_counts[cell_of, 0])
        idx = base + rank
        lo = math.log(mu_R[k]) - 3.5 * math.log(sigma_R[k])
        hi = math.log(mu_R[k]) + 3.5 * math.log(sigma_R[k])
        width = (hi - lo) / n_k[cell_of]
        lnR = lo + (rank + rng.random(tot_k)) * width
        pdf = (np.exp(-0.5 * ((lnR - math.log(mu_R[k])) / math.log(sigma_R[k])) ** 2)
               / (math.sqrt(2 * math.pi) * math.log(sigma_R[k])))
        R_s[idx] = np.exp(lnR)
        xi[idx] = DNC[k] * V * pdf * width
        mode[idx] = k
        off += tot_k
    m_s = c.four_pi_over_three * c.mass_density_AS_dry * R_s ** 3
    # wet masses: haze in equilibrium with S; cloud droplets carry r_l
    S_p = S[cell_x, cell_z]
    w_s = _w_s_for_activity(np.minimum(S_p, 0.999))
    m_w = m_s * (1.0 / w_s - 1.0)
    cloudy = r_l_z[cell_z] > 0
    act = cloudy & (R_s > 0.035)
    R_wet = rng.uniform(4.0, 10.0, N)
    driz = act & (rng.random(N) < drizzle_fraction)
    R_wet = np.where(driz, rng.uniform(25.0, 60.0, N), R_wet)
    # drizzle SIPs represent few, large drops
    xi = np.where(driz, np.exp(rng.uniform(math.log(1e4), math.log(1e6), N)), xi)
    m_w_act = c.four_pi_over_three * 1000.0 * R_wet ** 3
    m_w = np.where(act, m_w_act, m_w)
    # rescale activated masses per cell so sum xi m_w matches r_l rho_d V
    cell_flat = cell_x * Nz + cell_z
    target = (r_l_z[cell_z] * rho_d[cell_x, cell_z] * V * 1e18)
    have = np.bincount(cell_flat, weights=np.where(act & ~driz, xi * m_w, 0.0),
                       minlength=Nx * Nz)
    need = target - np.bincount(cell_flat, weights=np.where(driz, xi * m_w, 0.0),
                                minlength=Nx * Nz)[cell_flat]
    scale = np.where(have[cell_flat] > 0, np.maximum(need, 0.1 * have[cell_flat])
                     / np.maximum(have[cell_flat], 1e-300), 1.0)
    m_w = np.where(act & ~driz, m_w * scale, m_w)
    m_w = np.maximum(m_w, m_s * (1.0 / c.w_s_max_AS - 1.0) * 1.01)
    # positions uniformly inside the cell
    pos = np.empty((2, N))
    pos[0] = (cell_x + rng.random(N)) * dx
    pos[1] = (cell_z + rng.random(N)) * dz
    cells = np.array([cell_x, cell_z], dtype=np.int64)
    rel_pos = np.array([pos[0] / dx - cell_x, pos[1] / dz - cell_z])
    vel = _interp_vel(cells, rel_pos, vel_grid, Nz)
    active_ids = np.full(N, True)
    # liquid water mixing ratio diagnostic (grid.py:370-412)
    r_l = np.zeros((Nx, Nz))
    np.add.at(r_l, (cell_x, cell_z), m_w * xi)
    gsf[5] = r_l * 1.0E-18 * gsf[8]

    from .tables import load_kernel_data_Ecol
    E_col_grid, _, _, _, R_low_log, bin_log, nb = load_kernel_data_Ecol(kernel_type)
    dt = 1.0
    scale_dt_cond = 5
    no_col_per_adv = 2
    dt_sub = dt / (2 * scale_dt_cond)
    return dict(
        grid_scalar_fields=gsf, grid_mat_prop=gmp, grid_velocity=vel_grid,
        grid_mass_flux_air_dry=flux, p_ref=p_ref, p_ref_inv=1.0 / p_ref,
        grid_no_cells=np.array([Nx, Nz], dtype=np.int64),
        grid_ranges=np.array([[0.0, Nx * dx], [0.0, Nz * dz]]),
        grid_steps=np.array([dx, dz]), grid_volume_cell=V,
        pos=pos, vel=vel, cells=cells, rel_pos=rel_pos, m_w=m_w, m_s=m_s,
        xi=xi, solute_type="AS", water_removed=np.array([0.0]),
        id_list=np.arange(N), active_ids=active_ids, T_p=np.ones(N),
        delta_m_l=np.zeros((Nx, Nz)),
        dt=dt, dt_sub=dt_sub, dt_sub_half=0.5 * dt_sub,
        dt_col_over_dV=(dt / no_col_per_adv) / V, scale_dt_cond=scale_dt_cond,
        no_col_per_adv=no_col_per_adv, act_collisions=True,
        act_relaxation=True,
        init_profile_r_v=np.average(gsf[4], axis=0),
        init_profile_Theta=np.average(gsf[2], axis=0),
        relaxation_time_profile=300 * np.exp(zc / 200),
        no_iter_impl_mass=3, g_set=c.earth_gravity,
        E_col_grid=E_col_grid, no_kernel_bins=nb, R_kernel_low_log=R_low_log,
        bin_factor_R_log=bin_log, no_cols=np.array([0, 0], dtype=np.int64),
        mode=mode)


def _interp_vel(cells, rel_pos, gv, Nz):
    """Staggered bilinear interpolation (grid.py:195-323), vectorised."""
    i, j = cells
    a, b = rel_pos
    u0, w0 = gv
    u = np.empty(len(i))
    lin = ((j == 0) & (b <= 0.5)) | ((j == Nz - 1) & (b >= 0.5))
    up = b > 0.5
    jj = np.where(up, j, j - 1)
    bb = np.where(up, b - 0.5, b + 0.5)
    jjc = np.clip(jj, 0, Nz)
    u_bil = (a * (bb * u0[i + 1, jjc + 1] + (1 - bb) * u0[i + 1, jjc])
             + (1 - a) * (bb * u0[i, jjc + 1] + (1 - bb) * u0[i, jjc]))
    u_lin = a * u0[i + 1, j] + (1 - a) * u0[i, j]
    u = np.where(lin, u_lin, u_bil)
    right = a > 0.5
    ii = np.where(right, i, i - 1)
    aa = np.where(right, a - 0.5, a + 0.5)
    w = (aa * (b * w0[ii + 1, j + 1] + (1 - b) * w0[ii + 1, j])
         + (1 - aa) * (b * w0[ii, j + 1] + (1 - b) * w0[ii, j]))
    return np.array([u, w])


def make_golovin_box(kappa=1000, seed=1001, R_mean=9.3, LWC0=1E-3,
                     mass_density=1E3, dV=1.0, eta=1E-9):
    """Exponential-mass box-model ensemble (run_box_model.py:133-153,239-242).

    Single-SIP-per-bin sampling on a logarithmic mass grid with a fixed weight
    threshold: ``6 kappa`` bins span m_low..1e6 m_low above r_critmin = 0.6 um;
    each SIP takes a uniform random mass inside its bin and the weight
    pdf(m) * bin_width * DNC0 * dV; bins below eta * max weight are dropped
    (kappa = 1000 leaves about 5000 SIPs).  Returns (xis, masses, DNC0, LWC0).
    """
    rng = np.random.default_rng(seed)
    c_radius_to_mass = 4.0E-18 * math.pi * mass_density / 3.0
    m_mean = c_radius_to_mass * R_mean ** 3
    DNC0 = LWC0 / m_mean
    m_low = c.four_pi_over_three * mass_density * 0.6 ** 3  # fg
    m_mean_fg = m_mean * 1e18
    nbins = 6 * int(kappa)
    edges = m_low * np.logspace(0.0, 6.0, nbins + 1)
    width = np.diff(edges)
    mu = edges[:-1] + rng.random(nbins) * width
    w = np.exp(-mu / m_mean_fg) / m_mean_fg * width
    xis = DNC0 * dV * w
    keep = w > w.max() * eta
    return xis[keep].copy(), mu[keep].copy(), DNC0, LWC0
