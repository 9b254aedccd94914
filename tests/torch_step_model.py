"""FP64 PyTorch restatement of the differentiated step model, for reference
gradients by autograd.  Test infrastructure: nothing in the package imports it.

The model is the reference's time step with the SIPs' cells per sub-step and
the collisions given (recorded from a product run; a collection adds the
collected masses, p_crit times them for a multiple collection, or splits an
equal-multiplicity pair, collision/all_or_nothing.py:577-633): per advection step
the advective + relaxation increments of Theta and r_v of the two half steps
(integration.py:1483-1508, 1536-1561) with the upwind divergence of
integration.py:80-287; per sub-step the condensation of every SIP in a cell
(integration.py:840-940, T_p = the cell's T, :1059-1060) by the damped Newton
of integration.py:728-836 with the mass rate of microphysics.py:1359-1469 and
then the grid update of integration.py:402-438 with the ambient state of
atmosphere.py:373-443 and material_properties.py.  The hygroscopicity kappa
scales the ammonium-sulfate water activity, a_w = 1 + (kappa / 0.6)(a_w_AS -
1), and flux_scale multiplies the mass flux.
"""
import math

import torch

from lacmopy_gb300 import constants as c


def _poly(par, x):   # algebra.py compute_polynom
    res = float(par[0]) * x + float(par[1])
    for a in par[2:]:
        res = res * x + float(a)
    return res


def ambient(Th, rv, rho_d, p_ref):
    pdr = (rho_d * Th * c.specific_gas_constant_air_dry / p_ref) ** c.kappa_factor
    T = Th * pdr ** c.kappa_air_dry
    p = pdr * p_ref * (1.0 + rv / c.epsilon_gc)
    e_s = 2.53E11 * torch.exp(-5420.0 / T)
    S = rho_d * rv * T * c.specific_gas_constant_water_vapor / e_s
    K = 4.1868E-3 * (5.69 + 0.017 * (T - 273.15))
    D_v = 4.01218E-5 * T ** 1.94 / p
    L_v = 1.0E3 * (2500.82 - 2.358 * (T - 273.0))
    tau = 1.0 - T / 647.096
    sig_w = 0.2358 * tau ** 1.256 * (1.0 - 0.625 * tau)
    pw = c.par_water_dens
    rho_w = float(pw[0]) + float(pw[1]) * (T - float(pw[2])) ** 2
    return dict(T=T, p=p, e_s=e_s, S=S, K=K, D_v=D_v, L_v=L_v, sig_w=sig_w, rho_w=rho_w)


def mass_rate(m_w, m_s, ks, a):
    """gamma and dgamma/dm_w of an AS SIP (microphysics.py:1359-1469)."""
    m_p = m_w + m_s
    w_s = m_s / m_p
    rho_p = a["rho_w"] * _poly(c.par_rho_AS, w_s)
    R_p = (c.four_pi_over_three_inv * m_p / rho_p) ** (1.0 / 3.0)
    sigma_p = a["sig_w"] * (1.0 + c.par_sigma_AS * w_s / (1.0 - w_s))
    T = a["T"]
    l_a = 1.0E-6 * (R_p + (c.c_alpha_1 + c.c_alpha_2 * (T - c.T_alpha_0)) * a["K"] / a["p"])
    l_b = 1.0E-6 * (R_p + c.c_beta_1 * (1.0 + c.c_beta_2 * (T - c.T_alpha_0)) * a["D_v"])
    m_p_inv_SI = 1.0E18 / m_p
    drho = -a["rho_w"] * m_p_inv_SI / rho_p * w_s * _poly(c.par_rho_deriv_AS, w_s)
    dR_over_R = c.one_third * (m_p_inv_SI - drho)
    dR = 1.0E-6 * dR_over_R * R_p
    eps_k = 2.0E6 * sigma_p / (c.specific_gas_constant_water_vapor * T * rho_p * R_p)
    kel = torch.exp(eps_k)
    a_w = 1.0 + ks * (_poly(c.par_wat_act_AS, w_s) - 1.0)
    da_w = -ks * m_p_inv_SI * w_s * _poly(c.par_wat_act_deriv_AS, w_s)
    dsig = -c.par_sigma_AS * a["sig_w"] * m_p_inv_SI * (w_s / ((1. - w_s) * (1. - w_s)))
    S_eq = a_w * kel
    dS_eq = da_w * kel + S_eq * eps_k * (dsig / sigma_p - drho - dR_over_R)
    c1 = a["L_v"] ** 2 / (c.specific_gas_constant_water_vapor * a["K"] * T * T)
    c2 = c.specific_gas_constant_water_vapor * T / (a["D_v"] * a["e_s"])
    f3 = 1.0 / (l_a * S_eq * c1 + l_b * c2)
    f1f3 = 4.0 * math.pi * R_p * R_p * f3
    dg1 = (dS_eq * l_a + S_eq * dR) * c1 + dR * c2
    f2 = a["S"] - S_eq
    return 1.0E6 * f1f3 * f2, 1.0E-12 * f1f3 * (f2 * (2.0 * dR_over_R - f3 * dg1) - dS_eq)


def newton(m_w, m_s, ks, a, dt, no_iter):   # integration.py:786-836
    m_eff = m_s * (c.w_s_max_AS_inv - 1.0)

    def denom(x):
        return torch.where(x < 0.9, 1.0 / (1.0 - torch.where(x < 0.9, x, torch.zeros_like(x))),
                           torch.full_like(x, 10.0))

    g, dg = mass_rate(m_w, m_s, ks, a)
    m = torch.maximum(m_eff, m_w + dt * g * denom(dt * dg))
    for _ in range(no_iter - 1):
        g, dg = mass_rate(m, m_s, ks, a)
        m = torch.maximum(m_eff, m + (dt * g + m_w - m) * denom(dt * dg))
    return m


def _limiter(a0, a1, a2):   # integration.py:80-148
    big = (a1 - a2).abs() > 1.0E-8 * (a0 - a1).abs()
    den = torch.where(big, a1 - a2, torch.ones_like(a1))
    r = torch.where(big, (a0 - a1) / den, (a0 - a1) * 1.0E8 * torch.sign(a1 - a2))
    K = (1.0 + 2.0 * r) * c.one_third
    return torch.clamp_min(torch.minimum(2.0 * r, torch.clamp_max(K, 2.0)), 0.0)


def _face_fluxes(fx, u, N):
    """fx: the field padded by two cells on each side along axis 0."""
    a0, a1, a2 = fx[2:N + 3], fx[1:N + 2], fx[0:N + 1]
    f_pos = a1 + 0.5 * _limiter(a0, a1, a2) * (a1 - a2)
    a2n = fx[3:N + 4]
    f_neg = a0 + 0.5 * _limiter(a1, a0, a2n) * (a0 - a2n)
    return torch.where(u >= 0.0, u * f_pos, u * f_neg)


def divergence(f, flux, dx, dz):
    """integration.py:150-287, x periodic and z solid; f [nx][nz], flux
    [2][nx+1][nz+1]."""
    nx, nz = f.shape
    fx = torch.cat([f[nx - 2:nx], f, f[0:2]], 0)
    F = _face_fluxes(fx, flux[0][:, :nz], nx)
    div = (F[1:] - F[:-1]) / dx
    ft = f.t()
    fz = torch.cat([ft[0:1], ft[0:1], ft, ft[nz - 1:nz], ft[nz - 1:nz]], 0)
    G = _face_fluxes(fz, flux[1][:nx, :].t(), nz)
    G = torch.cat([torch.zeros_like(G[:1]), G[1:-1], torch.zeros_like(G[:1])], 0)
    return div + ((G[1:] - G[:-1]) / dz).t()


def relaxation(f, prof, trel, dt):   # integration.py:325-354
    return dt * (prof - f.sum(0) / f.shape[0]) / trel


def decode_events(events):
    """{sub-step: [(records [r][32] uint8 tensor, offsets, G), ...]} of a
    StepModel -> {sub-step: [(imin, imax, kind, a, b), ...]} in order."""
    import numpy as np
    out = {}
    for k, groups in events.items():
        lst = []
        for rec, _, _ in groups:
            r = rec.cpu().numpy()
            ints = r.view(np.int32).reshape(-1, 8)
            dbl = r.view(np.float64).reshape(-1, 4)
            lst += [(int(i[0]), int(i[1]), int(i[2]), float(d[2]), float(d[3]))
                    for i, d in zip(ints, dbl)]
        out[k] = lst
    return out


def collide(m_w, m_s, xi, evs):
    """collision/all_or_nothing.py:577-633 with the recorded outcomes;
    returns the new (m_w, m_s, xi) (xi a new tensor: the old one may be
    saved for the backward pass)."""
    if evs:
        xi = xi.clone()
    for imin, imax, kind, a, b in evs:
        w_min, w_max, s_min, s_max = m_w[imin], m_w[imax], m_s[imin], m_s[imax]
        xmin, xmax = float(xi[imin]), float(xi[imax])
        if kind == 2:
            m_w = m_w.index_put((torch.tensor([imin]),), (w_min + a * w_max).reshape(1))
            m_s = m_s.index_put((torch.tensor([imin]),), (s_min + a * s_max).reshape(1))
            xi[imax] = xmax - a * xmin
        elif kind == 1:
            ges = xmin + xmax
            w = 2.0 * (xmin * w_min + xmax * w_max) / ges
            sm = 2.0 * (xmin * s_min + xmax * s_max) / ges
            idx = torch.tensor([imin, imax])
            m_w = m_w.index_put((idx,), torch.stack([w, w]))
            m_s = m_s.index_put((idx,), torch.stack([sm, sm]))
            xi[imax] = 0.5 * 0.7 * ges
            xi[imin] = 0.5 * ges - xi[imax]
        else:
            m_w = m_w.index_put((torch.tensor([imin]),), (w_min + w_max).reshape(1))
            m_s = m_s.index_put((torch.tensor([imin]),), (s_min + s_max).reshape(1))
            xi[imax] = xmax - xmin
    return m_w, m_s, xi


def run(st, cells, m_s, kappa, flux_scale, n_adv, no_iter, events=None):
    """Final m_w of the model; cells [2 scale_dt_cond n_adv][n] (int, < 0:
    not condensing); m_s, kappa, flux_scale tensors (autograd); events
    {sub-step: [(imin, imax, kind, a, b), ...]} the collisions recorded
    before that sub-step (decode_events)."""
    events = events or {}
    nx, nz = (int(v) for v in st["grid_no_cells"])
    C = nx * nz
    t = lambda x: torch.as_tensor(x, dtype=torch.float64)
    gsf = t(st["grid_scalar_fields"])
    Th, rv = gsf[2].reshape(C).clone(), gsf[4].reshape(C).clone()
    rho_d, mdi, rdi = gsf[3].reshape(C), gsf[8].reshape(C), gsf[9].reshape(C)
    m_w = t(st["m_w"]).clone()
    xi = t(st["xi"]).clone()
    flux = t(st["grid_mass_flux_air_dry"]) * flux_scale
    dx, dz = (float(v) for v in st["grid_steps"])
    dt = float(st["dt_sub"])
    p_ref, V = float(st["p_ref"]), float(st["grid_volume_cell"])
    S = int(st["scale_dt_cond"])
    relax = bool(st["act_relaxation"])
    ks = kappa / 0.6
    cells = torch.as_tensor(cells, dtype=torch.int64)

    def inc_first(f, prof):
        v = -dt * divergence(f.reshape(nx, nz), flux, dx, dz).reshape(C) * rdi
        if relax:
            v = v + relaxation(f.reshape(nx, nz), t(prof), t(st["relaxation_time_profile"]),
                               dt).repeat(nx)
        return v

    def sub_step(m_w, m_s, Th, rv, cell, dTh, drv):
        act = cell >= 0
        ci = cell.clamp_min(0)
        a = ambient(Th, rv, rho_d, p_ref)
        ag = {k: v[ci] for k, v in a.items()}
        m_new = torch.where(act, newton(m_w, m_s, ks, ag, dt, no_iter), m_w)
        dml = torch.zeros(C, dtype=torch.float64).index_add(
            0, ci, torch.where(act, (m_new - m_w) * xi, torch.zeros_like(m_w))) * 1.0E-18
        Th1 = Th + dTh
        rv1 = rv + drv - dml * mdi
        ToT = (c.specific_gas_constant_air_dry / p_ref * rho_d * Th1) ** c.kappa_factor2
        Th2 = Th1 + ToT * (a["L_v"] * dml) / (c.specific_heat_capacity_air_dry_NTP * rho_d * V
                                              * (1.0 + rv1 * c.heat_factor_r_v))
        return m_new, Th2, rv1

    for adv in range(n_adv):
        dTh = inc_first(Th, st["init_profile_Theta"])
        drv = inc_first(rv, st["init_profile_r_v"])
        for k in range(S):
            kg = 2 * S * adv + k
            m_w, m_s, xi = collide(m_w, m_s, xi, events.get(kg, ()))
            m_w, Th, rv = sub_step(m_w, m_s, Th, rv, cells[kg], dTh, drv)
        dTh = 2.0 * inc_first(Th, st["init_profile_Theta"]) - dTh
        drv = 2.0 * inc_first(rv, st["init_profile_r_v"]) - drv
        for k in range(S):
            kg = (2 * adv + 1) * S + k
            m_w, m_s, xi = collide(m_w, m_s, xi, events.get(kg, ()))
            m_w, Th, rv = sub_step(m_w, m_s, Th, rv, cells[kg], dTh, drv)
    return m_w
