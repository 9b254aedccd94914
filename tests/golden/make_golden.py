"""Generate the golden fixtures under tests/golden/ from the reference itself.

Runs the unmodified LacmoPy reference (pure Python + NumPy; Numba replaced by
identity decorators, see refstub.py) on small seeded inputs and stores inputs,
injected uniform draws and outputs as compressed .npz files.  The draws are the
ones the reference pulls from NumPy's global MT19937 stream; they are recorded
by wrapping ``numpy.random.rand`` so kernels and the oracle can consume the
identical sequence.

Usage (from the repository root, in a container that has the reference; the
path of the reference's source tree is required):
    python tests/golden/make_golden.py <reference root> [fixture ...]
With fixture names (the gen_* functions without the prefix) only those
fixtures are regenerated.

NumPy's SVML (AVX-512) dispatch is switched off before NumPy is imported so
array pow/log/exp call scalar glibc libm like Numba-compiled code does.
"""
import os
import sys

os.environ.setdefault("NPY_DISABLE_CPU_FEATURES", "X86_V4 AVX512_ICL AVX512_SPR")

import copy  # noqa: E402
import hashlib  # noqa: E402

import numpy as np  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, REPO)

import refstub  # noqa: E402
from lacmopy_gb300 import synthetic  # noqa: E402

_recorded = []
_orig_rand = np.random.rand


def _recording_rand(*shape):
    r = _orig_rand(*shape)
    _recorded.append(np.array(r, dtype=np.float64).ravel())
    return r


def take_draws():
    out = np.concatenate(_recorded) if _recorded else np.zeros(0)
    _recorded.clear()
    return out


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print(f"wrote {name}: {os.path.getsize(path)} bytes")


def gen_mass_rate(R):
    rng = np.random.default_rng(11)
    n = 1500
    T_amb = rng.uniform(270.0, 295.0, n)
    p_amb = rng.uniform(8.0e4, 1.0e5, n)
    S_amb = rng.uniform(0.85, 1.01, n)
    e_s = 2.53E11 * np.exp(-5420.0 / T_amb)
    K = 4.1868E-3 * (5.69 + 0.017 * (T_amb - 273.15))
    D_v = 4.01218E-5 * T_amb ** 1.94 / p_amb
    L_v = 1.0E3 * (2500.82 - 2.358 * (T_amb - 273.0))
    T_p = T_amb + rng.uniform(-0.2, 0.2, n)
    m_s = np.exp(rng.uniform(np.log(1e-4), np.log(50.0), n))
    ws_target = np.exp(rng.uniform(np.log(1e-6), np.log(0.7), n))
    m_w = m_s * (1.0 / ws_target - 1.0)
    out = {k: [] for k in ["g_AS", "dg_AS", "g_NaCl", "dg_NaCl", "dm_AS",
                           "g0_AS", "dm_NaCl", "g0_NaCl", "R_AS", "R_NaCl",
                           "rho_AS", "rho_NaCl", "w_s", "sig_AS", "sig_NaCl"]}
    for k in range(n):
        args_amb = (float(T_amb[k]), float(p_amb[k]), float(S_amb[k]),
                    float(e_s[k]), float(L_v[k]), float(K[k]), float(D_v[k]))
        mw, ms, tp = np.float64(m_w[k]), np.float64(m_s[k]), np.float64(T_p[k])
        for sol in ("AS", "NaCl"):
            Rp, ws, rho = R.mp.compute_R_p_w_s_rho_p(mw, ms, tp, sol)
            sig = R.mat.compute_surface_tension_solution(ws, tp, sol)
            if sol == "AS":
                g, dg = R.mp.compute_mass_rate_and_derivative_AS_np(
                    mw, ms, ws, Rp, tp, rho, *args_amb, sig)
            else:
                g, dg = R.mp.compute_mass_rate_and_derivative_NaCl_np(
                    mw, ms, ws, Rp, tp, rho, *args_amb, sig)
            dm, g0 = R.integ.compute_dml_and_gamma_impl_Newton_full_np(
                0.1, 3, mw, ms, ws, Rp, tp, rho, *args_amb, sig, sol)
            out[f"g_{sol}"].append(float(g))
            out[f"dg_{sol}"].append(float(dg))
            out[f"dm_{sol}"].append(float(dm))
            out[f"g0_{sol}"].append(float(g0))
            out[f"R_{sol}"].append(float(Rp))
            out[f"rho_{sol}"].append(float(rho))
            out[f"sig_{sol}"].append(float(sig))
            if sol == "AS":
                out["w_s"].append(float(ws))
    save("mass_rate_newton.npz", T_amb=T_amb, p_amb=p_amb, S_amb=S_amb,
         e_s_amb=e_s, L_v=L_v, K=K, D_v=D_v, T_p=T_p, m_s=m_s, m_w=m_w,
         dt_sub=np.float64(0.1), no_iter=np.int64(3),
         **{k: np.array(v) for k, v in out.items()})


def gen_golovin(R):
    cases = {}
    xis0, m0, _, _ = synthetic.make_golovin_box(kappa=40, seed=5)
    # case 0: physical; case 1: boosted dt/dV (multiple collection p_crit > 1);
    # case 2: pairs of equal multiplicities (equal-xi branch)
    xis2 = xis0.copy()
    xis2[1::2] = xis2[0::2][:len(xis2[1::2])]
    for name, xis_in, dtdv, nsteps in [("phys", xis0, 1.0, 3),
                                       ("boost", xis0, 2.0e3, 2),
                                       ("eqxi", xis2, 300.0, 2)]:
        np.random.seed(1001)
        take_draws()
        xis = xis_in.copy()
        ms = m0.copy()
        no_cols = np.array([0, 0], dtype=np.int64)
        steps = []
        for s in range(nsteps):
            R.aon.collision_step_Golovin_np(xis, ms, dtdv, no_cols)
            steps.append((xis.copy(), ms.copy(), no_cols.copy()))
        cases[name] = dict(xis_in=xis_in, m_in=m0, dt_over_dV=np.float64(dtdv),
                           draws=take_draws(),
                           xis_out=np.array([s[0] for s in steps]),
                           m_out=np.array([s[1] for s in steps]),
                           no_cols_out=np.array([s[2] for s in steps]))
    save("collision_golovin.npz",
         **{f"{n}__{k}": v for n, d in cases.items() for k, v in d.items()})


def gen_ecol_box(R):
    out = {}
    for kt in ("Long_Bott", "Hall_Bott"):
        E, rg, R_low, bf, R_low_log, bf_log, nb = R.fh.load_kernel_data_Ecol(
            "Ecol_grid_R", f"Ecol_grid_data/{kt}/")
        rng = np.random.default_rng(7)
        n = 160
        R0 = np.exp(rng.uniform(np.log(1.0), np.log(80.0), n))
        rho = np.full(n, 1000.0)
        masses = R.mp.compute_mass_from_radius_vec(R0, rho)
        radii = R.mp.compute_radius_from_mass_vec(masses, rho)
        vel = np.zeros(n)
        R.ker.update_velocity_Beard(vel, radii)
        xis = np.exp(rng.uniform(np.log(1e4), np.log(3e7), n))
        np.random.seed(2002)
        take_draws()
        x, m, r, v = xis.copy(), masses.copy(), radii.copy(), vel.copy()
        no_cols = np.array([0, 0], dtype=np.int64)
        seq = []
        for s in range(2):
            R.aon.collision_step_Ecol_grid_R_np(
                x, m, r, v, rho, 1.0, E, nb, R_low_log, bf_log, no_cols)
            R.ker.update_velocity_Beard(v, r)
            seq.append((x.copy(), m.copy(), r.copy(), v.copy(), no_cols.copy()))
        pre = kt + "__"
        out.update({pre + "xis_in": xis, pre + "m_in": masses, pre + "r_in": radii,
                    pre + "v_in": vel, pre + "rho": rho, pre + "draws": take_draws(),
                    pre + "dt_over_dV": np.float64(1.0),
                    pre + "xis_out": np.array([s[0] for s in seq]),
                    pre + "m_out": np.array([s[1] for s in seq]),
                    pre + "r_out": np.array([s[2] for s in seq]),
                    pre + "v_out": np.array([s[3] for s in seq]),
                    pre + "no_cols_out": np.array([s[4] for s in seq])})
    save("collision_ecol_box.npz", **out)


def _small_state(seed, Nx=6, Nz=5, spcm=(8, 12), kernel_type="Long_Bott"):
    # r_tot above surface saturation: the shallow test column is cloudy, so
    # droplets and drizzle exist and collisions happen
    st = synthetic.make_icmw_state(Nx=Nx, Nz=Nz, no_spcm=spcm, seed=seed,
                                   kernel_type=kernel_type, drizzle_fraction=0.15,
                                   r_tot=12.5E-3)
    return st


def gen_cells_2d(R):
    out = {}
    variants = [("long", "Long_Bott", "AS", 1.0, False),
                ("hall", "Hall_Bott", "AS", 1.0, False),
                ("hall_nacl", "Hall_Bott", "NaCl", 1.0, False),
                ("const", "Hydro_E_const", "AS", 1.0, False),
                ("boost", "Hall_Bott", "AS", 300.0, True)]
    for name, kt, sol, boost, eqxi in variants:
        st = _small_state(31, kernel_type=("Hall_Bott" if kt == "Hydro_E_const" else kt))
        if kt == "Hydro_E_const":
            E, nb, lo, bl = 0.5, 0, 0.0, 1.0
        else:
            E = st["E_col_grid"]
            nb, lo, bl = st["no_kernel_bins"], st["R_kernel_low_log"], st["bin_factor_R_log"]
        xi = st["xi"].copy()
        if eqxi:
            xi[1::3] = xi[0::3][:len(xi[1::3])] * (1.0 + 1e-7)
        cells = st["cells"].copy()
        # two inactive SIPs (removed at the ground) take no part
        cells[1, 3] = -1
        cells[1, 50] = -1
        m_w, m_s, vel = st["m_w"].copy(), st["m_s"].copy(), st["vel"].copy()
        vel[1] -= 0.01 * st["m_w"] ** (1.0 / 3.0)
        T = st["grid_scalar_fields"][0].copy()
        dtdv = st["dt_col_over_dV"] * boost
        np.random.seed(4242)
        take_draws()
        x_o, mw_o, ms_o = xi.copy(), m_w.copy(), m_s.copy()
        no_cols = np.array([0, 0], dtype=np.int64)
        R.aon.collision_step_Ecol_grid_R_all_cells_2D_multicomp_np(
            x_o, mw_o, ms_o, vel, T, cells, st["grid_no_cells"], dtdv, E,
            nb, lo, bl, no_cols, sol)
        pre = name + "__"
        out.update({pre + "xi_in": xi, pre + "m_w_in": m_w, pre + "m_s_in": m_s,
                    pre + "vel": vel, pre + "T": T, pre + "cells": cells,
                    pre + "no_cells": st["grid_no_cells"],
                    pre + "dt_over_dV": np.float64(dtdv),
                    pre + "E_const": np.float64(E if isinstance(E, float) else -1.0),
                    pre + "kernel": np.array(kt), pre + "solute": np.array(sol),
                    pre + "no_kernel_bins": np.int64(nb),
                    pre + "R_kernel_low_log": np.float64(lo),
                    pre + "bin_factor_R_log": np.float64(bl),
                    pre + "draws": take_draws(), pre + "xi_out": x_o,
                    pre + "m_w_out": mw_o, pre + "m_s_out": ms_o,
                    pre + "no_cols_out": no_cols.copy()})
    save("collision_cells_2d.npz", **out)


def _state_arrays(st):
    keys = ["grid_scalar_fields", "grid_mat_prop", "grid_velocity",
            "grid_mass_flux_air_dry", "grid_no_cells", "grid_ranges",
            "grid_steps", "pos", "vel", "cells", "rel_pos", "m_w", "m_s", "xi",
            "water_removed", "active_ids", "T_p", "delta_m_l",
            "init_profile_r_v", "init_profile_Theta", "relaxation_time_profile"]
    return {k: np.array(st[k]) for k in keys}


def _prepare_removals(st):
    """Send some SIPs to the ground and mark two as already removed."""
    N = st["pos"].shape[1]
    low = np.nonzero(st["cells"][1] == 0)[0]
    st["pos"][1, low[:6]] = 1e-9
    st["vel"][1, low[:6]] = -1.5
    for ID in low[6:8]:
        st["active_ids"][ID] = False
        st["cells"][1, ID] = -1
        st["pos"][1, ID] = -0.2
        st["vel"][:, ID] = 0.0
    # relative positions as the reference computes them
    rp = st["rel_pos"]
    act = st["active_ids"]
    rp[0][act] = st["pos"][0][act] / st["grid_steps"][0] - st["cells"][0][act]
    rp[1][act] = st["pos"][1][act] / st["grid_steps"][1] - st["cells"][1][act]
    return st


def gen_particle_substep(R):
    out = {}
    for sol in ("AS", "NaCl"):
        st = _prepare_removals(_small_state(41, Nx=7, Nz=6, spcm=(6, 8)))
        inp = _state_arrays(st)
        s = copy.deepcopy(inp)
        gsf, gmp = s["grid_scalar_fields"], s["grid_mat_prop"]
        R.integ.propagate_particles_subloop_step_np(
            gsf, gmp, s["grid_velocity"], s["grid_no_cells"], s["grid_ranges"],
            s["grid_steps"], s["pos"], s["vel"], s["cells"], s["rel_pos"],
            s["m_w"], s["m_s"], s["xi"], s["water_removed"],
            np.arange(len(s["xi"])), s["active_ids"], s["T_p"], sol,
            s["delta_m_l"], 0.1, 0.05, 3, 9.80665)
        pre = sol + "__"
        out.update({pre + "in_" + k: v for k, v in inp.items()})
        out.update({pre + "out_" + k: v for k, v in s.items()})
    save("particle_substep.npz", **out)


def gen_grid_and_divergence(R):
    st = _small_state(51, Nx=7, Nz=6, spcm=(3, 3))
    gsf, gmp = st["grid_scalar_fields"].copy(), st["grid_mat_prop"].copy()
    rng = np.random.default_rng(3)
    shape = gsf[0].shape
    dTh = 1e-3 * rng.standard_normal(shape)
    drv = 1e-6 * rng.standard_normal(shape)
    dml = 1e-7 * rng.standard_normal(shape)
    g_out, m_out = gsf.copy(), gmp.copy()
    R.integ.propagate_grid_subloop_step_np(g_out, m_out, st["p_ref"], st["p_ref_inv"],
                                           dTh, drv, dml, st["grid_volume_cell"])
    flux = st["grid_mass_flux_air_dry"]
    div_rv = R.integ.compute_divergence_upwind_np(gsf[4], flux, st["grid_no_cells"],
                                                  st["grid_steps"], np.array([0, 1]))
    div_th = R.integ.compute_divergence_upwind_np(gsf[2], flux, st["grid_no_cells"],
                                                  st["grid_steps"], np.array([0, 1]))
    # a rough field with flat regions exercises the limiter's special cases
    rough = np.round(gsf[2] + 0.3 * rng.standard_normal(shape), 1)
    flux2 = flux * np.sign(rng.standard_normal(flux.shape))
    div_rough = R.integ.compute_divergence_upwind_np(rough, flux2, st["grid_no_cells"],
                                                     st["grid_steps"], np.array([0, 1]))
    relax = R.integ.compute_relaxation_term(gsf[4], st["init_profile_r_v"] * 1.001,
                                            st["relaxation_time_profile"], 0.1)
    save("grid_divergence.npz", gsf_in=gsf, gmp_in=gmp, dTheta=dTh, dr_v=drv,
         dml=dml, p_ref=np.float64(st["p_ref"]), V=np.float64(st["grid_volume_cell"]),
         gsf_out=g_out, gmp_out=m_out, flux=flux, flux2=flux2,
         no_cells=st["grid_no_cells"], steps=st["grid_steps"],
         div_rv=div_rv, div_th=div_th, rough=rough, div_rough=div_rough,
         profile=st["init_profile_r_v"] * 1.001, t_relax=st["relaxation_time_profile"],
         relax=relax)


def gen_interp(R):
    rng = np.random.default_rng(9)
    Nx, Nz = 6, 5
    gv = rng.standard_normal((2, Nx + 1, Nz + 1))
    n = 400
    cells = np.array([rng.integers(0, Nx, n), rng.integers(0, Nz, n)])
    rel = rng.random((2, n))
    rel[1, :40] = np.where(rel[1, :40] > 0.5, 1.0 - rel[1, :40], rel[1, :40])
    cells[1, :20] = 0
    cells[1, 20:40] = Nz - 1
    rel[1, 20:40] = 1.0 - rel[1, 20:40]
    cells[0, 40:60] = 0
    rel[0, 40:60] *= 0.5
    out = R.grid.interpolate_velocity_from_cell_bilinear(cells, rel, gv,
                                                         np.array([Nx, Nz]))
    save("interp.npz", gv=gv, cells=cells, rel=rel, vel=out)


def gen_adv_step(R):
    out = {}
    for name, ncol, kt in [("col2", 2, "Long_Bott"), ("col1", 1, "Hall_Bott"),
                           ("col10", 10, "Long_Bott")]:
        st = _prepare_removals(_small_state(61, Nx=6, Nz=5, spcm=(5, 7),
                                            kernel_type=kt))
        st["no_col_per_adv"] = ncol
        st["dt_col_over_dV"] = (st["dt"] / ncol) / st["grid_volume_cell"]
        inp = _state_arrays(st)
        s = copy.deepcopy(inp)
        no_cols = np.array([0, 0], dtype=np.int64)
        np.random.seed(777)
        take_draws()
        nsteps = 2
        for _ in range(nsteps):
            R.integ.integrate_adv_step_np(
                s["grid_scalar_fields"], s["grid_mat_prop"], s["grid_velocity"],
                s["grid_mass_flux_air_dry"], st["p_ref"], st["p_ref_inv"],
                s["grid_no_cells"], s["grid_ranges"], s["grid_steps"],
                st["grid_volume_cell"], s["pos"], s["vel"], s["cells"],
                s["rel_pos"], s["m_w"], s["m_s"], s["xi"], "AS",
                s["water_removed"], np.arange(len(s["xi"])), s["active_ids"],
                s["T_p"], s["delta_m_l"], st["dt"], st["dt_sub"],
                st["dt_sub_half"], st["dt_col_over_dV"], st["scale_dt_cond"],
                ncol, True, True, s["init_profile_r_v"], s["init_profile_Theta"],
                s["relaxation_time_profile"], 3, 9.80665, st["E_col_grid"],
                st["no_kernel_bins"], st["R_kernel_low_log"],
                st["bin_factor_R_log"], no_cols)
        pre = name + "__"
        out.update({pre + "in_" + k: v for k, v in inp.items()})
        out.update({pre + "out_" + k: v for k, v in s.items()})
        out.update({pre + "draws": take_draws(), pre + "no_cols": no_cols,
                    pre + "nsteps": np.int64(nsteps), pre + "kernel": np.array(kt),
                    pre + "no_col_per_adv": np.int64(ncol),
                    pre + "dt_col_over_dV": np.float64(st["dt_col_over_dV"]),
                    pre + "V": np.float64(st["grid_volume_cell"]),
                    pre + "p_ref": np.float64(st["p_ref"])})
    save("adv_step.npz", **out)


def gen_diagnostics(R):
    """evaluation.py: per-cell mixing ratios, number concentrations and
    radius moments; some SIPs removed at the ground (cells[1] = -1)."""
    import evaluation as ev
    st = _small_state(41, Nx=6, Nz=5, spcm=(8, 12), kernel_type="Hall_Bott")
    N = st["xi"].size
    rng = np.random.default_rng(41)
    cells = st["cells"].copy()
    act = st["active_ids"].copy()
    gone = rng.choice(N, 9, replace=False)
    cells[1, gone] = -1
    act[gone] = False
    m_w, m_s, xi = st["m_w"], st["m_s"], st["xi"]
    R_p = np.cbrt((m_w + m_s) / (4.0 / 3.0 * np.pi * 1.1E3))   # any positive radii
    mass_dry_inv = 1.0 / (rng.uniform(0.9, 1.3, (6, 5)) * 8.0E3)
    id_list = np.arange(N)
    masks = {"active": act, "large": act & (R_p > np.median(R_p)),
             "with_removed": act | np.isin(id_list, gone[:5])}
    out = {"m_w": m_w, "xi": xi, "cells": cells, "active_ids": act, "R_p": R_p,
           "mass_dry_inv": mass_dry_inv, "V0": np.float64(st["grid_volume_cell"]),
           "no_cells": np.array([6, 5])}
    for name, mask in masks.items():
        mr = np.zeros((6, 5))
        ev.update_mixing_ratio(mr, m_w, xi, cells, mass_dry_inv, id_list, mask)
        nc = np.zeros((6, 5))
        ev.update_number_concentration_per_dry_mass(nc, xi, cells, mass_dry_inv, id_list, mask)
        out["mask_" + name] = mask
        out["mixing_ratio_" + name] = mr
        out["number_conc_" + name] = nc
    for n in range(4):
        out[f"moment_{n}"] = ev.compute_moment_R_grid(n, R_p, xi, float(st["grid_volume_cell"]),
                                                      cells, act, id_list, np.array([6, 5]))
    save("diagnostics.npz", **out)


def gen_kernel_grid_m(R):
    """collision/all_or_nothing.py:392-491 on 200 SIPs with a tabulated
    kernel on a logarithmic mass grid, three steps (multiple collections in
    the last)."""
    rng = np.random.default_rng(23)
    n, nb = 200, 60
    m_low_log, bf_log = np.log(1e-3), np.log(10.0) / 6.0
    m_bins = np.exp(m_low_log + bf_log * np.arange(nb))
    Kg = 1.5E-18 * (m_bins[:, None] + m_bins[None, :]) * rng.uniform(0.5, 1.5, (nb, nb))
    xis0 = np.exp(rng.uniform(np.log(1e6), np.log(1e9), n))
    xis0[::37] = xis0[1::37][: len(xis0[::37])]   # some equal multiplicities
    m0 = np.exp(rng.uniform(np.log(1e-2), np.log(1e5), n))
    out = {"xis0": xis0, "m0": m0, "K": Kg, "nb": np.int64(nb), "m_low_log": m_low_log,
           "bf_log": bf_log}
    xis, m = xis0.copy(), m0.copy()
    no_cols = np.zeros(2, dtype=np.int64)
    for step, dtdv in enumerate((50.0, 500.0, 3000.0)):
        R.aon.collision_step_kernel_grid_m_np(xis, m, dtdv, Kg, nb, m_low_log, bf_log, no_cols)
        out[f"draws_{step}"] = take_draws()
        out[f"dtdv_{step}"] = np.float64(dtdv)
        out[f"xis_{step}"] = xis.copy()
        out[f"m_{step}"] = m.copy()
        out[f"no_cols_{step}"] = no_cols.copy()
    save("collision_kernel_grid_m.npz", **out)


def gen_tables(R):
    out = {}
    for kt in ("Long_Bott", "Hall_Bott"):
        E = np.load(f"Ecol_grid_data/{kt}/E_col_grid.npy")
        rg = np.load(f"Ecol_grid_data/{kt}/radius_grid_out.npy")
        out[kt + "__E_sha256"] = np.array(hashlib.sha256(E.tobytes()).hexdigest())
        out[kt + "__r_sha256"] = np.array(hashlib.sha256(rg.tobytes()).hexdigest())
        out[kt + "__shape"] = np.array(E.shape)
        out[kt + "__r_head"] = rg[:4]
    save("tables.npz", **out)


def gen_box_model_kgrid(R):
    """collision/box_model.py:44-205 simulate_collisions with
    kernel_method='kernel_grid_m': 150 SIPs, 6 steps saved every 2 s, the
    draws from NumPy's generator seeded with the run's seed."""
    import tempfile
    import collision.box_model as bm
    rng = np.random.default_rng(29)
    n, nb = 150, 60
    m_low_log, bf_log = np.log(1e-3), np.log(10.0) / 6.0
    m_bins = np.exp(m_low_log + bf_log * np.arange(nb))
    Kg = 1.5E-18 * (m_bins[:, None] + m_bins[None, :]) * rng.uniform(0.5, 1.5, (nb, nb))
    xis0 = np.exp(rng.uniform(np.log(1e6), np.log(1e9), n))
    m0 = np.exp(rng.uniform(np.log(1e-2), np.log(1e5), n))
    xis, m = xis0.copy(), m0.copy()
    no_cols = np.zeros(2, dtype=np.int64)
    seed, dV, dt, t_end, dt_save = 3711, 1.0E-3, 1.0, 6.0, 2.0
    with tempfile.TemporaryDirectory() as d:
        bm.simulate_collisions((xis, m), (Kg, nb, m_low_log, bf_log), "Long_Bott",
                               "kernel_grid_m", dV, dt, t_end, dt_save, no_cols, seed,
                               d + "/")
        xt = np.load(d + f"/xis_vs_time_{seed}.npy")
        mt = np.load(d + f"/masses_vs_time_{seed}.npy")
        tt = np.load(d + f"/save_times_{seed}.npy")
    take_draws()
    save("box_model_kgrid.npz", xis0=xis0, m0=m0, K=Kg, nb=np.int64(nb), m_low_log=m_low_log,
         bf_log=bf_log, seed=np.int64(seed), dV=dV, dt=dt, t_end=t_end, dt_save=dt_save,
         xis_vs_time=xt, masses_vs_time=mt, save_times=tt, no_cols=no_cols, xis=xis, m=m)


def gen_file_formats(R):
    """file_handling.py: the full-state files (save_grid_and_particles_full)
    and the frame files (save_grid_scalar_fields, dump_particle_data_all,
    dump_particle_data, dump_particle_tracer_data_block,
    save_sim_paras_to_file) the reference writes for a small seeded state,
    byte for byte, and what its load_grid_and_particles_full returns."""
    import tempfile
    st = _small_state(71, Nx=6, Nz=5, spcm=(4, 6))
    st["active_ids"][::17] = False
    st["cells"][1, ~st["active_ids"]] = -1
    steps = np.asarray(st["grid_steps"])
    dy = float(st["grid_volume_cell"]) / (steps[0] * steps[1])
    grid = R.grid.Grid(np.array(st["grid_ranges"]), steps, dy)
    gsf, gmp = st["grid_scalar_fields"], st["grid_mat_prop"]
    names = ("temperature", "pressure", "potential_temperature", "mass_density_air_dry",
             "mixing_ratio_water_vapor", "mixing_ratio_water_liquid", "saturation",
             "saturation_pressure", "mass_dry_inv", "rho_dry_inv")
    for k, nm in enumerate(names):
        setattr(grid, nm, gsf[k].copy())
    grid.velocity = st["grid_velocity"].copy()
    grid.mass_flux_air_dry = st["grid_mass_flux_air_dry"].copy()
    t = 600
    out = {}
    with tempfile.TemporaryDirectory() as d:
        path = d + "/"
        R.fh.save_grid_and_particles_full(t, grid, st["pos"], st["cells"], st["vel"], st["m_w"],
                                          st["m_s"], st["xi"], st["active_ids"], path)
        loaded = R.fh.load_grid_and_particles_full(t, path)
        R.fh.save_grid_scalar_fields(t, gsf, path, __import__("datetime").datetime.now())
        R.fh.dump_particle_data_all(t, st["pos"], st["vel"], st["cells"], st["m_w"], st["m_s"],
                                    st["xi"], st["active_ids"], path)
        tr = np.arange(3, st["xi"].size, 40)
        R.fh.dump_particle_data(t, st["pos"][:, tr], st["vel"][:, tr], st["m_w"][tr],
                                st["m_s"][tr], st["xi"][tr], gsf[0], gsf[4], path)
        tb = np.array([t + 60, t + 80])
        R.fh.dump_particle_tracer_data_block(
            tb, np.stack([np.array([st["pos"][:, tr], st["vel"][:, tr]])] * 2),
            np.stack([np.array([st["m_w"][tr], st["m_s"][tr], st["T_p"][tr]])] * 2),
            np.stack([st["xi"][tr]] * 2), np.array([0.5, 0.75]), path)
        R.fh.save_sim_paras_to_file([1.0, 0.1, 3, 6001], "dt dt_sub no_iter_impl_mass rnd_seed_sim",
                                    t, path)
        for fn in sorted(os.listdir(d)):
            out["file__" + fn] = np.frombuffer(open(path + fn, "rb").read(), dtype=np.uint8)
    g = loaded[0]
    for nm in ("pressure", "temperature", "potential_temperature", "mass_density_air_dry",
               "mixing_ratio_water_vapor", "mixing_ratio_water_liquid", "saturation",
               "saturation_pressure", "mass_dry_inv", "rho_dry_inv", "thermal_conductivity",
               "diffusion_constant", "heat_of_vaporization", "surface_tension",
               "specific_heat_capacity", "viscosity", "mass_density_fluid", "velocity",
               "mass_flux_air_dry", "ranges", "steps", "no_cells"):
        out["grid__" + nm] = np.asarray(getattr(g, nm))
    out["grid__step_y"] = np.float64(g.step_y)
    out["grid__volume_cell"] = np.float64(g.volume_cell)
    for nm, a in zip(("pos", "cells", "vel", "m_w", "m_s", "xi", "active_ids"), loaded[1:]):
        out["in__" + nm] = np.asarray(st[nm])
        out["loaded__" + nm] = np.asarray(a)
    for k, nm in enumerate(names):
        out["in__gsf_" + nm] = gsf[k]
    out["in__grid_mat_prop"] = gmp
    out["in__T_p"] = st["T_p"]
    out["in__grid_ranges"] = np.asarray(st["grid_ranges"])
    out["in__grid_steps"] = steps
    out["in__dy"] = np.float64(dy)
    out["in__trace_ids"] = tr
    out["t"] = np.int64(t)
    save("file_formats.npz", **out)


def gen_kernel_generators(R):
    """collision/kernel.py:793-942: kernel grids K(R1, R2) with Beard
    velocities for the Long and Hall efficiencies on two radius grids."""
    out = {}
    for kt, fn in (("Long_Bott", R.ker.generate_kernel_grid_Long_Bott_np),
                   ("Hall_Bott", R.ker.generate_kernel_grid_Hall_Bott_np)):
        for args in ((0.6, 2000.0, 10, 1000.0), (1.0, 4000.0, 20, 1000.0)):
            K, v, m, rg = fn(*args)
            tag = f"{kt}_{args[2]}"
            out[tag + "__args"] = np.array(args, dtype=np.float64)
            out[tag + "__K"] = K
            out[tag + "__vel"] = v
            out[tag + "__mass"] = m
            out[tag + "__radius"] = rg
    save("kernel_generators.npz", **out)


def gen_evaluation(R):
    """evaluation.py:1172-1660 on frames the reference's own writers saved
    (two seeds, two save times, small grids): size spectra around target
    cells, per-cell moments of every seed and time, box averages."""
    import datetime
    import tempfile
    sys.modules.pop("evaluation", None)
    import evaluation as ev
    out = {}
    times = np.array([0, 10])
    with tempfile.TemporaryDirectory() as d:
        paths = []
        for k in range(2):
            path = d + f"/seed{k}/"
            os.makedirs(path)
            for tn, t in enumerate(times):
                st = _small_state(90 + 10 * k + tn, Nx=6, Nz=5, spcm=(6, 8))
                st["active_ids"][::23] = False
                st["cells"][1, ~st["active_ids"]] = -1
                R.fh.save_grid_scalar_fields(t, st["grid_scalar_fields"], path,
                                             datetime.datetime.now())
                R.fh.dump_particle_data_all(t, st["pos"], st["vel"], st["cells"], st["m_w"],
                                            st["m_s"], st["xi"], st["active_ids"], path)
            np.save(path + "grid_save_times.npy", times)
            np.save(path + "data_saving_paras.npy", (10, 1, 10))
            paths.append(path)
            for fn in sorted(os.listdir(path)):
                out[f"file__seed{k}__{fn}"] = np.frombuffer(open(path + fn, "rb").read(),
                                                            dtype=np.uint8)
        mdi = st["grid_scalar_fields"][8]
        tg = np.array([[2, 4], [1, 3]])
        spec = ev.generate_size_spectra_R(paths, np.array([0, 1]), mdi, np.array([6, 5]), "AS",
                                          tg, 3, 3, 12, 8)
        for nm, a in zip(("f_R_p", "f_R_s", "bins_R_p", "bins_R_s", "save_times", "r_l",
                          "R_min", "R_max"), spec):
            out["spec__" + nm] = np.asarray(a)
        mom, mt = ev.generate_moments_all_seeds(paths, 4, np.array([0, 1]),
                                                float(st["grid_volume_cell"]),
                                                np.array([6, 5]), "AS")
        out["mom__moments"] = mom
        out["mom__save_times"] = mt
        out["box__avg"] = ev.avg_moments_over_boxes(mom, 2, np.array([0, 1]), 4,
                                                    np.array([1, 4]), np.array([1, 3]), 3, 3)
    out["in__mass_dry_inv"] = mdi
    out["in__target_cells"] = tg
    out["in__volume_cell"] = np.float64(st["grid_volume_cell"])
    save("evaluation.npz", **out)


def init_config(path, no_cells=(3, 15), steps=(20.0, 100.0), no_spcm=(4, 6), seed=1001,
                eta_threshold="fix"):
    """A small ICMW 2012 case 1 configuration with the reference's values
    (config.py:64-132) on a narrow column of few cells."""
    return {
        "paths": {"simdata": path}, "seed_SIP_gen": seed, "seed_sim": seed + 5000,
        "reseed": False, "solute_type": "AS",
        "grid_ranges": [[0.0, no_cells[0] * steps[0]], [0.0, no_cells[1] * steps[1]]],
        "grid_steps": list(steps), "dy": 1.0, "no_cells": np.array(no_cells),
        "p_0": 1015E2, "p_ref": 1E5, "r_tot_0": 7.5E-3, "Theta_l": 289.0,
        "no_spcm": list(no_spcm), "dist": "lognormal",
        "DNC0": np.array([60.0E6, 40.0E6]), "mu_R": 0.5 * np.array([0.04, 0.15]),
        "sigma_R": np.array([1.4, 1.6]), "eta": 1E-10, "eta_threshold": eta_threshold,
        "r_critmin": np.array([1., 3.]) * 1E-3, "m_high_over_m_low": 1.0E8,
        "S_init_max": 1.04, "dt_init": 0.1, "Newton_iterations": 2, "iter_cnt_limit": 4000}


def gen_init(R):
    """init.py:439-1236 initialize_grid_and_particles_SinSIP on a 3 x 15
    column (dz = 100 m: the upper levels are cloudy), with the generation
    configuration of set_config (init.py:43-108)."""
    import tempfile
    import init as ref_init
    out = {}
    for tag, eta_thr in (("fix", "fix"), ("weak", "weak")):
        with tempfile.TemporaryDirectory() as d:
            cfg = init_config(d + "/", eta_threshold=eta_thr)
            ref_init.set_config(cfg, "generation")
            grid, pos, cells, vel, m_w, m_s, xi, act = \
                ref_init.initialize_grid_and_particles_SinSIP(cfg)
            out[tag + "__dist_par"] = np.array(cfg["dist_par"])
            out[tag + "__idx_mode_nonzero"] = np.asarray(cfg["idx_mode_nonzero"])
            out[tag + "__no_modes"] = np.int64(cfg["no_modes"])
            for nm, a in (("pos", pos), ("cells", cells), ("vel", vel), ("m_w", m_w),
                          ("m_s", m_s), ("xi", xi), ("active_ids", act)):
                out[tag + "__" + nm] = np.asarray(a)
            for nm in ("pressure", "temperature", "potential_temperature",
                       "mass_density_air_dry", "mixing_ratio_water_vapor",
                       "mixing_ratio_water_liquid", "saturation", "saturation_pressure",
                       "mass_dry_inv", "velocity", "mass_flux_air_dry"):
                out[tag + "__grid_" + nm] = np.asarray(getattr(grid, nm))
            out[tag + "__modes"] = np.load(cfg["paths"]["grid"] + "modes_0.npy")
    save("init.npz", **out)


def gen_wang2007(R):
    """The bin-model moments of Wang et al. (2007) the reference compares its
    box model with (collision/ref_data/{Long_Bott,Hall_Bott}/
    Wang_2007_{moments,times}.txt, read at run_box_model.py:458-469), as
    shipped."""
    out = {}
    for kt in ("Long_Bott", "Hall_Bott"):
        d = "collision/ref_data/" + kt + "/"
        out[kt + "__moments"] = np.loadtxt(d + "Wang_2007_moments.txt")
        out[kt + "__times"] = np.loadtxt(d + "Wang_2007_times.txt")
    save("wang2007.npz", **out)


def gen_golovin_moments(R):
    """golovin.compute_moments_Golovin (golovin.py:48-58) of the box-model
    setup (config 1's DNC and LWC, b = 1.5 m^3 kg^-1 s^-1) at the report's
    save times, moments 0..3."""
    DNC, LWC, b = 2.97E8, 1.0E-3, 1.5
    t = np.arange(0.0, 3601.0, 600.0)
    mom = np.array([[R.golovin.compute_moments_Golovin(tt, n, DNC, LWC, b) for tt in t]
                    for n in range(4)])
    save("golovin_moments.npz", t=t, moments=mom, DNC=np.float64(DNC), LWC=np.float64(LWC),
         b=np.float64(b))


GENERATORS = [gen_tables, gen_mass_rate, gen_interp, gen_golovin, gen_ecol_box, gen_cells_2d,
              gen_grid_and_divergence, gen_particle_substep, gen_adv_step, gen_diagnostics,
              gen_kernel_grid_m, gen_box_model_kgrid, gen_file_formats,
              gen_kernel_generators, gen_evaluation,
              gen_init, gen_wang2007, gen_golovin_moments]


def main(ref_root, only=()):
    R = refstub.import_reference(ref_root)
    np.random.rand = _recording_rand
    for g in GENERATORS:
        if not only or g.__name__[len("gen_"):] in only:
            g(R)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <reference root> [fixture ...]")
    main(os.path.abspath(sys.argv[1]), set(sys.argv[2:]))
