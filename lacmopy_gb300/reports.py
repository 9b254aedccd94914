"""Measurement reports of the hot path on the GPU.

``golovin_box``: the collision box model with the Golovin kernel
(collision/box_model.py:44-205 driving collision/all_or_nothing.py:109-185),
an exponential initial mass distribution (R_mean = 9.3 um, LWC = 1 g m^-3,
rho = 1000 kg m^-3; run_box_model.py:133-153) and the moments of the SIP
ensemble against the analytic solution of the additive kernel
K = b (m1 + m2): dM0/dt = -b M1 M0, M1 constant, dM2/dt = 2 b M1 M2, so
M0(t) = M0(0) exp(-b M1 t) and M2(t) = M2(0) exp(2 b M1 t) (Golovin 1963).

``precision``: the mixed-precision path against the FP64 path from the same
spun-up 2-D state with the same Philox draws; per-output error statement.
``precision-ensemble``: the same comparison as ensemble statistics over
members with different collision draws (means, standard errors, confidence
intervals of the mixed - FP64 difference).

    python -m lacmopy_gb300.reports golovin [--kappa K] [--t-end T] [--seeds S ...]
    python -m lacmopy_gb300.reports precision [--spcm A B] [--spinup N] [--horizons N ...]
    python -m lacmopy_gb300.reports precision-ensemble [--members M] [--spinup N] [--horizon H]
    python -m lacmopy_gb300.reports adjoint [--spcm A B]

``adjoint``: gradients of the domain-mean liquid water path and the surface
rain after 600 s of the product's time step (collisions off, recorded cells)
with respect to per-SIP solute mass, hygroscopicity and the mass-flux scale
j_max (lacmopy_gb300.adjoint), timing, and finite-difference checks.
"""
import argparse
import ctypes
import json
import math
import time

import numpy as np

B_GOLOVIN = 1.5   # m^3 kg^-1 s^-1 (1500 cm^3 g^-1 s^-1), collision/kernel.py:461-480


def golovin_box(kappa=1000, t_end=600.0, dt=1.0, seeds=(1001, 1003), dt_save=None):
    """Run the GPU machine model (Philox draws) for each seed and compare the
    moments with the analytic Golovin solution at the save times."""
    import torch
    from . import collision, synthetic
    dt_save = dt_save or t_end
    rows = []
    pairs = 0
    secs = 0.0
    for seed in seeds:
        xis, masses, DNC0, LWC0 = synthetic.make_golovin_box(kappa=kappa, seed=seed)
        n = len(xis)
        no_cols = np.zeros(2, dtype=np.int64)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xs, ms, ts = collision.simulate_collisions((xis, masses), None, "Golovin", None, 1.0, dt,
                                                   t_end, dt_save, no_cols, seed,
                                                   draws="philox")
        torch.cuda.synchronize()
        secs += time.perf_counter() - t0
        pairs += n * (n - 1) // 2 * int(math.ceil(t_end / dt))
        m0 = [float(x.sum()) for x in xs]
        m1 = [float((x * m).sum()) for x, m in zip(xs, ms)]
        m2 = [float((x * m * m).sum()) for x, m in zip(xs, ms)]
        bM1 = B_GOLOVIN * LWC0   # s^-1 (b [m^3/kg/s] * M1 [kg/m^3])
        for k, t in enumerate(ts):
            rows.append({"seed": seed, "n_sips": n, "t": float(t),
                         "M0_rel": m0[k] / (m0[0] * math.exp(-bM1 * t)) - 1.0,
                         "M1_rel": m1[k] / m1[0] - 1.0,
                         "M2_rel": m2[k] / (m2[0] * math.exp(2.0 * bM1 * t)) - 1.0,
                         "no_cols": int(no_cols.sum())})
    final = [r for r in rows if r["t"] == max(r2["t"] for r2 in rows)]
    return {"rows": rows,
            "mean_M0_rel_final": float(np.mean([r["M0_rel"] for r in final])),
            "mean_M2_rel_final": float(np.mean([r["M2_rel"] for r in final])),
            "max_abs_M1_rel": float(max(abs(r["M1_rel"]) for r in rows)),
            "pair_evaluations_per_s": pairs / secs if secs > 0 else None,
            "wall_s": secs}


def compute_moments_Golovin(t, n, DNC, LWC, b):
    """golovin.py:48-58: the moments 0..3 of the Golovin solution from an
    exponential mass distribution (SI units)."""
    if n == 0:
        return DNC * np.exp(-b * LWC * t)
    if n == 1:
        return LWC
    if n == 2:
        return 2 * LWC * LWC / DNC * np.exp(2 * b * LWC * t)
    return LWC ** 3 / (DNC ** 2) * (12 * np.exp(4 * b * LWC * t) - 6 * np.exp(3 * b * LWC * t))


def golovin_ensemble(seeds=tuple(range(1001, 1041, 2)), kappa=1000, t_end=3600.0, dt=1.0,
                     dt_save=600.0, dV=1.0):
    """Config 1 as ensemble statistics: one box-model run per seed (the
    single-CTA box kernels of all seeds run side by side, one CUDA stream
    each, Philox draws), the moments M0..M3 (SI) of every run at the save
    times, their mean over the seeds with its standard error, against the
    analytic Golovin moments (golovin.py:48-58) of the runs' common initial
    DNC and LWC (their ensemble means: the sampled distribution is cut at
    0.6 um)."""
    import torch
    from . import _lib, synthetic
    from .device import _ptr, to_device
    lib = _lib.load()
    runs = []
    DNC0 = LWC0 = None
    for sd in seeds:
        xis, masses, DNC0, LWC0 = synthetic.make_golovin_box(kappa=kappa, seed=sd, dV=dV)
        runs.append({"x": to_device(xis), "m": to_device(masses),
                     "nc": torch.zeros(2, dtype=torch.int64, device="cuda"),
                     "stream": torch.cuda.Stream(), "seed": sd})
    no_steps = int(math.ceil(t_end / dt))
    dn = int(math.ceil(dt_save / dt))
    save_steps = list(range(0, no_steps, dn)) + [no_steps]
    mom = {sd: [] for sd in seeds}

    def moments(r):
        x, m = r["x"], r["m"] * 1.0E-18
        return [float((x * m ** k).sum()) / dV for k in range(4)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for step in range(no_steps + 1):
        if step in save_steps:
            torch.cuda.synchronize()
            for r in runs:
                mom[r["seed"]].append(moments(r))
        if step == no_steps:
            break
        for r in runs:
            n = r["x"].numel()
            _lib.check(lib.lacmo_collision_step_golovin(
                _ptr(r["x"]), _ptr(r["m"]), n, dt / dV, _ptr(r["nc"]), None, int(r["seed"]),
                step, ctypes.c_void_p(r["stream"].cuda_stream)), "golovin")
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    M = np.array([mom[sd] for sd in seeds])   # [seed, save, moment]
    # the analytic solution from the ensemble's own initial number and mass
    # (the sampled distribution is truncated at 0.6 um, 3e-4 of the number)
    DNC_s, LWC_s = float(M[:, 0, 0].mean()), float(M[:, 0, 1].mean())
    rows = []
    for k, st_ in enumerate(save_steps):
        t = st_ * dt
        row = {"t": t}
        for n in range(4):
            vals = M[:, k, n]
            ana = compute_moments_Golovin(t, n, DNC_s, LWC_s, B_GOLOVIN)
            se = float(vals.std(ddof=1) / math.sqrt(len(seeds)))
            row[f"M{n}_mean"] = float(vals.mean())
            row[f"M{n}_analytic"] = float(ana)
            row[f"M{n}_rel"] = float(vals.mean() / ana - 1.0)
            row[f"M{n}_se_rel"] = se / float(ana)
            row[f"M{n}_dev_over_se"] = float((vals.mean() - ana) / se) if se > 0 else 0.0
        rows.append(row)
    M1_cons = float(np.max(np.abs(M[:, :, 1] / M[:, :1, 1] - 1.0)))
    return {"seeds": len(seeds), "n_sips": int(runs[0]["x"].numel()), "t_end": t_end,
            "DNC0_nominal": DNC0, "LWC0_nominal": LWC0, "DNC0": DNC_s, "LWC0": LWC_s,
            "M1_conservation_max_rel": M1_cons, "rows": rows, "wall_s": wall}


def box_ecol_ensemble(kernel_name="Long_Bott", seeds=tuple(range(1001, 1021, 2)), kappa=600,
                      t_end=3600.0, dt=1.0, dt_save=200.0, dV=1.0):
    """The box model with the Long or Hall efficiency table and Beard
    velocities (collision/box_model.py:44-205 with collision/all_or_nothing.py:
    269-390), from the exponential distribution of config 1: one run per
    seed, the runs side by side on their own CUDA streams; the moments M0..M3
    (SI) averaged over the seeds at the save times, for comparison with the
    bin-model moments of Wang et al. (2007) the reference plots against
    (run_box_model.py:458-469)."""
    import torch
    from . import _lib, synthetic, tables
    from .device import _ptr, to_device
    lib = _lib.load()
    E, rg, R_low, bf, lo, bl, nb = tables.load_kernel_data_Ecol(kernel_name)
    E_d = to_device(E)
    runs = []
    for sd in seeds:
        xis, masses, DNC0, LWC0 = synthetic.make_golovin_box(kappa=kappa, seed=sd, dV=dV)
        if xis.size > _lib.ECOL_BOX_MAX_SIPS:
            raise ValueError(f"{xis.size} SIPs: above the box kernel's {_lib.ECOL_BOX_MAX_SIPS}")
        R = np.cbrt(masses / (4.0 / 3.0 * math.pi * 1000.0))   # um (fg, kg/m^3)
        runs.append({"x": to_device(xis), "m": to_device(masses), "R": to_device(R),
                     "v": torch.zeros(xis.size, dtype=torch.float64, device="cuda"),
                     "rho": torch.full((xis.size,), 1000.0, dtype=torch.float64, device="cuda"),
                     "nc": torch.zeros(2, dtype=torch.int64, device="cuda"),
                     "stream": torch.cuda.Stream(), "seed": sd})
    for r in runs:
        _lib.check(lib.lacmo_update_velocity_beard(_ptr(r["v"]), _ptr(r["R"]), r["R"].numel(),
                                                   ctypes.c_void_p(r["stream"].cuda_stream)),
                   "beard")
    no_steps = int(math.ceil(t_end / dt))
    dn = int(math.ceil(dt_save / dt))
    save_steps = list(range(0, no_steps, dn)) + [no_steps]
    mom = {r["seed"]: [] for r in runs}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for step in range(no_steps + 1):
        if step in save_steps:
            torch.cuda.synchronize()
            for r in runs:
                x, m = r["x"], r["m"] * 1.0E-18
                mom[r["seed"]].append([float((x * m ** k).sum()) / dV for k in range(4)])
        if step == no_steps:
            break
        for r in runs:
            sp = ctypes.c_void_p(r["stream"].cuda_stream)
            n = r["x"].numel()
            _lib.check(lib.lacmo_collision_step_ecol_grid_r_box(
                _ptr(r["x"]), _ptr(r["m"]), _ptr(r["R"]), _ptr(r["v"]), _ptr(r["rho"]), n,
                dt / dV, _ptr(E_d), int(nb), float(lo), float(bl), _ptr(r["nc"]), None,
                int(r["seed"]), step, sp), "ecol_box")
            _lib.check(lib.lacmo_update_velocity_beard(_ptr(r["v"]), _ptr(r["R"]), n, sp),
                       "beard")
    torch.cuda.synchronize()
    M = np.array([mom[r["seed"]] for r in runs])
    times = np.array(save_steps) * dt
    return {"kernel": kernel_name, "seeds": len(runs), "n_sips": int(runs[0]["x"].numel()),
            "times": times.tolist(), "moments_mean": M.mean(axis=0).T.tolist(),
            "moments_se": (M.std(axis=0, ddof=1) / math.sqrt(len(runs))).T.tolist(),
            "wall_s": time.perf_counter() - t0}


def _spin_up(st, steps, seed, draws="philox"):
    """The reference's spin-up (init.py:137-146: without gravity, collisions
    and relaxation) of ``steps`` advection steps in FP64, in place on the
    state dict; the simulation's own settings are kept for what follows."""
    from . import DeviceState
    if not steps:
        return
    keep = {k: st[k] for k in ("act_collisions", "act_relaxation", "g_set")}
    st.update(act_collisions=False, act_relaxation=False, g_set=0.0)
    d = DeviceState(st, draws=draws, seed=seed, precision="fp64")
    d.adv_step(steps, graph=True)
    d.export_to(st)
    del d
    st.update(keep)


def _lwp(s):
    return float((s["m_w"] * s["xi"] * s["active_ids"]).sum())


def precision(spcm=(52, 76), nx=75, nz=75, spinup=60, horizons=(10, 60), seed=1001,
              kernel="Long_Bott"):
    """Spin up in FP64 (the reference's spin-up: no gravity, collisions or
    relaxation), then advance copies of the spun-up state: FP64 and mixed
    precision with identical Philox draws, and FP64 with other draws (the
    seed-to-seed spread of the stochastic collisions, the noise floor of any
    comparison once collision outcomes differ).  Errors of the mixed run
    relative to the FP64 run at each horizon (steps after the spin-up)."""
    from . import DeviceState, synthetic
    st = synthetic.make_icmw_state(Nx=nx, Nz=nz, no_spcm=tuple(spcm), seed=seed,
                                   kernel_type=kernel)
    _spin_up(st, spinup, seed)
    cp = lambda: {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
    a = DeviceState(cp(), draws="philox", seed=seed + 1, precision="fp64")
    b = DeviceState(cp(), draws="philox", seed=seed + 1, precision="mixed")
    c = DeviceState(cp(), draws="philox", seed=seed + 2, precision="fp64")
    rel = lambda x, y: np.abs(x - y) / np.maximum(np.abs(y), 1e-300)

    def radius(s):
        return np.cbrt((s["m_w"] + s["m_s"]) / (4.0 / 3.0 * math.pi * 1000.0))

    rows = []
    done = 0
    for h in sorted(horizons):
        for ds in (a, b, c):
            ds.adv_step(h - done, graph=True)
            ds.update_grid_r_l()
        done = h
        A, B, Cn = a.snapshot(), b.snapshot(), c.snapshot()
        both = A["active_ids"] & B["active_ids"]
        mw = rel(B["m_w"][both], A["m_w"][both])
        rp = rel(radius(B)[both], radius(A)[both])
        g64, gmx, gno = A["grid_scalar_fields"], B["grid_scalar_fields"], Cn["grid_scalar_fields"]
        rows.append({
            "steps": h, "n_sips": int(A["xi"].size),
            "lwp_rel": abs(_lwp(B) - _lwp(A)) / _lwp(A),
            "lwp_rel_seed_spread": abs(_lwp(Cn) - _lwp(A)) / _lwp(A),
            "m_w_rel_median": float(np.median(mw)), "m_w_rel_p99": float(np.quantile(mw, 0.99)),
            "R_p_rel_median": float(np.median(rp)), "R_p_rel_p99": float(np.quantile(rp, 0.99)),
            "theta_rel_max": float(np.max(rel(gmx[2], g64[2]))),
            "theta_rel_max_seed_spread": float(np.max(rel(gno[2], g64[2]))),
            "r_v_rel_max": float(np.max(rel(gmx[4], g64[4]))),
            "r_v_rel_max_seed_spread": float(np.max(rel(gno[4], g64[4]))),
            "r_l_abs_over_max": float(np.max(np.abs(gmx[5] - g64[5])) / np.max(np.abs(g64[5]))),
            "r_l_abs_over_max_seed_spread": float(np.max(np.abs(gno[5] - g64[5]))
                                                  / np.max(np.abs(g64[5]))),
            "xi_differ_frac": float(np.mean(A["xi"] != B["xi"])),
            "no_cols_fp64": A["no_cols"].tolist(), "no_cols_mixed": B["no_cols"].tolist(),
            "no_cols_seed_spread": Cn["no_cols"].tolist(),
            "water_removed_rel": float(abs(B["water_removed"][0] - A["water_removed"][0])
                                       / max(abs(A["water_removed"][0]), 1e-300)),
            "cells_differ_frac": float(np.mean((A["cells"] != B["cells"]).any(axis=0))),
            "newton_fp64_repeats": b.fallbacks(),
        })
    return {"spinup_steps": spinup, "rows": rows}


def _member_stats(b, m, horizon, wr0):
    sn = b.snapshot(m)
    g = sn["grid_scalar_fields"]
    return {"lwp": _lwp(sn), "theta_mean": float(g[2].mean()), "r_v_mean": float(g[4].mean()),
            "rain_flux": float(sn["water_removed"][0] - wr0) / horizon,
            "no_cols": int(sn["no_cols"].sum())}


def precision_ensemble(members=16, spcm=(52, 76), nx=75, nz=75, spinup=7200, horizon=3600,
                       seed=1001, kernel="Long_Bott", **state_kw):
    """The precision form as ensemble statistics.  One state is spun up in
    FP64 (the reference's spin-up: no gravity, collisions or relaxation);
    ``members`` copies of it then advance ``horizon`` steps with
    collision draws keyed by different seeds, once in FP64 and once in mixed
    precision (member k has the same seed in both).  Collision outcomes
    make the members different realisations, so the mixed and FP64 paths are
    compared through the ensemble means of the domain liquid water (LWP
    proxy: sum of m_w xi), mean Theta, mean r_v and rain flux (water removed
    per second), with the standard error of each mean (seed-to-seed spread /
    sqrt(members)): the mixed path agrees when the difference of the means
    stays within a few standard errors of the difference."""
    from . import BatchState, DeviceState, synthetic
    st = synthetic.make_icmw_state(Nx=nx, Nz=nz, no_spcm=tuple(spcm), seed=seed,
                                   kernel_type=kernel, **state_kw)
    t0 = time.perf_counter()
    _spin_up(st, spinup, seed, draws="thinned")
    wr0 = float(st["water_removed"][0])
    seeds = [seed + 100 + k for k in range(members)]
    out = {"members": members, "spinup_steps": spinup, "horizon_steps": horizon,
           "n_sips_per_member": int(st["xi"].size), "kernel": kernel}
    stats = {}
    for prec in ("fp64", "mixed"):
        states = [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
                  for _ in range(members)]
        b = BatchState(states, seeds, precision=prec, draws="thinned")
        b.adv_step(horizon, graph=True)
        for m in range(members):
            b.update_grid_r_l(m)
        stats[prec] = [_member_stats(b, m, horizon, wr0) for m in range(members)]
        del b
    for key in ("lwp", "theta_mean", "r_v_mean", "rain_flux"):
        a = np.array([r[key] for r in stats["fp64"]])
        bm = np.array([r[key] for r in stats["mixed"]])
        se = math.sqrt(a.var(ddof=1) / members + bm.var(ddof=1) / members)
        diff = float(bm.mean() - a.mean())
        out[key] = {"fp64_mean": float(a.mean()), "mixed_mean": float(bm.mean()),
                    "fp64_sd": float(a.std(ddof=1)), "mixed_sd": float(bm.std(ddof=1)),
                    "diff": diff, "se_diff": se,
                    "diff_over_se": diff / se if se > 0 else 0.0,
                    "diff_rel": diff / abs(float(a.mean())) if a.mean() != 0 else 0.0,
                    "ci95_diff": [diff - 1.96 * se, diff + 1.96 * se]}
    out["no_cols_mean"] = {p: float(np.mean([r["no_cols"] for r in stats[p]])) for p in stats}
    out["wall_s"] = time.perf_counter() - t0
    return out


def adjoint(spcm=(52, 76), nx=75, nz=75, seconds=600, every_steps=60, seed=1001,
            kappa=0.6, fd_h=1e-5):
    """Gradients of the domain-mean liquid water path at the end and of the
    surface rain over ``seconds`` of the product's time step (with the
    state's collisions; the SIPs' cells and the collisions recorded from the
    product's own run and held fixed) by m_s, kappa and the mass-flux scale
    (dJ/dj_max = that / j_max),
    checkpointed every ``every_steps`` advection steps; the forward model
    against the product's run, timing, and central finite differences of the
    kappa and flux-scale derivatives."""
    import torch
    from . import adjoint as adj, synthetic
    st = synthetic.make_icmw_state(Nx=nx, Nz=nz, no_spcm=tuple(spcm), seed=seed,
                                   kernel_type="Long_Bott")
    n_adv = int(round(seconds / float(st["dt"])))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    model = adj.StepModel(st, n_adv)
    torch.cuda.synchronize()
    t_rec = time.perf_counter() - t0
    m_w, _, _ = model.run()
    rel = float(((m_w - model.product.m_w).abs() / model.product.m_w.abs().clamp_min(1e-300))
                .max())
    # init.py:1146-1148, the domain sizes Lx, Lz
    Lx, Lz = (float(a) * float(b) for a, b in zip(st["grid_steps"], st["grid_no_cells"]))
    j_max = 0.6 * math.sqrt(Lx * Lx + Lz * Lz) / math.sqrt(2.0 * 1500.0 * 1500.0)
    out = {"n_sips": model.n, "advection_steps": n_adv, "sub_steps": model.K,
           "collisions": model.collisions, "collision_events": int(model.n_events),
           "record_s": t_rec, "replay_max_rel_diff_m_w": rel, "j_max": j_max}
    for name, w in (("lwp", model.lwp_weights()), ("rain", model.rain_weights())):
        m_s = model.m_s0.clone().requires_grad_(True)
        k = torch.tensor(kappa, dtype=torch.float64, device="cuda", requires_grad=True)
        sc = torch.tensor(1.0, dtype=torch.float64, device="cuda", requires_grad=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        J = adj.objective(model, m_s, k, sc, weights=w, checkpoint_every=every_steps)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        J.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()

        def J_of(**kw):
            m, _, _ = model.run(**kw)
            return float((w * m).sum())
        fd_k = (J_of(kappa=kappa + fd_h) - J_of(kappa=kappa - fd_h)) / (2 * fd_h)
        fd_s = (J_of(flux_scale=1.0 + fd_h) - J_of(flux_scale=1.0 - fd_h)) / (2 * fd_h)
        g = m_s.grad
        out[name] = {"J_kg_m2": float(J.detach()), "dJ_dkappa": float(k.grad),
                     "dJ_dkappa_fd": fd_k, "dJ_dflux_scale": float(sc.grad),
                     "dJ_dflux_scale_fd": fd_s, "dJ_dj_max": float(sc.grad) / j_max,
                     "fd_rel_err_kappa": abs(float(k.grad) - fd_k) / max(abs(fd_k), 1e-300),
                     "fd_rel_err_flux_scale": abs(float(sc.grad) - fd_s) / max(abs(fd_s), 1e-300),
                     "dJ_dms_max_abs": float(g.abs().max()), "dJ_dms_mean": float(g.mean()),
                     "forward_s": t1 - t0, "backward_s": t2 - t1}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["golovin", "golovin-ensemble", "precision",
                                     "precision-ensemble", "box-ecol", "adjoint"])
    ap.add_argument("--kernel", default="Long_Bott")
    ap.add_argument("--members", type=int, default=16)
    ap.add_argument("--horizon", type=int, default=3600)
    ap.add_argument("--kappa", type=int, default=1000)
    ap.add_argument("--t-end", type=float, default=3600.0)
    ap.add_argument("--dt-save", type=float, default=600.0)
    ap.add_argument("--seeds", type=int, nargs="+", default=[1001, 1003])
    ap.add_argument("--spcm", type=int, nargs=2, default=[52, 76])
    ap.add_argument("--spinup", type=int, default=7200)
    ap.add_argument("--horizons", type=int, nargs="+", default=[1, 10, 60, 600, 3600])
    a = ap.parse_args()
    if a.what == "golovin":
        r = golovin_box(a.kappa, a.t_end, 1.0, tuple(a.seeds), a.dt_save)
    elif a.what == "golovin-ensemble":
        r = golovin_ensemble(tuple(a.seeds) if len(a.seeds) > 2 else tuple(range(1001, 1041, 2)),
                             a.kappa, a.t_end, 1.0, a.dt_save)
    elif a.what == "box-ecol":
        r = box_ecol_ensemble(a.kernel, kappa=600, t_end=a.t_end)
    elif a.what == "adjoint":
        r = adjoint(tuple(a.spcm))
    elif a.what == "precision-ensemble":
        r = precision_ensemble(a.members, tuple(a.spcm), spinup=a.spinup, horizon=a.horizon)
    else:
        r = precision(tuple(a.spcm), spinup=a.spinup, horizons=tuple(a.horizons))
    print(json.dumps(r))


if __name__ == "__main__":
    main()
