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

    python -m lacmopy_gb300.reports golovin [--kappa K] [--t-end T] [--seeds S ...]
    python -m lacmopy_gb300.reports precision [--spcm A B] [--spinup N] [--horizons N ...]
    python -m lacmopy_gb300.reports adjoint [--spcm A B]

``adjoint``: gradients of the domain-mean liquid water path after 600 s of
condensation sub-steps with respect to per-SIP solute mass and hygroscopicity
(lacmopy_gb300.adjoint), timing, and a finite-difference check.
"""
import argparse
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


def _lwp(s):
    return float((s["m_w"] * s["xi"] * s["active_ids"]).sum())


def precision(spcm=(52, 76), nx=75, nz=75, spinup=60, horizons=(10, 60), seed=1001,
              kernel="Long_Bott"):
    """Spin up in FP64, then advance copies of the spun-up state: FP64 and mixed
    precision with identical Philox draws, and FP64 with other draws (the
    seed-to-seed spread of the stochastic collisions, the noise floor of any
    comparison once collision outcomes differ).  Errors of the mixed run
    relative to the FP64 run at each horizon (steps after the spin-up)."""
    from . import DeviceState, synthetic
    st = synthetic.make_icmw_state(Nx=nx, Nz=nz, no_spcm=tuple(spcm), seed=seed,
                                   kernel_type=kernel)
    d = DeviceState(st, draws="philox", seed=seed, precision="fp64")
    if spinup:
        d.adv_step(spinup, graph=True)
    d.export_to(st)
    del d
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


def adjoint(spcm=(52, 76), nx=75, nz=75, seconds=600, every_steps=60, seed=1001,
            kappa=0.6, fd_h=1e-5):
    """d(domain-mean LWP)/d m_s and d/d kappa through ``seconds`` of
    condensation sub-steps (collisions and motion held fixed), checkpointed
    every ``every_steps`` advection steps; timing and a central finite
    difference of d/d kappa."""
    import torch
    from . import adjoint as adj, synthetic
    st = synthetic.make_icmw_state(Nx=nx, Nz=nz, no_spcm=tuple(spcm), seed=seed,
                                   kernel_type="Long_Bott")
    model = adj.CondensationModel(st)
    n_sub = int(round(seconds / model.dt_sub))
    every = int(round(every_steps * 1.0 / model.dt_sub))
    m_s = model.m_s0.clone().requires_grad_(True)
    k = torch.tensor(kappa, dtype=torch.float64, device="cuda", requires_grad=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J = adj.liquid_water(model, m_s, k, n_sub=n_sub, checkpoint_every=every)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    J.backward()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    w = model.lwp_weights()

    def J_of(kv):
        m_w, _, _ = model.run(model.m_s0, kv, n_sub)
        return float((w * m_w).sum())
    fd = (J_of(kappa + fd_h) - J_of(kappa - fd_h)) / (2 * fd_h)
    g = m_s.grad
    return {"n_sips": model.n, "sub_steps": n_sub, "checkpoint_every_sub_steps": every,
            "lwp": float(J.detach()), "dlwp_dkappa": float(k.grad), "dlwp_dkappa_fd": fd,
            "fd_rel_err": abs(float(k.grad) - fd) / abs(fd),
            "dlwp_dms_max_abs": float(g.abs().max()), "dlwp_dms_mean": float(g.mean()),
            "forward_s": t1 - t0, "backward_s": t2 - t1}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["golovin", "precision", "adjoint"])
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
    elif a.what == "adjoint":
        r = adjoint(tuple(a.spcm))
    else:
        r = precision(tuple(a.spcm), spinup=a.spinup, horizons=tuple(a.horizons))
    print(json.dumps(r))


if __name__ == "__main__":
    main()
