"""Pin the CPU oracle to the reference: bit-exact against the golden fixtures.

The fixtures were produced by running the reference (LacmoPy) itself with
Numba stubbed out (tests/golden/make_golden.py).  The oracle variant "py"
evaluates x**2 the way CPython does in that run and must agree bit for bit
on every output.  The "numba" variant (x**2 as x*x, the Numba semantics the
GPU follows) must agree bit for bit on collision decisions and counters and to
1e-12 relative elsewhere.
"""
import numpy as np
import pytest

from conftest import golden, sub


def test_mass_rate_and_newton(oracle_py):
    g = golden("mass_rate_newton.npz")
    amb = [g[k] for k in ("T_amb", "p_amb", "S_amb", "e_s_amb", "L_v", "K", "D_v")]
    for sol in ("AS", "NaCl"):
        R, w, rho = oracle_py.R_ws_rho(sol, g["m_w"], g["m_s"], g["T_p"])
        assert np.array_equal(R, g[f"R_{sol}"])
        assert np.array_equal(rho, g[f"rho_{sol}"])
        sig = oracle_py.surface_tension(sol, w, g["T_p"])
        assert np.array_equal(sig, g[f"sig_{sol}"])
        gam, dg = oracle_py.mass_rate_and_derivative(sol, g["m_w"], g["m_s"], w, R, g["T_p"], rho,
                                                      *amb, sig)
        assert np.array_equal(gam, g[f"g_{sol}"])
        assert np.array_equal(dg, g[f"dg_{sol}"])
        dm, g0 = oracle_py.newton_full(sol, g["dt_sub"], g["no_iter"], g["m_w"], g["m_s"], w, R,
                                       g["T_p"], rho, *amb, sig)
        assert np.array_equal(dm, g[f"dm_{sol}"])
        assert np.array_equal(g0, g[f"g0_{sol}"])


def test_interpolation(oracle_py):
    g = golden("interp.npz")
    out = oracle_py.interpolate_velocity(g["cells"], g["rel"], g["gv"])
    assert np.array_equal(out, g["vel"])


@pytest.mark.parametrize("case", ["phys", "boost", "eqxi"])
def test_golovin(oracle_py, case):
    d = sub(golden("collision_golovin.npz"), case)
    xis, m = d["xis_in"].copy(), d["m_in"].copy()
    no_cols = np.zeros(2, dtype=np.int64)
    n = len(xis)
    per = n * (n - 1) // 2
    for s in range(d["xis_out"].shape[0]):
        oracle_py.collision_step_Golovin_np(xis, m, d["dt_over_dV"], no_cols,
                                            np.ascontiguousarray(d["draws"][s * per:(s + 1) * per]))
        assert np.array_equal(xis, d["xis_out"][s])
        assert np.array_equal(m, d["m_out"][s])
        assert np.array_equal(no_cols, d["no_cols_out"][s])


@pytest.mark.parametrize("kt", ["Long_Bott", "Hall_Bott"])
def test_ecol_box(oracle_py, kt):
    from lacmopy_gb300.tables import load_kernel_data_Ecol
    E, rg, _, _, lo, bl, nb = load_kernel_data_Ecol(kt)
    d = sub(golden("collision_ecol_box.npz"), kt)
    x, m, r, v = (d[k].copy() for k in ("xis_in", "m_in", "r_in", "v_in"))
    no_cols = np.zeros(2, dtype=np.int64)
    n = len(x)
    per = n * (n - 1) // 2
    for s in range(2):
        oracle_py.collision_step_Ecol_grid_R_np(x, m, r, v, d["rho"], d["dt_over_dV"], E, nb, lo,
                                                bl, no_cols,
                                                np.ascontiguousarray(d["draws"][s * per:(s + 1) * per]))
        oracle_py.update_velocity_Beard(v, r)
        for k, a in (("xis_out", x), ("m_out", m), ("r_out", r), ("v_out", v)):
            assert np.array_equal(a, d[k][s]), k
        assert np.array_equal(no_cols, d["no_cols_out"][s])


CELL_CASES = ["long", "hall", "hall_nacl", "const", "boost"]


def _cells_case(d):
    from lacmopy_gb300.tables import load_kernel_data_Ecol
    kt = str(d["kernel"])
    if kt == "Hydro_E_const":
        E = float(d["E_const"])
    else:
        E = load_kernel_data_Ecol(kt)[0]
    return E


@pytest.mark.parametrize("case", CELL_CASES)
def test_cells_2d(oracle_py, oracle_nb, case):
    d = sub(golden("collision_cells_2d.npz"), case)
    E = _cells_case(d)
    for orc, exact in ((oracle_py, True), (oracle_nb, False)):
        xi, mw, ms = d["xi_in"].copy(), d["m_w_in"].copy(), d["m_s_in"].copy()
        no_cols = np.zeros(2, dtype=np.int64)
        pos = orc.collision_step_Ecol_grid_R_all_cells_2D_multicomp_np(
            xi, mw, ms, d["vel"], d["T"], d["cells"], d["no_cells"], d["dt_over_dV"], E,
            d["no_kernel_bins"], d["R_kernel_low_log"], d["bin_factor_R_log"], no_cols,
            str(d["solute"]), np.ascontiguousarray(d["draws"]))
        assert pos[0] == len(d["draws"])
        assert np.array_equal(no_cols, d["no_cols_out"])
        if exact:
            assert np.array_equal(xi, d["xi_out"])
            assert np.array_equal(mw, d["m_w_out"])
            assert np.array_equal(ms, d["m_s_out"])
        else:
            np.testing.assert_allclose(xi, d["xi_out"], rtol=1e-12)
            np.testing.assert_allclose(mw, d["m_w_out"], rtol=1e-12)
            np.testing.assert_allclose(ms, d["m_s_out"], rtol=1e-12)


def _bool(a):
    return np.ascontiguousarray(a, dtype=np.bool_)


@pytest.mark.parametrize("sol", ["AS", "NaCl"])
def test_particle_substep(oracle_py, sol):
    d = sub(golden("particle_substep.npz"), sol)
    s = {k[3:]: np.array(v) for k, v in d.items() if k.startswith("in_")}
    s["active_ids"] = _bool(s["active_ids"])
    oracle_py.propagate_particles_subloop_step_np(
        s["grid_scalar_fields"], s["grid_mat_prop"], s["grid_velocity"], s["grid_no_cells"],
        s["grid_ranges"], s["grid_steps"], s["pos"], s["vel"], s["cells"], s["rel_pos"],
        s["m_w"], s["m_s"], s["xi"], s["water_removed"], None, s["active_ids"], s["T_p"], sol,
        s["delta_m_l"], 0.1, 0.05, 3, 9.80665)
    for k in ("pos", "vel", "cells", "rel_pos", "m_w", "water_removed", "active_ids", "T_p",
              "delta_m_l"):
        assert np.array_equal(s[k], d["out_" + k]), k


def test_grid_divergence_relaxation(oracle_py):
    g = golden("grid_divergence.npz")
    gsf, gmp = g["gsf_in"].copy(), g["gmp_in"].copy()
    oracle_py.propagate_grid_subloop_step_np(gsf, gmp, g["p_ref"], 1.0 / g["p_ref"], g["dTheta"],
                                             g["dr_v"], g["dml"], g["V"])
    assert np.array_equal(gsf, g["gsf_out"])
    assert np.array_equal(gmp, g["gmp_out"])
    f = g["gsf_in"]
    assert np.array_equal(oracle_py.compute_divergence_upwind_np(f[4], g["flux"], g["no_cells"],
                                                                 g["steps"]), g["div_rv"])
    assert np.array_equal(oracle_py.compute_divergence_upwind_np(f[2], g["flux"], g["no_cells"],
                                                                 g["steps"]), g["div_th"])
    assert np.array_equal(oracle_py.compute_divergence_upwind_np(g["rough"], g["flux2"],
                                                                 g["no_cells"], g["steps"]),
                          g["div_rough"])
    assert np.array_equal(oracle_py.compute_relaxation_term(f[4], g["profile"], g["t_relax"], 0.1),
                          g["relax"])


@pytest.mark.parametrize("case", ["col2", "col1", "col10"])
def test_adv_step(oracle_py, case):
    from lacmopy_gb300.tables import load_kernel_data_Ecol
    d = sub(golden("adv_step.npz"), case)
    E, _, _, _, lo, bl, nb = load_kernel_data_Ecol(str(d["kernel"]))
    s = {k[3:]: np.array(v) for k, v in d.items() if k.startswith("in_")}
    s["active_ids"] = _bool(s["active_ids"])
    no_cols = np.zeros(2, dtype=np.int64)
    pos = np.zeros(1, dtype=np.int64)
    draws = np.ascontiguousarray(d["draws"])
    p_ref = float(d["p_ref"])
    for _ in range(int(d["nsteps"])):
        oracle_py.integrate_adv_step_np(
            s["grid_scalar_fields"], s["grid_mat_prop"], s["grid_velocity"],
            s["grid_mass_flux_air_dry"], p_ref, 1.0 / p_ref, s["grid_no_cells"], s["grid_ranges"],
            s["grid_steps"], float(d["V"]), s["pos"], s["vel"], s["cells"], s["rel_pos"],
            s["m_w"], s["m_s"], s["xi"], "AS", s["water_removed"], None, s["active_ids"],
            s["T_p"], s["delta_m_l"], 1.0, 0.1, 0.05, float(d["dt_col_over_dV"]), 5,
            int(d["no_col_per_adv"]), True, True, s["init_profile_r_v"], s["init_profile_Theta"],
            s["relaxation_time_profile"], 3, 9.80665, E, nb, lo, bl, no_cols, draws, pos)
    assert pos[0] == len(draws)
    assert np.array_equal(no_cols, d["no_cols"])
    for k in ("grid_scalar_fields", "grid_mat_prop", "pos", "vel", "cells", "rel_pos", "m_w",
              "m_s", "xi", "water_removed", "active_ids", "T_p", "delta_m_l"):
        assert np.array_equal(s[k], d["out_" + k]), k


def test_tables_regenerate_bit_exactly():
    import hashlib
    from lacmopy_gb300.tables import load_kernel_data_Ecol
    g = golden("tables.npz")
    for kt in ("Long_Bott", "Hall_Bott"):
        E, rg = load_kernel_data_Ecol(kt)[:2]
        assert hashlib.sha256(np.ascontiguousarray(E).tobytes()).hexdigest() == str(g[kt + "__E_sha256"])
        assert hashlib.sha256(np.ascontiguousarray(rg).tobytes()).hexdigest() == str(g[kt + "__r_sha256"])


def test_diagnostics(oracle_py, oracle_nb):
    """evaluation.py mixing ratios, number concentrations (masks with removed
    SIPs, whose cells[1] = -1 index the top row) and radius moments 0..3."""
    g = golden("diagnostics.npz")
    no_cells = g["no_cells"]
    for name in ("active", "large", "with_removed"):
        mask = g["mask_" + name]
        mr = oracle_py.update_cell_sum(0, g["m_w"], g["xi"], g["cells"], no_cells,
                                       g["mass_dry_inv"], mask)
        nc = oracle_py.update_cell_sum(1, g["m_w"], g["xi"], g["cells"], no_cells,
                                       g["mass_dry_inv"], mask)
        assert np.array_equal(mr, g["mixing_ratio_" + name]), name
        assert np.array_equal(nc, g["number_conc_" + name]), name
    for n in range(4):
        m = oracle_py.compute_moment_R_grid(n, g["R_p"], g["xi"], g["V0"], g["cells"],
                                            g["active_ids"], no_cells)
        assert np.array_equal(m, g[f"moment_{n}"]), n
        # Numba's integer power (repeated squaring) agrees to rounding
        m_nb = oracle_nb.compute_moment_R_grid(n, g["R_p"], g["xi"], g["V0"], g["cells"],
                                               g["active_ids"], no_cells)
        np.testing.assert_allclose(m_nb, g[f"moment_{n}"], rtol=1e-14, atol=0)


def test_kernel_grid_m(oracle_py):
    """collision/all_or_nothing.py:392-491, three steps with the reference's
    draws (ordinary, equal-multiplicity and multiple collections)."""
    g = golden("collision_kernel_grid_m.npz")
    xis, m = g["xis0"].copy(), g["m0"].copy()
    no_cols = np.zeros(2, dtype=np.int64)
    for step in range(3):
        oracle_py.collision_step_kernel_grid_m_np(xis, m, g[f"dtdv_{step}"], g["K"], g["nb"],
                                                  g["m_low_log"], g["bf_log"], no_cols,
                                                  g[f"draws_{step}"])
        assert np.array_equal(no_cols, g[f"no_cols_{step}"]), step
        assert np.array_equal(xis, g[f"xis_{step}"]), step
        assert np.array_equal(m, g[f"m_{step}"]), step


def test_box_model_kernel_grid_m_loop(oracle_py):
    """collision/box_model.py:44-205 with kernel_method='kernel_grid_m': the
    oracle's step in the loop, with NumPy's generator seeded as the reference
    seeds it, reproduces the reference's saved snapshots."""
    import math
    g = golden("box_model_kgrid.npz")
    xis, m = g["xis0"].copy(), g["m0"].copy()
    no_cols = np.zeros(2, dtype=np.int64)
    rs = np.random.RandomState(int(g["seed"]))
    n = xis.size
    dt, t_end, dt_save = float(g["dt"]), float(g["t_end"]), float(g["dt_save"])
    dtdv = dt / float(g["dV"])
    no_steps, dn = int(math.ceil(t_end / dt)), int(math.ceil(dt_save / dt))
    snaps = []
    for step in range(no_steps):
        if step % dn == 0:
            snaps.append(xis.copy())
        oracle_py.collision_step_kernel_grid_m_np(xis, m, dtdv, g["K"], g["nb"], g["m_low_log"],
                                                  g["bf_log"], no_cols, rs.rand(n * (n - 1) // 2))
    snaps.append(xis.copy())
    assert np.array_equal(np.array(snaps), g["xis_vs_time"])
    assert np.array_equal(no_cols, g["no_cols"])
    assert np.array_equal(m, g["m"])


def test_golovin_moments_restatement_vs_reference():
    """reports.compute_moments_Golovin equals the reference's
    golovin.compute_moments_Golovin (golovin.py:48-58) on the box setup."""
    from lacmopy_gb300 import reports
    d = golden("golovin_moments.npz")
    for n in range(4):
        for k, t in enumerate(d["t"]):
            assert reports.compute_moments_Golovin(t, n, float(d["DNC"]), float(d["LWC"]),
                                                   float(d["b"])) == d["moments"][n, k]
