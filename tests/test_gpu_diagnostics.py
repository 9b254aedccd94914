"""GPU diagnostics (lacmopy_gb300/evaluation.py, csrc/k_diag.cu) and the
kernel-grid-m box step against the oracle and the reference's own outputs
(tests/golden/diagnostics.npz, collision_kernel_grid_m.npz)."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def test_diagnostics_match_golden_and_oracle(oracle_nb):
    from lacmopy_gb300 import evaluation as E
    g = golden("diagnostics.npz")
    N = g["xi"].size
    ids = np.arange(N)
    for name in ("active", "large", "with_removed"):
        mask = g["mask_" + name]
        mr = np.zeros((6, 5))
        E.update_mixing_ratio(mr, g["m_w"], g["xi"], g["cells"], g["mass_dry_inv"], ids, mask)
        nc = np.zeros((6, 5))
        E.update_number_concentration_per_dry_mass(nc, g["xi"], g["cells"], g["mass_dry_inv"],
                                                   ids, mask)
        if name == "with_removed":   # removed SIPs follow the top-row cell's own SIPs
            np.testing.assert_allclose(mr, g["mixing_ratio_" + name], rtol=1e-14, atol=0)
            np.testing.assert_allclose(nc, g["number_conc_" + name], rtol=1e-14, atol=0)
        else:
            assert np.array_equal(mr, g["mixing_ratio_" + name]), name
            assert np.array_equal(nc, g["number_conc_" + name]), name
    for n in range(4):
        m = E.compute_moment_R_grid(n, g["R_p"], g["xi"], g["V0"], g["cells"], g["active_ids"],
                                    ids, g["no_cells"])
        ref = oracle_nb.compute_moment_R_grid(n, g["R_p"], g["xi"], g["V0"], g["cells"],
                                              g["active_ids"], g["no_cells"])
        assert np.array_equal(m, ref), n   # Numba's integer power, bit for bit
        np.testing.assert_allclose(m, g[f"moment_{n}"], rtol=1e-14, atol=0)


def test_diagnostics_full_grid_vs_oracle(oracle_nb):
    """75 x 75 cells x 64 SIPs: bit for bit against the oracle."""
    from lacmopy_gb300 import evaluation as E, synthetic
    st = synthetic.make_icmw_state(Nx=75, Nz=75, seed=5, kernel_type="Long_Bott")
    N = st["xi"].size
    rng = np.random.default_rng(2)
    R_p = 10.0 ** rng.uniform(-2, 2, N)
    mdi = rng.uniform(1e-4, 2e-4, (75, 75))
    mask = rng.random(N) < 0.7
    mr = np.zeros((75, 75))
    E.update_mixing_ratio(mr, st["m_w"], st["xi"], st["cells"], mdi, np.arange(N), mask)
    ref = oracle_nb.update_cell_sum(0, st["m_w"], st["xi"], st["cells"], (75, 75), mdi, mask)
    assert np.array_equal(mr, ref)
    m3 = E.compute_moment_R_grid(3, R_p, st["xi"], 8000.0, st["cells"], st["active_ids"],
                                 np.arange(N), (75, 75))
    ref3 = oracle_nb.compute_moment_R_grid(3, R_p, st["xi"], 8000.0, st["cells"],
                                           st["active_ids"], (75, 75))
    assert np.array_equal(m3, ref3)


def test_kernel_grid_m_box_vs_golden():
    """Box model with a tabulated K(m1, m2) (collision/all_or_nothing.py:
    392-491): the reference's outputs with its own draws, bit for bit."""
    from lacmopy_gb300 import collision as Cg
    g = golden("collision_kernel_grid_m.npz")
    xis, m = g["xis0"].copy(), g["m0"].copy()
    no_cols = np.zeros(2, dtype=np.int64)
    for step in range(3):
        Cg.collision_step_kernel_grid_m_np(xis, m, g[f"dtdv_{step}"], g["K"], g["nb"],
                                           g["m_low_log"], g["bf_log"], no_cols,
                                           draws=g[f"draws_{step}"])
        assert np.array_equal(no_cols, g[f"no_cols_{step}"]), step
        assert np.array_equal(xis, g[f"xis_{step}"]), step
        assert np.array_equal(m, g[f"m_{step}"]), step


def test_simulate_collisions_kernel_grid_m_vs_golden(tmp_path):
    """The box-model time loop with kernel_method='kernel_grid_m'
    (collision/box_model.py:44-205): saved snapshots, save times, counters and
    the final state against the reference's run with the same seed (draws from
    NumPy's generator seeded like the reference), bit for bit."""
    from lacmopy_gb300 import collision as Cg
    g = golden("box_model_kgrid.npz")
    xis, m = g["xis0"].copy(), g["m0"].copy()
    no_cols = np.zeros(2, dtype=np.int64)
    seed = int(g["seed"])
    xt, mt, tt = Cg.simulate_collisions(
        (xis, m), (g["K"], int(g["nb"]), float(g["m_low_log"]), float(g["bf_log"])), "Long_Bott",
        "kernel_grid_m", float(g["dV"]), float(g["dt"]), float(g["t_end"]), float(g["dt_save"]),
        no_cols, seed, str(tmp_path) + "/")
    assert np.array_equal(tt, g["save_times"])
    assert np.array_equal(no_cols, g["no_cols"])
    assert np.array_equal(xt, g["xis_vs_time"])
    assert np.array_equal(mt, g["masses_vs_time"])
    assert np.array_equal(xis, g["xis"]) and np.array_equal(m, g["m"])
    assert np.array_equal(np.load(tmp_path / f"xis_vs_time_{seed}.npy"), g["xis_vs_time"])


def test_kernel_grid_m_box_with_generated_table(oracle_py, tmp_path):
    """The box model with a kernel table made by the generator
    (collision/kernel.py:793-867) and its mass-grid binning: the GPU loop
    equals the oracle's step in a loop with the same seeded draws."""
    import math
    from lacmopy_gb300 import collision as Cg
    from lacmopy_gb300 import tables
    K, vel, mass, rg = tables.generate_kernel_grid_Long_Bott_np(0.6, 3000.0, 10, 1000.0)
    nb, m_lo, bf = tables.kernel_grid_m_parameters(1.0E18 * mass)   # kg -> fg
    rng = np.random.default_rng(8)
    n = 300
    xis0 = np.exp(rng.uniform(np.log(1e4), np.log(1e7), n))
    m0 = np.exp(rng.uniform(np.log(1e5), np.log(1e9), n))   # fg: R of 3 to 60 um
    seed, dV, dt, t_end, dt_save = 4242, 1.0, 1.0, 4.0, 2.0
    xis, m = xis0.copy(), m0.copy()
    nc = np.zeros(2, np.int64)
    Cg.simulate_collisions((xis, m), (K, nb, m_lo, bf), "Long_Bott", "kernel_grid_m", dV, dt,
                           t_end, dt_save, nc, seed, str(tmp_path) + "/")
    rs = np.random.RandomState(seed)
    xo, mo = xis0.copy(), m0.copy()
    nco = np.zeros(2, np.int64)
    for _ in range(int(math.ceil(t_end / dt))):
        oracle_py.collision_step_kernel_grid_m_np(xo, mo, dt / dV, K, nb, m_lo, bf, nco,
                                                  rs.rand(n * (n - 1) // 2))
    assert nco.sum() > 0
    assert np.array_equal(nc, nco)
    assert np.array_equal(xis, xo) and np.array_equal(m, mo)
