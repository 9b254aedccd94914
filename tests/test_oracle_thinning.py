"""The thinned Philox draws (lacmopy_gb300/csrc/lacmo_thin.h, restated in the
oracle) sample the same all-or-nothing process as one uniform per pair: over
independent seeds the collision counts, the number of multiple collections,
the conserved water mass and the multiplicity sum agree within sampling error
(oracle, CPU); the oracle's own probability tables equal the kernels'."""
import numpy as np
import pytest

from conftest import with_rain


@pytest.mark.parametrize("boost,rain", [(20.0, 0), (400.0, 0), (1.0, 1), (1.0, 3)])
def test_thinned_and_per_pair_draws_agree_in_distribution(oracle_nb, boost, rain):
    from lacmopy_gb300 import synthetic
    st = synthetic.make_icmw_state(Nx=24, Nz=24, seed=13, kernel_type="Hall_Bott",
                                   drizzle_fraction=0.1, r_tot=12.5E-3)
    if rain:
        st = with_rain(st, rain)
    out = {}
    for thin in (False, True):
        rows = []
        for seed in range(40):
            xi, mw, ms = st["xi"].copy(), st["m_w"].copy(), st["m_s"].copy()
            nc = np.zeros(2, np.int64)
            cs = np.zeros(1, np.int64)
            oracle_nb.collision_step_all_cells_philox(
                xi, mw, ms, st["vel"], st["grid_scalar_fields"][0], st["cells"],
                st["grid_no_cells"], st["dt_col_over_dV"] * boost, st["E_col_grid"],
                st["no_kernel_bins"], st["R_kernel_low_log"], st["bin_factor_R_log"], nc, "AS",
                1000 + seed, cs, thin=thin)
            rows.append((nc[0], nc[1], xi.sum(), (xi * mw).sum()))
        out[thin] = np.array(rows, dtype=float)
    a, b = out[False], out[True]
    assert a[:, 0].mean() > 100
    for col in (0, 1, 2):
        se = np.sqrt(a[:, col].var() / len(a) + b[:, col].var() / len(b))
        d = abs(a[:, col].mean() - b[:, col].mean())
        assert d <= 4.5 * se + 1e-9 * abs(a[:, col].mean()), (col, d, se)
    # collisions move water between SIPs but conserve it
    np.testing.assert_allclose(b[:, 3], a[0, 3], rtol=1e-12)


def test_integer_thresholds_take_the_same_decisions():
    """The kernels compare 53-bit integers u53 < ceil(2^53 X) where the oracle
    compares u = u53 2^-53 < X: the two agree for every u53."""
    import re
    from fractions import Fraction
    from lacmopy_gb300.csrc_gen import thin_tables, threshold53
    H, P = thin_tables()
    txt = open(__import__("os").path.join(__import__("os").path.dirname(__file__), "..",
                                          "lacmopy_gb300", "csrc", "lacmo_thin_tables.h")).read()
    ht = [int(v) for v in re.findall(r"(\d+)ull", txt)]
    flat = [x for row in H for x in row] + [x for row in P for x in row]
    assert ht == [threshold53(x) for x in flat]
    for x in flat:
        t = threshold53(x)
        assert Fraction(t - 1, 2 ** 53) < Fraction(x) <= Fraction(t, 2 ** 53)


def test_rate_tables_are_probabilities():
    """H[e][m] = 1 - (1 - q)^m grows with m and falls with e; P[e][r] =
    q / H[e][r] is a probability, 1 for the last pair."""
    from lacmopy_gb300.csrc_gen import thin_tables
    H, P = thin_tables()
    H, P = np.array(H), np.array(P)
    assert np.all(np.diff(H, axis=1) > 0) and np.all(np.diff(H, axis=0) < 0)
    assert np.all((P > 0) & (P <= 1)) and np.all(P[:, 0] == 1.0)


def test_oracle_tables_equal_the_kernel_tables(oracle_nb):
    """The oracle computes its probability tables and thresholds itself (big
    integers, rounded once); they equal the kernels' generated header."""
    import ctypes
    import re
    H, P = (np.zeros((126, 32)) for _ in range(2))
    HT, PT = (np.zeros((126, 32), dtype=np.uint64) for _ in range(2))
    lib = oracle_nb.lib
    lib.orc_thin_tables.argtypes = [ctypes.c_void_p] * 4
    lib.orc_thin_tables(H.ctypes.data, P.ctypes.data, HT.ctypes.data, PT.ctypes.data)
    from lacmopy_gb300.csrc_gen import thin_tables
    Hk, Pk = thin_tables()
    assert np.array_equal(H, np.array(Hk)) and np.array_equal(P, np.array(Pk))
    txt = open(__import__("os").path.join(__import__("os").path.dirname(__file__), "..",
                                          "lacmopy_gb300", "csrc", "lacmo_thin_tables.h")).read()
    ht = np.array([int(v) for v in re.findall(r"(\d+)ull", txt)], dtype=np.uint64)
    assert np.array_equal(np.concatenate([HT.ravel(), PT.ravel()]), ht)
