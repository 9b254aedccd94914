"""Box model against the analytic Golovin solution, and the precision-form
error statement, at sizes that run in seconds (the full-size runs are
`python -m lacmopy_gb300.reports golovin|precision`)."""
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from lacmopy_gb300 import build
    build.build()


def test_golovin_box_moments_vs_analytic():
    """~5000 SIPs, 600 s: number and second moment follow the additive-kernel
    solution within the sampling noise of two realisations; mass is
    conserved to rounding."""
    from lacmopy_gb300 import reports
    r = reports.golovin_box(kappa=1000, t_end=600.0, seeds=(1001, 1003), dt_save=300.0)
    assert r["max_abs_M1_rel"] < 1e-12
    assert abs(r["mean_M0_rel_final"]) < 0.03
    assert abs(r["mean_M2_rel_final"]) < 0.15
    assert all(row["no_cols"] > 0 for row in r["rows"] if row["t"] > 0)


def test_precision_form_small():
    """Mixed vs FP64 from the same spun-up state, 30 x 30 cells at 128
    SIPs/cell: domain liquid water within 1e-5, Theta within 1e-7, r_v within
    1e-6, water masses within 1e-4 for 99% of the SIPs."""
    from lacmopy_gb300 import reports
    r = reports.precision(spcm=(52, 76), nx=30, nz=30, spinup=20, horizons=(20,))["rows"][0]
    assert r["lwp_rel"] < 1e-5
    assert r["theta_rel_max"] < 1e-7
    assert r["r_v_rel_max"] < 1e-6
    assert r["m_w_rel_p99"] < 1e-4
    assert r["cells_differ_frac"] < 1e-3
