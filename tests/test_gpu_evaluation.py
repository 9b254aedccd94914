"""Size spectra, per-cell moments and box averages of saved simulations
(evaluation.py:1172-1660) against the reference's own results on frames the
reference wrote (tests/golden/evaluation.npz).  Radii come from the GPU's
cube root (within 1e-15 of the reference's pow) and the histogram weights add
up in any order on the GPU: the moments agree to 1e-12 relative, the spectra
to 1e-9 relative or 1e-15 absolute (sparse bins); bins, save times and r_l
are exact."""
import numpy as np
import pytest

from conftest import golden, sub

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
RTOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from lacmopy_gb300 import build
    build.build()


@pytest.fixture()
def frames(tmp_path):
    g = golden("evaluation.npz")
    for key, data in sub(g, "file").items():
        seed, fn = key.split("__", 1)
        (tmp_path / seed).mkdir(exist_ok=True)
        (tmp_path / seed / fn).write_bytes(data.tobytes())
    return g, [str(tmp_path / f"seed{k}") + "/" for k in range(2)]


def test_size_spectra_vs_reference(frames):
    from lacmopy_gb300 import evaluation as E
    g, paths = frames
    inp = sub(g, "in")
    got = E.generate_size_spectra_R(paths, np.array([0, 1]), inp["mass_dry_inv"],
                                    np.array([6, 5]), "AS", inp["target_cells"], 3, 3, 12, 8)
    want = sub(g, "spec")
    for nm, a in zip(("f_R_p", "f_R_s", "bins_R_p", "bins_R_s", "save_times", "r_l", "R_min",
                      "R_max"), got):
        if nm in ("save_times", "r_l"):
            np.testing.assert_array_equal(np.asarray(a), want[nm], err_msg=nm)
        elif nm in ("f_R_p", "f_R_s"):
            # a bin's weights add up in another order on the GPU, and bins
            # holding a few SIPs carry the last-bit differences of their sums
            np.testing.assert_allclose(np.asarray(a), want[nm], rtol=1e-9, atol=1e-15,
                                       err_msg=nm)
        else:
            np.testing.assert_allclose(np.asarray(a), want[nm], rtol=RTOL, atol=0, err_msg=nm)
    assert want["f_R_p"].sum() > 0


def test_moments_and_box_averages_vs_reference(frames):
    from lacmopy_gb300 import evaluation as E
    g, paths = frames
    inp = sub(g, "in")
    mom, t = E.generate_moments_all_seeds(paths, 4, np.array([0, 1]), float(inp["volume_cell"]),
                                          np.array([6, 5]), "AS")
    np.testing.assert_array_equal(t, g["mom__save_times"])
    np.testing.assert_allclose(mom, g["mom__moments"], rtol=RTOL, atol=0)
    box = E.avg_moments_over_boxes(g["mom__moments"], 2, np.array([0, 1]), 4, np.array([1, 4]),
                                   np.array([1, 3]), 3, 3)
    np.testing.assert_array_equal(box, g["box__avg"])


def test_histogram_matches_numpy():
    from lacmopy_gb300 import evaluation as E
    rng = np.random.default_rng(4)
    x = np.exp(rng.normal(0.0, 1.5, 20000))
    w = rng.uniform(0.5, 2.0, x.size)
    bins = np.logspace(-2, 1.5, 31)
    want = np.histogram(x, bins, weights=w)[0]
    np.testing.assert_allclose(E.histogram_weighted(x, bins, w), want, rtol=1e-12)
    # the last edge is inside the last bin, as in numpy
    xe = np.array([bins[0], bins[-1], bins[5], 1e9])
    np.testing.assert_array_equal(E.histogram_weighted(xe, bins), np.histogram(xe, bins)[0])
