"""Initialisation on the GPU (init.py:439-1236) against the reference's own run
of initialize_grid_and_particles_SinSIP on a 3 x 15 column
(tests/golden/init.npz; the upper levels are cloudy, so the saturation
adjustment runs hundreds of Newton iterations there).

Exact: the SIP count, solute masses, cells, positions and mode labels (the
generator takes the reference's own uniforms and its arithmetic).  To
tolerance: multiplicities (CUDA's log/exp in the lognormal weights, 1e-13),
water masses (the equilibrium mass fraction from a device root finder instead
of scipy's fminbound / brentq, then the adjustment's iterations: 1e-6
relative), velocities and grid fields (1e-8 relative)."""
import copy

import numpy as np
import pytest

from conftest import golden, sub

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from lacmopy_gb300 import build
    build.build()


def _config(path, eta_threshold):
    return {
        "paths": {"simdata": path}, "seed_SIP_gen": 1001, "seed_sim": 6001, "reseed": False,
        "solute_type": "AS", "grid_ranges": [[0.0, 60.0], [0.0, 1500.0]],
        "grid_steps": [20.0, 100.0], "dy": 1.0, "no_cells": np.array([3, 15]),
        "p_0": 1015E2, "p_ref": 1E5, "r_tot_0": 7.5E-3, "Theta_l": 289.0,
        "no_spcm": [4, 6], "dist": "lognormal", "DNC0": np.array([60.0E6, 40.0E6]),
        "mu_R": 0.5 * np.array([0.04, 0.15]), "sigma_R": np.array([1.4, 1.6]), "eta": 1E-10,
        "eta_threshold": eta_threshold, "r_critmin": np.array([1., 3.]) * 1E-3,
        "m_high_over_m_low": 1.0E8, "S_init_max": 1.04, "dt_init": 0.1,
        "Newton_iterations": 2, "iter_cnt_limit": 4000}


@pytest.mark.parametrize("tag", ["fix", "weak"])
def test_init_vs_reference(tag, tmp_path):
    from lacmopy_gb300 import file_handling as fh
    from lacmopy_gb300 import init as I
    want = sub(golden("init.npz"), tag)
    cfg = I.set_config_generation(_config(str(tmp_path) + "/", tag))
    np.testing.assert_array_equal(np.array(cfg["dist_par"]), want["dist_par"])
    grid, pos, cells, vel, m_w, m_s, xi, act = I.initialize_grid_and_particles_SinSIP(cfg)
    assert m_s.size == want["m_s"].size
    np.testing.assert_array_equal(m_s, want["m_s"])
    np.testing.assert_array_equal(cells, want["cells"])
    np.testing.assert_array_equal(pos, want["pos"])
    np.testing.assert_array_equal(act, want["active_ids"])
    np.testing.assert_array_equal(np.load(cfg["paths"]["grid"] + "modes_0.npy"), want["modes"])
    np.testing.assert_allclose(xi, want["xi"], rtol=1e-13, atol=0)
    # water masses: the saturation adjustment runs up to thousands of Newton
    # iterations, and a SIP at its activation threshold can take the other
    # branch (its mass then differs by orders of magnitude); such SIPs carry
    # a negligible share of the water
    rel = np.abs(m_w - want["m_w"]) / np.abs(want["m_w"])
    assert np.mean(rel > 1e-6) <= 0.01, np.flatnonzero(rel > 1e-6)
    assert np.mean(rel > 1e-2) <= 0.005
    np.testing.assert_allclose((m_w * xi).sum(), (want["m_w"] * want["xi"]).sum(), rtol=1e-6)
    np.testing.assert_allclose(vel, want["vel"], rtol=1e-8, atol=1e-14)
    for nm in ("pressure", "temperature", "potential_temperature", "mass_density_air_dry",
               "mixing_ratio_water_vapor", "saturation", "saturation_pressure",
               "mass_dry_inv", "velocity", "mass_flux_air_dry"):
        np.testing.assert_allclose(getattr(grid, nm), want["grid_" + nm], rtol=1e-8, atol=1e-14,
                                   err_msg=nm)
    np.testing.assert_allclose(grid.mixing_ratio_water_liquid,
                               want["grid_mixing_ratio_water_liquid"], rtol=1e-6, atol=1e-14)
    # the state files load back to what was returned
    g2, pos2, cells2, vel2, mw2, ms2, xi2, act2 = fh.load_grid_and_particles_full(
        0, cfg["paths"]["grid"])
    np.testing.assert_array_equal(mw2, m_w)
    np.testing.assert_array_equal(g2.temperature, grid.temperature)


def test_init_mass_fraction_root_and_maximum():
    """The equilibrium mass fraction solves S_eq(w_s) = S below the
    activation maximum, and is the maximum above it (a check of the device
    root finder against the Koehler curve evaluated on the host)."""
    from lacmopy_gb300 import _lib
    from lacmopy_gb300 import init as I
    from lacmopy_gb300.device import _ptr, _stream, to_device
    import math
    lib = _lib.load()
    T = 285.0
    m_s = to_device(np.array([1e-3, 1e-2, 0.1, 1.0, 10.0]))
    for S in (0.9, 0.99, 1.0005, 1.05):
        w = torch.empty_like(m_s)
        _lib.check(lib.lacmo_init_mass_fraction(0, 5, _ptr(m_s), S, T, I.VOLUME_TO_RADIUS, 0.78,
                                                I.solubility(T, "AS"), _ptr(w), _stream()), "init")
        w = w.cpu().numpy()
        assert np.all((w > 0) & (w <= 0.78))
