"""File formats of the reference (file_handling.py) against files the reference
itself wrote (tests/golden/file_formats.npz, made by make_golden.py):
the files written here are byte for byte the reference's, and the reference's
files load here to the values the reference's own loader returns."""
import numpy as np

from conftest import golden, sub


def _fixture():
    g = golden("file_formats.npz")
    return g, sub(g, "file"), sub(g, "grid"), sub(g, "in"), sub(g, "loaded")


def _grid(inp, ref_grid):
    from lacmopy_gb300 import file_handling as fh
    grid = fh.GridData(inp["grid_ranges"], inp["grid_steps"], float(inp["dy"]))
    for nm in ("temperature", "pressure", "potential_temperature", "mass_density_air_dry",
               "mixing_ratio_water_vapor", "mixing_ratio_water_liquid", "saturation",
               "saturation_pressure", "mass_dry_inv", "rho_dry_inv"):
        setattr(grid, nm, inp["gsf_" + nm].copy())
    grid.velocity = ref_grid["velocity"].copy()
    grid.mass_flux_air_dry = ref_grid["mass_flux_air_dry"].copy()
    return grid


def _written(tmp_path):
    return {p.name: p.read_bytes() for p in tmp_path.iterdir()}


def test_full_state_files_byte_for_byte(tmp_path):
    from lacmopy_gb300 import file_handling as fh
    g, files, ref_grid, inp, _ = _fixture()
    t = int(g["t"])
    grid = _grid(inp, ref_grid)
    fh.save_grid_and_particles_full(t, grid, inp["pos"], inp["cells"], inp["vel"], inp["m_w"],
                                    inp["m_s"], inp["xi"], inp["active_ids"],
                                    str(tmp_path) + "/")
    got = _written(tmp_path)
    names = [f"grid_basics_{t}.txt", f"arr_file1_{t}.npy", f"arr_file2_{t}.npy",
             f"particle_vectors_{t}.npy", f"particle_cells_{t}.npy",
             f"particle_scalars_{t}.npy", f"multiplicity_{t}.npy", f"active_ids_{t}.npy"]
    assert sorted(got) == sorted(names)
    for nm in names:
        assert got[nm] == files[nm].tobytes(), nm


def test_frame_files_byte_for_byte(tmp_path):
    from lacmopy_gb300 import file_handling as fh
    g, files, ref_grid, inp, _ = _fixture()
    t = int(g["t"])
    p = str(tmp_path) + "/"
    gsf = np.array([inp["gsf_" + nm] for nm in
                    ("temperature", "pressure", "potential_temperature", "mass_density_air_dry",
                     "mixing_ratio_water_vapor", "mixing_ratio_water_liquid", "saturation",
                     "saturation_pressure", "mass_dry_inv", "rho_dry_inv")])
    fh.save_grid_scalar_fields(t, gsf, p)
    fh.dump_particle_data_all(t, inp["pos"], inp["vel"], inp["cells"], inp["m_w"], inp["m_s"],
                              inp["xi"], inp["active_ids"], p)
    tr = inp["trace_ids"]
    fh.dump_particle_data(t, inp["pos"][:, tr], inp["vel"][:, tr], inp["m_w"][tr],
                          inp["m_s"][tr], inp["xi"][tr], gsf[0], gsf[4], p)
    tb = np.array([t + 60, t + 80])
    fh.dump_particle_tracer_data_block(
        tb, np.stack([np.array([inp["pos"][:, tr], inp["vel"][:, tr]])] * 2),
        np.stack([np.array([inp["m_w"][tr], inp["m_s"][tr], inp["T_p"][tr]])] * 2),
        np.stack([inp["xi"][tr]] * 2), np.array([0.5, 0.75]), p)
    fh.save_sim_paras_to_file([1.0, 0.1, 3, 6001], "dt dt_sub no_iter_impl_mass rnd_seed_sim",
                              t, p)
    got = _written(tmp_path)
    assert got
    for nm, data in got.items():
        assert nm in files, nm
        assert data == files[nm].tobytes(), nm


def test_reference_files_load_to_the_reference_values(tmp_path):
    from lacmopy_gb300 import file_handling as fh
    g, files, ref_grid, inp, loaded = _fixture()
    t = int(g["t"])
    for nm, data in files.items():
        (tmp_path / nm).write_bytes(data.tobytes())
    grid, pos, cells, vel, m_w, m_s, xi, act = fh.load_grid_and_particles_full(
        t, str(tmp_path) + "/")
    for nm, want in ref_grid.items():
        np.testing.assert_array_equal(np.asarray(getattr(grid, nm)), want, err_msg=nm)
    for nm, got in zip(("pos", "cells", "vel", "m_w", "m_s", "xi", "active_ids"),
                       (pos, cells, vel, m_w, m_s, xi, act)):
        np.testing.assert_array_equal(got, loaded[nm], err_msg=nm)
    # the frame loaders read the frame files back
    vec, cl, scal, xis, acts = fh.load_particle_data_all(str(tmp_path) + "/", [t])
    np.testing.assert_array_equal(vec[0, 0], inp["pos"])
    np.testing.assert_array_equal(acts[0], inp["active_ids"])
    fields = fh.load_grid_scalar_fields(str(tmp_path) + "/", [t])
    np.testing.assert_array_equal(fields[0, 3], inp["gsf_temperature"])
    v, s, x = fh.load_particle_data_from_blocks(str(tmp_path) + "/", [t + 60], 2)
    assert v.shape[0] == 2 and s.shape[1] == 3


def test_state_dict_round_trip():
    """GridData converts to and from the step functions' grid arrays."""
    from lacmopy_gb300 import file_handling as fh
    from lacmopy_gb300 import synthetic
    st = synthetic.make_icmw_state(Nx=6, Nz=5, no_spcm=(3, 4), seed=3)
    grid = fh.GridData.from_state(st)
    arrs = grid.state_arrays()
    for k in ("grid_scalar_fields", "grid_mat_prop", "grid_velocity", "grid_mass_flux_air_dry",
              "grid_no_cells", "grid_ranges", "grid_steps"):
        np.testing.assert_array_equal(arrs[k], np.asarray(st[k]), err_msg=k)
    assert arrs["grid_volume_cell"] == st["grid_volume_cell"]
