"""On-disk state and frame formats of the reference (file_handling.py), and a
frame writer that dumps device-resident states without stalling them.

The files keep the reference's names, array shapes and orders exactly, so a
state or frame written here loads in the reference and the other way round
(the format has to be the same; the code is this package's own):

* full system state (file_handling.py:622-762): ``grid_basics_<t>.txt``
  (x_min x_max z_min z_max dx dz dy t), ``arr_file1_<t>.npy`` (p, T, rho_d,
  r_v, r_l, e_s, S, Theta), ``arr_file2_<t>.npy`` (u, w, dry mass flux x, z),
  ``particle_vectors_<t>.npy`` ([pos, vel]), ``particle_cells_<t>.npy``,
  ``particle_scalars_<t>.npy`` ([m_w, m_s]), ``multiplicity_<t>.npy``,
  ``active_ids_<t>.npy``;
* frames of a simulation (file_handling.py:101-145, 188-233, 292-413,
  466-543): ``grid_scalar_fields_t_<t>.npy`` (r_v, r_l, Theta, T, p, S),
  ``particle_*_data_all_<t>.npy``, tracer dumps and tracer blocks.

``GridData`` carries the grid attributes these functions read and write
(the reference's Grid attribute names) and converts to and from the
``grid_scalar_fields`` / ``grid_mat_prop`` arrays of the step functions.
"""
import os
import queue
import threading

import numpy as np

from . import synthetic

P_REF = 1.0E5   # grid.py:620


class GridData:
    """The atmospheric grid of a saved state (the reference's Grid attributes
    that the state files hold or that follow from them)."""

    def __init__(self, grid_ranges, grid_steps, dy):
        ranges = np.array(grid_ranges, dtype=np.float64)
        self.steps = np.array(grid_steps, dtype=np.float64)
        self.step_y = float(dy)
        # grid.py:563-572: cell counts from the steps, upper ranges on the grid
        self.no_cells = np.array([int(np.ceil((ranges[d, 1] - ranges[d, 0]) / self.steps[d]))
                                  for d in range(2)], dtype=np.int64)
        ranges[:, 1] = ranges[:, 0] + self.steps * self.no_cells
        self.ranges = ranges
        self.sizes = np.array([ranges[0, 1] - ranges[0, 0], ranges[1, 1] - ranges[1, 0]])
        self.volume_cell = self.steps[0] * self.steps[1] * self.step_y
        self.p_ref, self.p_ref_inv = P_REF, 1.0 / P_REF
        shape = tuple(self.no_cells)
        for name in ("pressure", "temperature", "potential_temperature", "mass_density_air_dry",
                     "mixing_ratio_water_vapor", "mixing_ratio_water_liquid",
                     "saturation_pressure", "saturation", "mass_dry_inv", "rho_dry_inv"):
            setattr(self, name, np.zeros(shape))
        self.velocity = np.zeros((2, shape[0] + 1, shape[1] + 1))
        self.mass_flux_air_dry = np.zeros_like(self.velocity)
        for name in synthetic.MAT_PROP_NAMES:
            setattr(self, name, np.zeros(shape))

    def update_material_properties(self):
        """grid.py:713-727."""
        mp = synthetic.material_properties(self.grid_scalar_fields())
        for name, arr in zip(synthetic.MAT_PROP_NAMES, mp):
            setattr(self, name, arr)

    def grid_scalar_fields(self):
        """The [10, Nx, Nz] scalar fields of the step functions
        (integration.py:1966-1975)."""
        return np.array([getattr(self, k) for k in synthetic.GRID_FIELD_NAMES])

    def grid_mat_prop(self):
        """The [7, Nx, Nz] material properties (integration.py:1976-1982)."""
        return np.array([getattr(self, k) for k in synthetic.MAT_PROP_NAMES])

    @classmethod
    def from_state(cls, st, dy=None):
        """A grid from a step-function state dict (the arrays are copied)."""
        steps = np.asarray(st["grid_steps"], dtype=np.float64)
        if dy is None:
            dy = float(st["grid_volume_cell"]) / (steps[0] * steps[1])
        g = cls(np.asarray(st["grid_ranges"]), steps, dy)
        for name, arr in zip(synthetic.GRID_FIELD_NAMES, np.asarray(st["grid_scalar_fields"])):
            setattr(g, name, np.array(arr))
        for name, arr in zip(synthetic.MAT_PROP_NAMES, np.asarray(st["grid_mat_prop"])):
            setattr(g, name, np.array(arr))
        g.velocity = np.array(st["grid_velocity"])
        g.mass_flux_air_dry = np.array(st["grid_mass_flux_air_dry"])
        return g

    def state_arrays(self):
        """The grid entries of a step-function state dict."""
        return dict(grid_scalar_fields=self.grid_scalar_fields(),
                    grid_mat_prop=self.grid_mat_prop(), grid_velocity=self.velocity,
                    grid_mass_flux_air_dry=self.mass_flux_air_dry, p_ref=self.p_ref,
                    p_ref_inv=self.p_ref_inv, grid_no_cells=self.no_cells,
                    grid_ranges=self.ranges, grid_steps=self.steps,
                    grid_volume_cell=self.volume_cell)


def _t(t):
    return str(int(t))


# ---- full system state ---------------------------------------------------------
def save_grid_basics_to_textfile(grid, t, filename):
    """file_handling.py:415-434."""
    with open(filename, "w") as f:
        f.write("# grid.ranges[0] grid.ranges[1] grid.steps grid.step_y t\n")
        f.write(f"{grid.ranges[0][0]} {grid.ranges[0][1]} ")
        f.write(f"{grid.ranges[1][0]} {grid.ranges[1][1]} ")
        f.write(f"{grid.steps[0]} {grid.steps[1]} {grid.step_y} {t}")


def save_grid_arrays_to_npy_file(grid, filename1, filename2):
    """file_handling.py:436-464."""
    np.save(filename1, np.array([grid.pressure, grid.temperature, grid.mass_density_air_dry,
                                 grid.mixing_ratio_water_vapor, grid.mixing_ratio_water_liquid,
                                 grid.saturation_pressure, grid.saturation,
                                 grid.potential_temperature]))
    np.save(filename2, np.array([grid.velocity[0], grid.velocity[1], grid.mass_flux_air_dry[0],
                                 grid.mass_flux_air_dry[1]]))


def save_grid_to_files(grid, t, basics_file, arr_file1, arr_file2):
    """file_handling.py:545-570."""
    save_grid_basics_to_textfile(grid, t, basics_file)
    save_grid_arrays_to_npy_file(grid, arr_file1, arr_file2)


def load_grid_from_files(basics_file, arr_file1, arr_file2):
    """file_handling.py:572-620: the grid with its material properties and
    inverse dry masses recomputed from the loaded fields."""
    basics = np.loadtxt(basics_file)
    scalars = np.load(arr_file1)
    vectors = np.load(arr_file2)
    g = GridData([[basics[0], basics[1]], [basics[2], basics[3]]], [basics[4], basics[5]],
                 basics[6])
    (g.pressure, g.temperature, g.mass_density_air_dry, g.mixing_ratio_water_vapor,
     g.mixing_ratio_water_liquid, g.saturation_pressure, g.saturation,
     g.potential_temperature) = (np.array(a) for a in scalars[:8])
    g.update_material_properties()
    g.rho_dry_inv = np.ones_like(g.mass_density_air_dry) / g.mass_density_air_dry
    g.mass_dry_inv = (1.0 / g.volume_cell) * g.rho_dry_inv
    g.velocity = np.array([vectors[0], vectors[1]])
    g.mass_flux_air_dry = np.array([vectors[2], vectors[3]])
    return g


def save_particles_to_files(pos, cells, vel, m_w, m_s, xi, active_ids, vector_filename,
                            scalar_filename, cells_filename, xi_filename, active_ids_filename):
    """file_handling.py:47-99."""
    np.save(vector_filename, [pos, vel])
    np.save(cells_filename, cells)
    np.save(scalar_filename, [m_w, m_s])
    np.save(xi_filename, xi)
    np.save(active_ids_filename, active_ids)


def _full_state_files(t, path):
    grid_files = [path + f"grid_basics_{_t(t)}.txt", path + f"arr_file1_{_t(t)}.npy",
                  path + f"arr_file2_{_t(t)}.npy"]
    particle_files = dict(vector=path + f"particle_vectors_{_t(t)}.npy",
                          scalar=path + f"particle_scalars_{_t(t)}.npy",
                          cells=path + f"particle_cells_{_t(t)}.npy",
                          xi=path + f"multiplicity_{_t(t)}.npy",
                          active=path + f"active_ids_{_t(t)}.npy")
    return grid_files, particle_files


def liquid_mixing_ratio(m_w, xi, cells, active_ids, mass_dry_inv):
    """r_l of every cell from the active SIPs, summed in ascending SIP ID as
    file_handling.py:678-682 and grid.py:370-412 do, times 1e-18 / m_dry."""
    r_l = np.zeros(np.shape(mass_dry_inv))
    ids = np.flatnonzero(active_ids)
    # np.add.at accumulates in index order, the reference's loop order
    np.add.at(r_l, (cells[0, ids], cells[1, ids]), m_w[ids] * xi[ids])
    return r_l * (1.0E-18 * mass_dry_inv)


def save_grid_and_particles_full(t, grid, pos, cells, vel, m_w, m_s, xi, active_ids, path):
    """file_handling.py:622-691: r_l recomputed from the particles, then the
    grid and particle files of time t."""
    grid.mixing_ratio_water_liquid = liquid_mixing_ratio(np.asarray(m_w), np.asarray(xi),
                                                         np.asarray(cells),
                                                         np.asarray(active_ids),
                                                         grid.mass_dry_inv)
    gf, pf = _full_state_files(t, path)
    save_grid_to_files(grid, t, *gf)
    save_particles_to_files(pos, cells, vel, m_w, m_s, xi, active_ids, pf["vector"], pf["scalar"],
                            pf["cells"], pf["xi"], pf["active"])


def load_grid_and_particles_full(t, path):
    """file_handling.py:693-762: (grid, pos, cells, vel, m_w, m_s, xi,
    active_ids)."""
    gf, pf = _full_state_files(t, path)
    grid = load_grid_from_files(*gf)
    vectors = np.load(pf["vector"])
    scalars = np.load(pf["scalar"])
    return (grid, vectors[0], np.load(pf["cells"]), vectors[1], scalars[0], scalars[1],
            np.load(pf["xi"]), np.load(pf["active"]))


def save_sim_paras_to_file(sim_paras, sim_par_names, t, path):
    """file_handling.py:20-45: the names line, then every value (list and
    array items one by one), each followed by a space."""
    with open(path + f"sim_paras_t_{_t(t)}.txt", "w") as f:
        f.write(sim_par_names + "\n")
        for item in sim_paras:
            items = item if type(item) is list or type(item) is np.ndarray else [item]
            for el in items:
                f.write(f"{el} ")


# ---- frames -------------------------------------------------------------------------
def save_grid_scalar_fields(t, grid_scalar_fields, path, start_time=None):
    """file_handling.py:466-511: r_v, r_l, Theta, T, p, S of time t."""
    gsf = grid_scalar_fields
    np.save(path + f"grid_scalar_fields_t_{_t(t)}.npy",
            (gsf[4], gsf[5], gsf[2], gsf[0], gsf[1], gsf[6]))


def load_grid_scalar_fields(path, save_times):
    """file_handling.py:513-543."""
    return np.array([np.load(path + f"grid_scalar_fields_t_{_t(t)}.npy") for t in save_times])


def dump_particle_data_all(t, pos, vel, cells, m_w, m_s, xi, active_ids, path):
    """file_handling.py:292-343."""
    np.save(path + f"particle_vector_data_all_{_t(t)}.npy", (pos, vel))
    np.save(path + f"particle_cells_data_all_{_t(t)}.npy", cells)
    np.save(path + f"particle_scalar_data_all_{_t(t)}.npy", (m_w, m_s))
    np.save(path + f"particle_xi_data_all_{_t(t)}.npy", xi)
    np.save(path + f"particle_active_ids_data_all_{_t(t)}.npy", active_ids)


def load_particle_data_all(path, save_times):
    """file_handling.py:345-413: (vec, cells, scal, xi, active_ids) over the
    save times."""
    names = ("particle_vector_data_all_", "particle_cells_data_all_",
             "particle_scalar_data_all_", "particle_xi_data_all_",
             "particle_active_ids_data_all_")
    return tuple(np.array([np.load(path + f"{nm}{_t(t)}.npy") for t in save_times])
                 for nm in names)


def dump_particle_data(t, pos, vel, m_w, m_s, xi, T_grid, rv_grid, path):
    """file_handling.py:101-144 (tracer particles and the T, r_v grids)."""
    np.save(path + f"particle_vector_data_{_t(t)}.npy", (pos, vel))
    np.save(path + f"particle_scalar_data_{_t(t)}.npy", (m_w, m_s))
    np.save(path + f"particle_xi_data_{_t(t)}.npy", xi)
    np.save(path + f"grid_T_rv_{_t(t)}.npy", (T_grid, rv_grid))


def load_particle_data(path, save_times):
    """file_handling.py:146-186: (vec, scal, xi, grid T/r_v)."""
    names = ("particle_vector_data_", "particle_scalar_data_", "particle_xi_data_",
             "grid_T_rv_")
    return tuple(np.array([np.load(path + f"{nm}{_t(t)}.npy") for t in save_times])
                 for nm in names)


def dump_particle_tracer_data_block(time_block, traced_vectors, traced_scalars, traced_xi,
                                    traced_water, path):
    """file_handling.py:188-232."""
    t = _t(time_block[0])
    np.save(path + f"particle_vector_data_{t}.npy", traced_vectors)
    np.save(path + f"particle_scalar_data_{t}.npy", traced_scalars)
    np.save(path + f"particle_xi_data_{t}.npy", traced_xi)
    np.save(path + f"water_removed_{t}.npy", traced_water)
    np.save(path + f"particle_time_block_{t}.npy", time_block)


def load_particle_data_from_blocks(path, grid_save_times, pt_dumps_per_grid_frame):
    """file_handling.py:234-290: the tracer dumps of the blocks saved at the
    grid save times, dump by dump: (vec, scal, xi)."""
    vec, scal, xi = [], [], []
    for t in grid_save_times:
        v = np.load(path + f"particle_vector_data_{_t(t)}.npy")
        s = np.load(path + f"particle_scalar_data_{_t(t)}.npy")
        x = np.load(path + f"particle_xi_data_{_t(t)}.npy")
        if v.ndim == 4:   # a block of dumps
            for n in range(pt_dumps_per_grid_frame):
                vec.append(v[n]); scal.append(s[n]); xi.append(x[n])
        elif v.ndim == 3:   # a single dump
            vec.append(v); scal.append(s); xi.append(x)
        else:
            raise ValueError(f"unexpected tracer data shape {v.shape}")
    return np.array(vec), np.array(scal), np.array(xi)


# ---- device states ----------------------------------------------------------------
class FrameWriter:
    """Frame dumps of device-resident states that do not stall them.

    ``dump(ds, t)`` brings r_l of the device state up to date
    (grid.py:370-412, on the GPU), snapshots the frame's arrays device to
    device on the state's own stream (so steps queued after ``dump`` cannot
    change them), copies the snapshot to pinned host buffers on a side
    stream and returns: the state's own stream keeps running its next steps.
    A writer thread waits for each copy and writes the frame's files in the
    reference's format (``save_grid_scalar_fields``,
    ``dump_particle_data_all`` and ``no_cols_<t>.npy``, as integration.py:
    2055-2066 writes them).  ``close()`` waits for every frame to be on disk.
    """

    def __init__(self, path, depth=2):
        import torch
        self.torch = torch
        self.path = path
        os.makedirs(path, exist_ok=True)
        self.stream = torch.cuda.Stream()
        self.depth = depth        # buffer sets per state size
        self.pools = {}           # state size -> queue of free buffer sets
        self.made = {}
        self.jobs = queue.Queue()
        self.error = None
        self.thread = threading.Thread(target=self._run, daemon=True)
        self.thread.start()

    def _buffers(self, ds):
        key = (ds.n, ds.nx, ds.nz)
        pool = self.pools.setdefault(key, queue.Queue())
        try:
            return key, pool.get_nowait()
        except queue.Empty:
            while self.made.get(key, 0) >= self.depth:
                # every set in flight: wait for the writer to free one
                try:
                    return key, pool.get(timeout=1.0)
                except queue.Empty:
                    if not self.thread.is_alive():
                        raise RuntimeError("frame writer thread stopped") from self.error
        self.made[key] = self.made.get(key, 0) + 1
        t = self.torch
        n, nx, nz = key
        shapes = {"gsf": ((10, nx, nz), t.float64), "pos": ((2, n), t.float64),
                  "vel": ((2, n), t.float64), "cells": ((2, n), t.int64),
                  "act": ((n,), t.uint8), "m_w": ((n,), t.float64), "m_s": ((n,), t.float64),
                  "xi": ((n,), t.float64), "no_cols": ((2,), t.int64)}
        # a pinned host set and a device snapshot set per buffer set
        host = {k: t.empty(sh, dtype=dt, pin_memory=True) for k, (sh, dt) in shapes.items()}
        dev = {k: t.empty(sh, dtype=dt, device=ds.pos.device) for k, (sh, dt) in shapes.items()}
        return key, (host, dev)

    def dump(self, ds, t):
        if self.error is not None:
            raise self.error
        torch = self.torch
        ds.update_grid_r_l()
        cells, act = ds.cells_and_active()
        key, (buf, snap) = self._buffers(ds)
        cur = torch.cuda.current_stream()
        for name, src in (("gsf", ds.gsf), ("pos", ds.pos), ("vel", ds.vel), ("cells", cells),
                          ("act", act), ("m_w", ds.m_w), ("m_s", ds.m_s), ("xi", ds.xi),
                          ("no_cols", ds.no_cols)):
            snap[name].copy_(src)   # device to device, on the state's stream
        taken = torch.cuda.Event()
        taken.record(cur)
        self.stream.wait_event(taken)
        with torch.cuda.stream(self.stream):
            for name in buf:
                buf[name].copy_(snap[name], non_blocking=True)
            done = torch.cuda.Event()
            done.record(self.stream)
        self.jobs.put((t, key, (buf, snap), done))

    def _run(self):
        while True:
            job = self.jobs.get()
            if job is None:
                return
            t, key, bufs, done = job
            buf = bufs[0]
            try:
                done.synchronize()
                p = self.path
                save_grid_scalar_fields(t, buf["gsf"].numpy(), p)
                dump_particle_data_all(t, buf["pos"].numpy(), buf["vel"].numpy(),
                                       buf["cells"].numpy(), buf["m_w"].numpy(),
                                       buf["m_s"].numpy(), buf["xi"].numpy(),
                                       buf["act"].numpy().astype(bool), p)
                np.save(p + f"no_cols_{_t(t)}.npy", buf["no_cols"].numpy())
            except BaseException as e:   # reported by the next dump() or close()
                self.error = e
            finally:
                self.pools[key].put(bufs)   # the buffer set is free again either way

    def close(self):
        self.jobs.put(None)
        self.thread.join()
        if self.error is not None:
            raise self.error
