"""Autotuner of the hot kernels' launch shapes.

The library compiles each hot kernel for a few register budgets (resident
blocks per SM) and sizes the cell-ordering grid by a blocks-per-SM factor;
process-wide knobs (``lacmo_tune_set``) choose among them at launch time, and
a CUDA graph keeps the shapes it was captured with.  The fastest choice moves
with the workload (SIPs per cell, precision, draw mode), so this module times
the options on the ensemble itself:

* ``tune_batch(states, seeds, ...)`` builds a throw-away batch from the member
  states, times every option of every knob (coordinate descent in the order
  particle kernel, collision kernel, cell ordering; each option timed in two
  interleaved rounds, the best time counts), sets the winners and stores them
  in a JSON cache keyed by the device and the workload;
* a later call with the same key takes the cached choice without timing;
* ``tune_live(batch)`` does the same on a live batch (a developed, raining
  ensemble: the key includes the largest water mass).

The results of a step do not depend on the knobs (bit for bit in FP64), only
its speed.  The reference runs one simulation per CPU process
(run_lacmo.sh) and has nothing to tune.
"""
import ctypes
import json
import math
import os

import numpy as np

from . import _lib

KNOBS = {"particle_blocks_per_sm": _lib.TUNE_PARTICLE_BLOCKS,
         "collision_blocks_per_sm": _lib.TUNE_COLLISION_BLOCKS,
         "order_blocks_per_sm": _lib.TUNE_ORDER_CTAS}


def default_cache_path():
    return os.environ.get("LACMO_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "lacmopy_gb300",
                                       "launch_shapes.json"))


def options(knob):
    lib = _lib.load()
    vals = (ctypes.c_int * 8)()
    n = lib.lacmo_tune_options(KNOBS[knob], vals, 8)
    if n < 0:
        raise _lib.LacmoError(f"unknown knob {knob}")
    return [int(vals[i]) for i in range(n)]


def current():
    lib = _lib.load()
    return {k: int(lib.lacmo_tune_get(v)) for k, v in KNOBS.items()}


def apply(choice):
    """Set the knobs of ``choice`` ({knob name: value}); others keep theirs."""
    lib = _lib.load()
    for k, v in choice.items():
        _lib.check(lib.lacmo_tune_set(KNOBS[k], int(v)), f"tune_set {k}={v}")


def reset():
    """Every knob back to its default (the first option)."""
    apply({k: options(k)[0] for k in KNOBS})


def _key(device_name, precision, draws, M, nx, nz, n_tot, mean_pc, max_pc, mw_max):
    return "|".join([device_name, precision, str(draws), f"M{M}", f"{nx}x{nz}",
                     f"n2^{int(round(math.log2(max(n_tot, 1))))}",
                     f"mean{16 * int(round(mean_pc / 16))}", f"max{16 * int(round(max_pc / 16))}",
                     f"mw2^{int(round(math.log2(max(mw_max, 1e-30))))}"])


def workload_key(states, precision, draws, device_name):
    """What the best shapes depend on: the device, the arithmetic, the draw
    mode, the member count and grid, the SIPs per cell (total on a log2
    scale, mean and largest cell in steps of 16) and the largest water mass
    (log2; it tells a fresh cloud from a raining one, whose collision work
    per cell is several times larger)."""
    nx, nz = (int(v) for v in states[0]["grid_no_cells"])
    n_tot = sum(int(np.asarray(s["xi"]).size) for s in states)
    per_cell = []
    mw_max = 0.0
    for s in states:
        cells = np.asarray(s["cells"])
        act = np.asarray(s["active_ids"], dtype=bool)
        cnt = np.bincount(cells[0, act] * nz + cells[1, act], minlength=nx * nz)
        per_cell.append((cnt.mean(), cnt.max()))
        if act.any():
            mw_max = max(mw_max, float(np.asarray(s["m_w"])[act].max()))
    mean_pc = float(np.mean([p[0] for p in per_cell]))
    max_pc = int(max(p[1] for p in per_cell))
    return _key(device_name, precision, draws, len(states), nx, nz, n_tot, mean_pc, max_pc,
                mw_max)


def batch_key(batch, device_name):
    """workload_key of a live BatchState, from its device arrays."""
    import torch
    m0 = batch.members[0]
    nx, nz = m0.nx, m0.nz
    per_cell = []
    mw_max = 0.0
    for m in batch.members:
        act = m.cell >= 0
        cnt = torch.bincount(m.cell[act].long(), minlength=nx * nz).double()
        per_cell.append((float(cnt.mean()), float(cnt.max())))
        if bool(act.any()):
            mw_max = max(mw_max, float(m.m_w[act].max()))
    return _key(device_name, batch.precision, batch.draws, len(batch.members), nx, nz,
                batch.n_total, float(np.mean([p[0] for p in per_cell])),
                int(max(p[1] for p in per_cell)), mw_max)


def load_cache(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(path, cache):
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _descend(batch, steps, rounds):
    """Coordinate descent over the knobs, timing steps of ``batch`` (which
    advances); sets the winners and returns the timings."""
    import torch
    timings = {}
    for knob in KNOBS:
        best = {}
        for _ in range(rounds):
            for v in options(knob):
                apply({knob: v})
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                batch.adv_step(1)   # warm-up with this shape
                a.record()
                batch.adv_step(steps)
                b.record()
                torch.cuda.synchronize()
                ms = a.elapsed_time(b) / steps
                best[v] = min(best.get(v, float("inf")), ms)
        win = min(best, key=best.get)
        apply({knob: win})
        timings[knob] = {str(v): t for v, t in best.items()}
    return timings


def tune_live(batch, steps=2, rounds=2, cache_path=None, force=False):
    """tune_batch on a live BatchState: the timed steps advance it (a
    developed ensemble keeps its regime), the winners are cached under its
    own key."""
    import torch
    path = cache_path or default_cache_path()
    key = batch_key(batch, torch.cuda.get_device_name())
    cache = load_cache(path)
    if not force and key in cache:
        choice = cache[key]["choice"]
        apply(choice)
        return choice
    reset()
    timings = _descend(batch, steps, rounds)
    choice = current()
    cache[key] = {"choice": choice, "ms_per_step": timings}
    save_cache(path, cache)
    return choice


def tune_batch(states, seeds, precision="mixed", draws="thinned", steps=2, rounds=2,
               cache_path=None, force=False):
    """Choose the launch shapes for a batch of these member states (see the
    module docstring), set them and return {knob: value}."""
    import torch
    from .device import BatchState
    path = cache_path or default_cache_path()
    key = workload_key(states, precision, draws, torch.cuda.get_device_name())
    cache = load_cache(path)
    if not force and key in cache:
        choice = cache[key]["choice"]
        apply(choice)
        return choice
    reset()
    batch = BatchState(states, seeds, precision=precision, draws=draws)
    batch.adv_step(1)   # first launches: lazy set-up outside the timings
    torch.cuda.synchronize()
    timings = _descend(batch, steps, rounds)
    del batch
    torch.cuda.empty_cache()
    choice = current()
    cache[key] = {"choice": choice, "ms_per_step": timings}
    save_cache(path, cache)
    return choice
