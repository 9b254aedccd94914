"""The collision entry point that allocates nothing, against the regular one.

lacmo_collision_step_cells_noalloc is meant for callers that cannot allocate
device memory when they run a collision step (code inside another
framework's memory pool or under a fixed budget, plugin hosts that forbid
cudaMalloc after start-up): its scratch lives in a fixed array inside the
library.  This test calls it through the C ABI twice in a row (injected
draws, then Philox draws) and checks each result against
lacmo_collision_step_cells with the same inputs, bit for bit, as the other
collision tests do.  The second call also shows that scratch left by the
first call does not leak into the next one.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from lacmopy_gb300 import build
    build.build()


def test_noalloc_collision_matches_workspace_path():
    from lacmopy_gb300 import DeviceState, _lib, synthetic
    from lacmopy_gb300.device import _ptr, _stream, to_device

    lib = _lib.load()
    st = synthetic.make_icmw_state(Nx=60, Nz=60, no_spcm=(26, 38), seed=77,
                                   kernel_type="Hall_Bott", drizzle_fraction=0.1, r_tot=9.0E-3)
    seed = 2024
    # the regular entry point, through DeviceState (workspace from the caller)
    ref = DeviceState(st, draws="philox", seed=seed)
    draws1 = np.random.default_rng(5).random(ref.pair_count())
    ref.collision_step(draws1)         # call 1: injected draws
    ref.collision_step(None)           # call 2: Philox, collision-step counter 1
    want = ref.snapshot()

    # the entry point that allocates nothing; the test owns all buffers
    n = st["xi"].size
    Nx, Nz = int(st["grid_no_cells"][0]), int(st["grid_no_cells"][1])
    xi, mw, ms = to_device(st["xi"]), to_device(st["m_w"]), to_device(st["m_s"])
    vel = to_device(st["vel"])
    T = to_device(st["grid_scalar_fields"][0])
    cells, act = to_device(st["cells"], torch.int64), to_device(st["active_ids"].astype(np.uint8),
                                                                torch.uint8)
    cell = torch.empty(n, dtype=torch.int32, device="cuda")
    _lib.check(lib.lacmo_cells_import(_ptr(cells), _ptr(act), _ptr(cell), n, Nx, Nz, _stream()),
               "cells_import")
    no_cols = torch.zeros(2, dtype=torch.int64, device="cuda")
    prm = ref.params
    d1 = to_device(draws1)
    calls = [(_lib.Draws(d1.data_ptr(), d1.numel(), seed), 0), (_lib.Draws(None, 0, seed), 1)]
    for draws, step in calls:
        rc = lib.lacmo_collision_step_cells_noalloc(
            _ptr(xi), _ptr(mw), _ptr(ms), _ptr(vel), _ptr(T), _ptr(cell), n, Nx, Nz,
            ctypes.byref(prm), ctypes.byref(draws), step, _ptr(no_cols), _stream())
        _lib.check(rc, "collision_step_cells_noalloc")
    torch.cuda.synchronize()
    got_cols = no_cols.cpu().numpy()
    assert got_cols.sum() > 0
    assert np.array_equal(got_cols, want["no_cols"])
    assert np.array_equal(xi.cpu().numpy(), want["xi"])
    assert np.array_equal(mw.cpu().numpy(), want["m_w"])
    assert np.array_equal(ms.cpu().numpy(), want["m_s"])


def test_noalloc_rejects_sizes_above_capacity():
    from lacmopy_gb300 import _lib
    lib = _lib.load()
    x = ctypes.c_void_p(256)
    prm = _lib.Params()
    prm.no_iter_impl_mass = 3
    d = _lib.Draws(None, 0, 1)
    too_many = 524288 + 1
    rc = lib.lacmo_collision_step_cells_noalloc(x, x, x, x, x, x, too_many, 10, 10,
                                                ctypes.byref(prm), ctypes.byref(d), 0, x, None)
    assert rc == -5
    rc = lib.lacmo_collision_step_cells_noalloc(x, x, x, x, x, x, 100, 200, 200,
                                                ctypes.byref(prm), ctypes.byref(d), 0, x, None)
    assert rc == -5
