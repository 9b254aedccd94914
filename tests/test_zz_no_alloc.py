"""The collision entry point that allocates nothing, against the regular one.

lacmo_collision_step_cells_noalloc is meant for callers that cannot allocate
device memory when they run a collision step (code inside another
framework's memory pool or under a fixed budget, plugin hosts that forbid
cudaMalloc after start-up): its scratch lives in a fixed array inside the
library.  This test calls it through the C ABI twice in a row (injected
draws, then Philox draws; per-pair and thinned Philox draws) and checks each
result against lacmo_collision_step_cells with the same inputs, bit for bit,
as the other collision tests do.  The second call also shows that scratch
left by the first call does not leak into the next one.  The failure paths
report through lacmo_noalloc_status: a draw buffer one draw short skips the
step and leaves the state unchanged, a cell index beyond the grid and a cell
above 65,535 SIPs are flagged and left out.
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


def _status(lib):
    f, p = ctypes.c_uint32(0), ctypes.c_int64(0)
    from lacmopy_gb300 import _lib
    from lacmopy_gb300.device import _stream
    _lib.check(lib.lacmo_noalloc_status(ctypes.byref(f), ctypes.byref(p), _stream()),
               "noalloc_status")
    return int(f.value), int(p.value)


def _device_inputs(st):
    from lacmopy_gb300 import _lib
    from lacmopy_gb300.device import _ptr, _stream, to_device
    lib = _lib.load()
    n = st["xi"].size
    Nx, Nz = int(st["grid_no_cells"][0]), int(st["grid_no_cells"][1])
    d = {"xi": to_device(st["xi"]), "m_w": to_device(st["m_w"]), "m_s": to_device(st["m_s"]),
         "vel": to_device(st["vel"]), "T": to_device(st["grid_scalar_fields"][0]),
         "no_cols": torch.zeros(2, dtype=torch.int64, device="cuda"),
         "cell": torch.empty(n, dtype=torch.int32, device="cuda")}
    cells = to_device(st["cells"], torch.int64)
    act = to_device(st["active_ids"].astype(np.uint8), torch.uint8)
    _lib.check(lib.lacmo_cells_import(_ptr(cells), _ptr(act), _ptr(d["cell"]), n, Nx, Nz,
                                      _stream()), "cells_import")
    return d, n, Nx, Nz


def _call(lib, d, n, Nx, Nz, prm, draws, step):
    from lacmopy_gb300.device import _ptr, _stream
    return lib.lacmo_collision_step_cells_noalloc(
        _ptr(d["xi"]), _ptr(d["m_w"]), _ptr(d["m_s"]), _ptr(d["vel"]), _ptr(d["T"]),
        _ptr(d["cell"]), n, Nx, Nz, ctypes.byref(prm), ctypes.byref(draws), step,
        _ptr(d["no_cols"]), _stream())


@pytest.mark.parametrize("thin", [False, True])
def test_noalloc_collision_matches_workspace_path(thin):
    from lacmopy_gb300 import DeviceState, _lib, synthetic
    from lacmopy_gb300.device import _ptr, _stream, to_device

    lib = _lib.load()
    st = synthetic.make_icmw_state(Nx=60, Nz=60, no_spcm=(26, 38), seed=77,
                                   kernel_type="Hall_Bott", drizzle_fraction=0.1, r_tot=9.0E-3)
    if thin:   # more collisions, so that segments with hits occur
        st["dt_col_over_dV"] = st["dt_col_over_dV"] * 40.0
    seed = 2024
    # the regular entry point, through DeviceState (workspace from the caller)
    ref = DeviceState(st, draws="thinned" if thin else "philox", seed=seed)
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


def test_noalloc_short_draws_skip_the_step_and_report():
    """One draw short: the step is skipped as a whole (state unchanged), the
    flag and the pair count the buffer needs are reported."""
    from lacmopy_gb300 import DeviceState, _lib, synthetic
    lib = _lib.load()
    st = synthetic.make_icmw_state(Nx=12, Nz=10, no_spcm=(6, 8), seed=5, kernel_type="Hall_Bott")
    pairs = DeviceState(st, draws="philox").pair_count()
    d, n, Nx, Nz = _device_inputs(st)
    prm = DeviceState(st, draws="philox").params
    buf = torch.rand(pairs - 1, dtype=torch.float64, device="cuda")
    draws = _lib.Draws(buf.data_ptr(), buf.numel(), 1)
    before = {k: d[k].clone() for k in ("xi", "m_w", "m_s")}
    for _ in range(2):   # the flag is reported on a repeated call too
        _lib.check(_call(lib, d, n, Nx, Nz, prm, draws, 0), "noalloc")
        flags, p = _status(lib)
        assert flags & _lib.FLAG_DRAWS_SHORT
        assert p == pairs
        for k, v in before.items():
            assert torch.equal(d[k], v), k
    # sized from the reported count, the repeated call runs and clears the flag
    buf = torch.rand(pairs, dtype=torch.float64, device="cuda")
    draws = _lib.Draws(buf.data_ptr(), buf.numel(), 1)
    _lib.check(_call(lib, d, n, Nx, Nz, prm, draws, 0), "noalloc")
    flags, _ = _status(lib)
    assert not flags & _lib.FLAG_DRAWS_SHORT


def test_noalloc_cell_beyond_the_grid_is_flagged_and_left_out():
    """A SIP whose cell index lies beyond nx*nz is left out of the binning and
    flagged; the other SIPs collide exactly as with that SIP removed."""
    from lacmopy_gb300 import DeviceState, _lib, synthetic
    lib = _lib.load()
    st = synthetic.make_icmw_state(Nx=12, Nz=10, no_spcm=(6, 8), seed=6, kernel_type="Hall_Bott",
                                   drizzle_fraction=0.3, r_tot=12.5E-3)
    st["dt_col_over_dV"] = st["dt_col_over_dV"] * 60.0
    seed = 99
    bad = 17
    ref_st = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
    ref_st["active_ids"][bad] = False
    ref_st["cells"][1, bad] = -1
    ref = DeviceState(ref_st, draws="philox", seed=seed)
    ref.collision_step(None)
    want = ref.snapshot()
    d, n, Nx, Nz = _device_inputs(st)
    d["cell"][bad] = Nx * Nz + 3
    draws = _lib.Draws(None, 0, seed)
    _lib.check(_call(lib, d, n, Nx, Nz, ref.params, draws, 0), "noalloc")
    flags, _ = _status(lib)
    assert flags & _lib.FLAG_CELL_RANGE
    assert np.array_equal(d["no_cols"].cpu().numpy(), want["no_cols"])
    assert want["no_cols"].sum() > 0
    for k in ("xi", "m_w", "m_s"):
        assert np.array_equal(d[k].cpu().numpy(), want[k]), k


def test_noalloc_cell_above_65535_sips_is_flagged():
    """A cell above 65,535 SIPs (within the 524,288-SIP capacity) is not
    collided; the flag says so and the state is unchanged."""
    from lacmopy_gb300 import _lib
    from lacmopy_gb300.device import to_device
    lib = _lib.load()
    n, Nx, Nz = 70000, 2, 2
    rng = np.random.default_rng(1)
    d = {"xi": to_device(rng.uniform(1e3, 1e6, n)), "m_w": to_device(rng.uniform(1.0, 1e3, n)),
         "m_s": to_device(rng.uniform(1e-3, 1e-1, n)),
         "vel": to_device(rng.normal(0.0, 1.0, (2, n))),
         "T": to_device(np.full((Nx, Nz), 285.0)),
         "no_cols": torch.zeros(2, dtype=torch.int64, device="cuda"),
         "cell": torch.zeros(n, dtype=torch.int32, device="cuda")}
    prm = _lib.Params()
    prm.no_iter_impl_mass = 3
    prm.dt_col_over_dV = 1.0
    prm.E_col_const = 0.5
    before = {k: d[k].clone() for k in ("xi", "m_w", "m_s")}
    draws = _lib.Draws(None, 0, 3)
    _lib.check(_call(lib, d, n, Nx, Nz, prm, draws, 0), "noalloc")
    flags, p = _status(lib)
    assert flags & _lib.FLAG_CELL_TOO_BIG
    assert p == n * (n - 1) // 2
    for k, v in before.items():
        assert torch.equal(d[k], v), k
    assert int(d["no_cols"].sum()) == 0
