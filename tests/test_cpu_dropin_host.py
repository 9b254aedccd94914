"""Host-side checks of the one-call drop-in step (no GPU): which NumPy arrays
the kept device buffers can take directly, and the copy-list structures the
C ABI reads."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_host_view_takes_matching_contiguous_arrays():
    from lacmopy_gb300.device import DeviceState
    hv = DeviceState._host_view
    t64 = torch.empty((2, 5), dtype=torch.float64)
    a = np.zeros((2, 5))
    assert hv(a, t64, True) is a
    assert hv(np.zeros((2, 5), np.float32), t64, False) is None      # element type
    assert hv(np.zeros((2, 4)), t64, False) is None                  # count
    assert hv(np.zeros((5, 4))[:, :2].T, t64, False) is None         # not contiguous
    ro = np.zeros((2, 5))
    ro.flags.writeable = False
    assert hv(ro, t64, False) is ro and hv(ro, t64, True) is None    # read-only: input only
    assert hv(torch.zeros(10, dtype=torch.float64), t64, False) is None
    assert hv(3.0, t64, False) is None
    # booleans travel as bytes
    tu8 = torch.empty(7, dtype=torch.uint8)
    b = np.array([True, False, True, True, False, False, True])
    v = hv(b, tu8, True)
    assert v is not None and v.dtype == np.uint8 and np.shares_memory(v, b)
    assert hv(np.zeros(2 * 5, np.int64).reshape(2, 5), torch.empty((2, 5), dtype=torch.int64),
              True) is not None


def test_copy_and_call_structures_match_the_header():
    """lacmo_copy_t and lacmo_dropin_t as the header lays them out (LP64)."""
    from lacmopy_gb300 import _lib
    assert ctypes.sizeof(_lib.Copy) == 24
    offs = {name: getattr(_lib.Dropin, name).offset for name, _ in _lib.Dropin._fields_}
    assert offs["in_"] == 0 and offs["n_in"] == 8 and offs["out"] == 16
    assert offs["sips"] == 32 and offs["ws"] == 64 and offs["ws_bytes"] == 72
    assert offs["plan"] == 112 and offs["col_step"] == 120 and offs["col_step_out"] == 128
    assert offs["copy_mode"] == 136 and ctypes.sizeof(_lib.Dropin) == 144
    assert (_lib.COPY_AUTO, _lib.COPY_ENGINE, _lib.COPY_KERNEL) == (0, 1, 2)
