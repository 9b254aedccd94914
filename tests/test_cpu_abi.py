"""CPU-side checks: the C ABI library loads and exports every declared entry
point, the constants header matches the Python constants, and the
correctly-rounded math (host build of the same header the kernels use) is
correctly rounded against mpmath."""
import ctypes
import os
import re

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(REPO, "include", "lacmo_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(lacmo_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from lacmopy_gb300 import build
    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    names = _declared()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.lacmo_abi_version() == 1
    lib.lacmo_error_string.restype = ctypes.c_char_p
    assert lib.lacmo_error_string(-3) == b"injected draw buffer too short"


def _arity():
    """Number of parameters of every function the header declares."""
    txt = open(os.path.join(REPO, "include", "lacmo_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(lacmo_\w+)\s*\(([^;{]*?)\)\s*;", txt, flags=re.S):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_python_binding_covers_header():
    from lacmopy_gb300 import _lib
    assert set(_declared()) == set(_lib.PROTOTYPES)
    arity = _arity()
    wrong = {n: (len(args), arity[n]) for n, (_, args) in _lib.PROTOTYPES.items()
             if n in arity and len(args) != arity[n]}
    assert not wrong, wrong


def test_workspace_size_and_argument_errors():
    from lacmopy_gb300 import _lib
    lib = _lib.load()
    assert lib.lacmo_workspace_bytes(360000, 75, 75) > 360000 * 40
    assert lib.lacmo_workspace_bytes(-1, 75, 75) == 0
    # argument checks happen before any CUDA call: usable without a GPU
    assert lib.lacmo_prepare(None, None, None, None, 0, None) == -1
    assert lib.lacmo_collision_step_golovin(None, None, 10, 1.0, None, None, 0, 0, None) == -1
    x = ctypes.c_void_p(16)
    assert lib.lacmo_collision_step_golovin(x, x, 9000, 1.0, x, None, 0, 0, None) == -5
    # the one-call drop-in step: a missing call, or one without its structures
    assert lib.lacmo_dropin_adv_step(None, None) == -1
    call = _lib.Dropin()
    assert lib.lacmo_dropin_adv_step(ctypes.byref(call), None) == -1


def test_constants_header_matches_python():
    from lacmopy_gb300.csrc_gen import render_constants
    assert open(os.path.join(REPO, "lacmopy_gb300", "csrc", "lacmo_constants.h")).read() == \
        render_constants()


def test_crmath_correctly_rounded(oracle_cr):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    rng = np.random.default_rng(0)
    x = np.exp(rng.uniform(-25, 25, 3000))
    y = np.concatenate([np.full(1500, 1.0 / 3.0), rng.uniform(-4, 4, 1500)])
    p, hp = oracle_cr.cr_pow(x, y)
    l, hl = oracle_cr.cr_log(x)
    for k in range(x.size):
        assert p[k] == float(mpmath.power(mpmath.mpf(float(x[k])), mpmath.mpf(float(y[k]))))
        assert l[k] == float(mpmath.log(mpmath.mpf(float(x[k]))))
    assert hp.sum() == 0 and hl.sum() == 0


def test_crmath_specials(oracle_cr):
    x = np.array([1.0, 0.0, -1.0, np.inf, np.nan, 5e-324, 1e308])
    l, _ = oracle_cr.cr_log(x)
    assert l[0] == 0.0 and l[1] == -np.inf and np.isnan(l[2]) and l[3] == np.inf
    assert np.isnan(l[4]) and np.isclose(l[5], np.log(5e-324)) and np.isclose(l[6], np.log(1e308))
    p, _ = oracle_cr.cr_pow(np.array([1.0, 0.0, -8.0, np.inf, 8.0]), 1.0 / 3.0)
    assert p[0] == 1.0 and p[1] == 0.0 and np.isnan(p[2]) and p[3] == np.inf
    assert abs(p[4] - 2.0) < 1e-15
