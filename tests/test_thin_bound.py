"""CPU checks of the certified bounds behind the thinned draws
(lacmopy_gb300/csrc/lacmo_thin.h, built into the oracle library): the FP32
cube root is within a few ulp, and the segment bound is at least the exact
FP64 p_crit of the reference (collision/all_or_nothing.py:553-575) for every
pair it covers, given FP32 copies with the errors the kernel's copies have."""
import math

import numpy as np


def test_fp32_cube_root_within_a_few_ulp(oracle_cr):
    rng = np.random.default_rng(3)
    x = (10.0 ** rng.uniform(-30, 30, 200000)).astype(np.float32)
    y = oracle_cr.lt_cbrtf(x).astype(np.float64)
    rel = np.abs(y / np.cbrt(x.astype(np.float64)) - 1.0)
    assert rel.max() < 3.0e-7


def _p_crit(xa, xb, Ra, Rb, e, ua, ub, wa, wb, dtdv):
    # the reference's operation order
    Rs = Ra + Rb
    dv = math.sqrt((ua - ub) ** 2 + (wa - wb) ** 2)
    return max(xa, xb) * dtdv * (math.pi * Rs * Rs * e * dv * 1.0E-12)


def test_segment_bound_covers_every_pair(oracle_cr):
    rng = np.random.default_rng(11)
    nb = 48
    E = rng.uniform(0.0, 4.0, (nb, nb))
    E[rng.random((nb, nb)) < 0.1] = 0.0
    Ef = E.astype(np.float32)
    erow = Ef.max(axis=1)
    checked = 0
    for trial in range(60):
        n = int(rng.integers(2, 97))
        xi = 10.0 ** rng.uniform(3, 10, n)
        R = 10.0 ** rng.uniform(-2, 3.5, n)
        u = rng.normal(0, 2, n)
        w = rng.normal(0, 4, n)
        same = rng.random(n) < 0.2            # equal velocities: cancellation
        u[same], w[same] = u[0], w[0]
        k = rng.integers(0, nb, n)
        dtdv = 10.0 ** rng.uniform(-9, -4)
        delta = rng.uniform(-1e-6, 1e-6, n)   # the FP32 radius error the kernel allows
        xf = xi.astype(np.float32)
        Rf = (R * (1.0 + delta)).astype(np.float32)
        uf, wf = u.astype(np.float32), w.astype(np.float32)
        for a in range(n - 1):
            for lo in range(((a + 1) // 32) * 32, n, 32):
                hi = min(lo + 32, n)
                Q = oracle_cr.segment_bound(xf, Rf, uf, wf, a, lo, hi, erow[k[a]],
                                            np.float32(dtdv))
                assert Q >= 0.0
                for j in range(max(lo, a + 1), hi):
                    p = _p_crit(xi[a], xi[j], R[a], R[j], E[k[a], k[j]], u[a], u[j], w[a], w[j],
                                dtdv)
                    assert p <= Q, (trial, a, j, p, Q)
                    checked += 1
    assert checked > 10000


def test_segment_bound_rejects_invalid_blocks(oracle_cr):
    x = np.array([1e6, 2e6, 0.0, 3e6], np.float32)
    R = np.array([10.0, 20.0, 30.0, 40.0], np.float32)
    u = np.zeros(4, np.float32)
    w = np.array([0.1, 0.2, 0.3, np.nan], np.float32)
    assert oracle_cr.segment_bound(x, R, u, w, 0, 0, 4, 1.0, 1e-6) < 0   # x = 0, NaN in block
    assert oracle_cr.segment_bound(x, R, u, w, 2, 0, 2, 1.0, 1e-6) < 0   # SIP a has x = 0
    assert oracle_cr.segment_bound(x, R, u, w, 0, 0, 2, 1.0, 1e-6) >= 0
