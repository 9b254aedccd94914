"""How often the GPU's correctly rounded collision math (radius pow(x, 1/3),
kernel-bin log) differs from glibc libm, the reference's math under Numba:
the oracle's "cr" variant is the GPU's (bit for bit, tests/test_gpu_parity.py)
and its "nb" variant uses glibc.  The full-size parity test allows up to one
SIP in a thousand to differ from the glibc run; this measures the per-call
rates on 2 million log-uniform masses from aerosol to rain sizes."""
import numpy as np


def test_glibc_vs_correctly_rounded_rates(oracle_nb, oracle_cr):
    rng = np.random.default_rng(2024)
    n = 2_000_000
    m = np.exp(rng.uniform(np.log(1e-3), np.log(1e9), n))   # fg
    rho = rng.uniform(1000.0, 1770.0, n)
    R = {}
    for name, o in (("nb", oracle_nb), ("cr", oracle_cr)):
        out = np.empty(n)
        o.lib.orc_radius_from_mass_col(m, rho, n, out)
        R[name] = out
    r_rate = float(np.mean(R["nb"] != R["cr"]))
    # kernel bins of the Long/Bott table (R in um)
    lo, bl, nb = np.log(0.6), np.log(1.0 + 1.0 / 32.0), 372
    k = {}
    for name, o in (("nb", oracle_nb), ("cr", oracle_cr)):
        out = np.empty(n, dtype=np.int64)
        o.lib.orc_kernel_index(R["cr"], n, lo, bl, nb, out)   # same radii: the log alone
        k[name] = out
    k_rate = float(np.mean(k["nb"] != k["cr"]))
    print(f"radius mismatch rate {r_rate:.3e}, bin mismatch rate (log alone) {k_rate:.3e}")
    assert r_rate < 1e-3
    assert k_rate < 1e-4
    # the differences are last-bit roundings
    d = R["nb"] != R["cr"]
    if d.any():
        assert np.all(np.abs(R["nb"][d] - R["cr"][d]) <= np.spacing(R["cr"][d]))
