"""Write lacmo_crmath_tables.h: reduction tables for lacmo_crmath.h.

Run from the repository root: ``python lacmopy_gb300/csrc/gen_crmath_tables.py``
(needs mpmath).  The header is committed.

log table, 512 entries indexed by the exponent's lowest bit and the top 8
mantissa bits of m in [0.5, 2): r = 1/(bin centre) rounded to 9 significant
bits (so m * r - 1 is exact in double), and -log(r) as a double-double.  The
bins that contain 1.0 use r = 1.
exp table, 256 entries: 2^(j/256) as a double-double.
Constants: ln 2 split into a 42-bit head and two 53-bit tails, ln2/256 split
into a 34-bit head and two tails (k * head is exact for |k| < 2^19), 256/ln2,
1/k and 1/k! as double-doubles.  Tables are emitted as value lists so the
including header can instantiate a host and a device copy.
"""
import os

import mpmath

mpmath.mp.prec = 300
HERE = os.path.dirname(os.path.abspath(__file__))


def dd(v):
    hi = float(v)
    lo = float(v - mpmath.mpf(hi))
    return hi, lo


def round_bits(v, bits):
    m, e = mpmath.frexp(v)
    scale = mpmath.mpf(2) ** bits
    return float(mpmath.nint(m * scale) / scale * mpmath.mpf(2) ** e)


def split3(v, head_bits):
    m, e = mpmath.frexp(v)
    scale = mpmath.mpf(2) ** head_bits
    hi = float(mpmath.floor(m * scale) / scale * mpmath.mpf(2) ** e)
    rest = v - mpmath.mpf(hi)
    mid = float(rest)
    lo = float(rest - mpmath.mpf(mid))
    return hi, mid, lo


def main():
    lines = ["/* Generated by gen_crmath_tables.py (mpmath, 300-bit). */", "#pragma once", ""]
    r_tab, lh_tab, ll_tab = [], [], []
    for idx in range(512):
        if idx < 256:
            centre = mpmath.mpf(0.5) + (mpmath.mpf(idx) + 0.5) / 512
        else:
            centre = mpmath.mpf(1) + (mpmath.mpf(idx - 256) + 0.5) / 256
        if idx in (255, 256):
            r = 1.0
        else:
            r = round_bits(1 / centre, 9)
        h, l = dd(-mpmath.log(mpmath.mpf(r)))
        r_tab.append(r); lh_tab.append(h); ll_tab.append(l)
    def arr(name, vals):
        out = [f"#define {name.upper()}_VALUES \\"]
        for k in range(0, len(vals), 4):
            out.append("  " + ", ".join(float(v).hex() for v in vals[k:k + 4]) + ", \\")
        out.append("")
        return out
    lines += arr("lacmo_cr_log_r", r_tab)
    lines += arr("lacmo_cr_log_mlr_hi", lh_tab)
    lines += arr("lacmo_cr_log_mlr_lo", ll_tab)
    eh, el = [], []
    for j in range(256):
        h, l = dd(mpmath.mpf(2) ** (mpmath.mpf(j) / 256))
        eh.append(h); el.append(l)
    lines += arr("lacmo_cr_exp_hi", eh)
    lines += arr("lacmo_cr_exp_lo", el)
    ln2 = mpmath.log(2)
    h, m, l = split3(ln2, 42)
    lines += [f"#define LACMO_CR_LN2_HI ({h.hex()})", f"#define LACMO_CR_LN2_MID ({m.hex()})",
              f"#define LACMO_CR_LN2_LO ({l.hex()})"]
    h, m, l = split3(ln2 / 256, 34)
    lines += [f"#define LACMO_CR_LN2_256_HI ({h.hex()})", f"#define LACMO_CR_LN2_256_MID ({m.hex()})",
              f"#define LACMO_CR_LN2_256_LO ({l.hex()})"]
    lines += [f"#define LACMO_CR_INV_LN2_256 ({float(256 / ln2).hex()})"]
    for k in range(1, 14):
        h, l = dd(mpmath.mpf(1) / k)
        lines += [f"#define LACMO_CR_INV{k}_HI ({h.hex()})", f"#define LACMO_CR_INV{k}_LO ({l.hex()})"]
    for k in range(2, 10):
        h, l = dd(mpmath.mpf(1) / mpmath.factorial(k))
        lines += [f"#define LACMO_CR_INVF{k}_HI ({h.hex()})", f"#define LACMO_CR_INVF{k}_LO ({l.hex()})"]
    with open(os.path.join(HERE, "lacmo_crmath_tables.h"), "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
