"""Generate csrc/lacmo_constants.h from lacmopy_gb300.constants, and
csrc/lacmo_thin_tables.h (the hit probabilities of the thinned collision
draws, computed in exact rational arithmetic).

``python -m lacmopy_gb300.csrc_gen`` rewrites both headers (hexadecimal float
literals, so the CUDA kernels and the oracle see identical values).
"""
import os
from fractions import Fraction

from .constants import named_doubles

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc")
HEADER = os.path.join(HERE, "lacmo_constants.h")
THIN_HEADER = os.path.join(HERE, "lacmo_thin_tables.h")
# thinning bounds q = 2^-e, e = THIN_E_MIN .. THIN_E_MAX; chunks of up to THIN_L pairs
THIN_E_MIN, THIN_E_MAX, THIN_L = 2, 127, 32


def render_constants():
    lines = ["/* Generated by lacmopy_gb300/csrc_gen.py from lacmopy_gb300/constants.py. */",
             "/* Physical constants and fit coefficients of the SIP hot path,   */",
             "/* bit-identical to the values the reference model computes.      */",
             "#pragma once", ""]
    for k, v in named_doubles().items():
        lines.append(f"#define LC_{k} ({float(v).hex()}) /* {v!r} */")
    return "\n".join(lines) + "\n"


def thin_tables():
    """H[e][m] = 1 - (1 - 2^-e)^m, the probability that at least one of m
    independent uniforms falls below q = 2^-e, and P[e][r] = q / H[e][r], the
    probability that the first of r remaining pairs is a hit given that one
    of them is; each exact, rounded once to double."""
    H, P = [], []
    for e in range(THIN_E_MIN, THIN_E_MAX + 1):
        q = Fraction(1, 2 ** e)
        hr = [float(1 - (1 - q) ** m) for m in range(1, THIN_L + 1)]
        pr = [float(q / (1 - (1 - q) ** r)) for r in range(1, THIN_L + 1)]
        H.append(hr)
        P.append(pr)
    return H, P


def render_thin_tables():
    H, P = thin_tables()
    ne = THIN_E_MAX - THIN_E_MIN + 1
    lines = ["/* Generated by lacmopy_gb300/csrc_gen.py (exact rational arithmetic). */",
             "/* Thinned collision draws: q = 2^-e, e = LACMO_THIN_E_MIN ..        */",
             "/* LACMO_THIN_E_MAX; chunks of up to LACMO_THIN_L pairs.             */",
             "/* LACMO_THIN_H[e - E_MIN][m - 1] = 1 - (1 - q)^m                    */",
             "/* LACMO_THIN_P[e - E_MIN][r - 1] = q / (1 - (1 - q)^r)              */",
             "#pragma once", "",
             f"#define LACMO_THIN_E_MIN {THIN_E_MIN}",
             f"#define LACMO_THIN_E_MAX {THIN_E_MAX}",
             f"#define LACMO_THIN_L {THIN_L}", "",
             "#ifndef LACMO_THIN_QUAL",
             "#define LACMO_THIN_QUAL static const",
             "#endif"]
    for name, T in (("LACMO_THIN_H", H), ("LACMO_THIN_P", P)):
        lines.append(f"LACMO_THIN_QUAL double {name}[{ne}][{THIN_L}] = {{")
        for row in T:
            lines.append("  {" + ", ".join(v.hex() for v in row) + "},")
        lines.append("};")
    # the same decisions on the 53-bit integer u53 of a uniform u = u53 2^-53:
    # u < X  <=>  u53 < ceil(X 2^53)
    lines += ["/* LACMO_THIN_HT / _PT = ceil(2^53 LACMO_THIN_H / _P): u < H <=> u53 < HT */"]
    for name, T in (("LACMO_THIN_HT", H), ("LACMO_THIN_PT", P)):
        lines.append(f"LACMO_THIN_QUAL uint64_t {name}[{ne}][{THIN_L}] = {{")
        for row in T:
            lines.append("  {" + ", ".join(f"{threshold53(v)}ull" for v in row) + "},")
        lines.append("};")
    return "\n".join(lines) + "\n"


def threshold53(x):
    """ceil(x 2^53) for a double x in [0, 1], exactly."""
    f = Fraction(x) * 2 ** 53
    return -((-f.numerator) // f.denominator)


if __name__ == "__main__":
    with open(HEADER, "w") as f:
        f.write(render_constants())
    with open(THIN_HEADER, "w") as f:
        f.write(render_thin_tables())
