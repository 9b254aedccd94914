"""Write lacmo_constants.h from lacmopy_gb300.constants (hex-float literals).

Run from the repository root: ``python lacmopy_gb300/csrc/gen_constants.py``.
The header is committed; tests/test_constants.py checks it is up to date.
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from lacmopy_gb300.constants import named_doubles  # noqa: E402


def render():
    lines = ["/* Generated by gen_constants.py from lacmopy_gb300/constants.py. */",
             "/* Physical constants and fit coefficients of the SIP hot path,   */",
             "/* bit-identical to the values the reference model computes.      */",
             "#pragma once", ""]
    for k, v in named_doubles().items():
        lines.append(f"#define LC_{k} ({float(v).hex()}) /* {v!r} */")
    return "\n".join(lines) + "\n"


if __name__ == "__main__":
    with open(os.path.join(HERE, "lacmo_constants.h"), "w") as f:
        f.write(render())
