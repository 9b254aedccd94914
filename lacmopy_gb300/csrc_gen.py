"""Generate csrc/lacmo_constants.h from lacmopy_gb300.constants.

``python -m lacmopy_gb300.csrc_gen`` rewrites the header (hexadecimal float
literals, so the CUDA kernels see the reference's exact constants).
"""
import os

from .constants import named_doubles

HEADER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", "lacmo_constants.h")


def render_constants():
    lines = ["/* Generated by lacmopy_gb300/csrc_gen.py from lacmopy_gb300/constants.py. */",
             "/* Physical constants and fit coefficients of the SIP hot path,   */",
             "/* bit-identical to the values the reference model computes.      */",
             "#pragma once", ""]
    for k, v in named_doubles().items():
        lines.append(f"#define LC_{k} ({float(v).hex()}) /* {v!r} */")
    return "\n".join(lines) + "\n"


if __name__ == "__main__":
    with open(HEADER, "w") as f:
        f.write(render_constants())
