"""Writes gd_pow10.h: the binary64 values nearest to 10^k, k = -340 .. 340 (0 for those below
the smallest subnormal, +inf above the largest double), for the fast path of the "%.6g"
formatter in gd_text.cuh.  Exact rational arithmetic (fractions.Fraction) rounded once by
float(), which rounds to nearest, ties to even.

    python golikov_2d_gb300/csrc/gen_pow10.py
"""
import os
from fractions import Fraction

LO, HI = -340, 340


def main():
    vals = []
    for k in range(LO, HI + 1):
        try:
            v = float(Fraction(10) ** k)
        except OverflowError:
            v = float("inf")
        vals.append(v)
    lines = ["// gd_pow10.h -- generated by gen_pow10.py: the binary64 values nearest to 10^k,",
             f"// k = {LO} .. {HI} (index k - ({LO})); 0 below the subnormals, inf above DBL_MAX.",
             "#pragma once", "", f"#define GD_POW10_LO ({LO})", f"#define GD_POW10_HI ({HI})",
             "#define GD_POW10_TABLE \\"]
    for i in range(0, len(vals), 4):
        chunk = ", ".join("__builtin_inf()" if v == float("inf") else v.hex() for v in vals[i:i + 4])
        lines.append("    " + chunk + ("," if i + 4 < len(vals) else "") + " \\")
    lines.append("")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "gd_pow10.h")
    with open(out, "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
