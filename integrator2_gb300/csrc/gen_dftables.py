"""Writes i2_dftables.h: the breakpoint tables of the double-float logarithm and arctangent
(i2_dfloat.cuh), each value rounded to an unevaluated float pair hi + lo from its float64 value
(float64's log and arctan are within an ulp of 2^-53, well below the pair's 2^-48).

    python integrator2_gb300/csrc/gen_dftables.py

Tables:
  log:  F_j = 0.75 + j/512, j = 0..384 (F_j exact in binary32): log(F_j) and 1/F_j
  atan: c_j = j/512, j = 0..512: atan(c_j)
  sincos: s_j = j/512, j = 0..403: sin(s_j), cos(s_j)
  constants: ln 2, pi, pi/2 (pairs); pi/2 in three parts for the argument reduction of sin/cos
"""
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def split(v: float):
    hi = np.float32(v)
    lo = np.float32(v - float(hi))
    assert float(hi) + float(lo) - v == 0.0 or abs(float(hi) + float(lo) - v) <= 2.0 ** -48 * abs(v)
    return float(hi).hex(), float(lo).hex()


def fmt(h, l):
    # C99 hexadecimal float literals of the float values (exact)
    return f"{{{h}f, {l}f}}"


def main():
    log_rows = []
    for j in range(385):
        F = 0.75 + j / 512.0
        assert np.float32(F) == F
        lh, ll = split(math.log(F))
        ih, il = split(1.0 / F)
        log_rows.append(f"    {{{lh}f, {ll}f, {ih}f, {il}f}}, /* j = {j} */")
    atan_rows = []
    for j in range(513):
        h, l = split(math.atan(j / 512.0))
        atan_rows.append(f"    {fmt(h, l)}, /* j = {j} */")
    sc_rows = []
    for j in range(404):
        sh, sl = split(math.sin(j / 512.0))
        ch, cl = split(math.cos(j / 512.0))
        sc_rows.append(f"    {{{sh}f, {sl}f, {ch}f, {cl}f}}, /* j = {j} */")
    consts = {"kDfLn2": math.log(2.0), "kDfPi": math.pi, "kDfHalfPi": math.pi / 2}
    out = ["// i2_dftables.h -- written by gen_dftables.py; do not edit.",
           "// Breakpoint tables of the double-float logarithm and arctangent (i2_dfloat.cuh): each value",
           "// is the float64 value rounded to an unevaluated pair of binary32 numbers hi + lo.",
           "#pragma once", "",
           "// {log(F_j).hi, log(F_j).lo, (1/F_j).hi, (1/F_j).lo}, F_j = 0.75 + j/512, j = 0..384",
           "#define I2_DF_LOG_TABLE { \\"]
    out += [r + " \\" for r in log_rows]
    out += ["}", "",
            "// {atan(j/512).hi, atan(j/512).lo}, j = 0..512",
            "#define I2_DF_ATAN_TABLE { \\"]
    out += [r + " \\" for r in atan_rows]
    out += ["}", "",
            "// {sin(j/512).hi, sin(j/512).lo, cos(j/512).hi, cos(j/512).lo}, j = 0..403",
            "#define I2_DF_SINCOS_TABLE { \\"]
    out += [r + " \\" for r in sc_rows]
    out += ["}", ""]
    # pi/2 = P1 + P2 + P3 to about 1e-22: P1 and P2 each the binary32 rounding of what is left;
    # 6.123233995736766e-17 is pi/2 - fl64(pi/2) (rounded to float64)
    p1 = np.float32(math.pi / 2)
    rest = math.pi / 2 - float(p1) + 6.123233995736766e-17
    p2 = np.float32(rest)
    p3 = np.float32(rest - float(p2))
    for name, v in (("PIO2_1", p1), ("PIO2_2", p2), ("PIO2_3", p3)):
        out.append(f"#define I2_{name} {float(v).hex()}f")
    for name, v in consts.items():
        h, l = split(v)
        out.append(f"#define I2_{name.upper()[3:]}_HI {h}f")
        out.append(f"#define I2_{name.upper()[3:]}_LO {l}f")
    out.append("")
    with open(os.path.join(HERE, "i2_dftables.h"), "w") as f:
        f.write("\n".join(out))


if __name__ == "__main__":
    main()
