"""Writes fs_mathtab.h: the constant tables of the table-driven FP64
logarithm and exponential in fs_fastmath.cuh, computed with 60-digit decimal
arithmetic (Python's decimal module) and rounded once to the nearest double,
so the header is the same whichever machine runs this script.

  python fluidsim_gb300/csrc/make_mathtab.py   # rewrites fs_mathtab.h beside it
"""
import decimal
import math
import os

D = decimal.Decimal
decimal.getcontext().prec = 60
LN2 = D(2).ln()


def nearest(v):
    """The double nearest to the Decimal v (float(Decimal) rounds correctly)."""
    return float(v)


def trunc_bits(v, bits):
    """v with its significand cut to `bits` bits (towards zero)."""
    m, e = math.frexp(nearest(v))
    scale = 2 ** bits
    return math.ldexp(int(m * scale) / scale, e)


def main():
    lines = ["// fs_mathtab.h -- generated by make_mathtab.py; do not edit.",
             "// Tables of the table-driven logarithm and exponential (fs_fastmath.cuh).",
             "#pragma once", ""]
    # log: F_j = 1 + j/128, j = 0..127: {1/F_j, ln F_j as head + tail}; the
    # head is a multiple of 2^-32, so e * FS_LN2_HI + head is exact in double
    rows = []
    for j in range(128):
        F = D(1) + D(j) / D(128)
        lnf = F.ln()
        head = float(int((lnf * D(2) ** 32).to_integral_value(rounding=decimal.ROUND_HALF_EVEN))) / 2.0 ** 32
        rows.append("    %s, %s, %s," % (nearest(D(1) / F).hex(), head.hex(), nearest(lnf - D(head)).hex()))
    lines += ["#define FS_LOG_TAB_N 128",
              "static __device__ const double fs_log_tab[3 * FS_LOG_TAB_N] = {"] + rows + ["};", ""]
    # exp: S_j = 2^(j/64), j = 0..63: {S_hi, S_lo} with S_hi + S_lo = S_j to ~107 bits
    rows = []
    for j in range(64):
        S = (D(j) / D(64) * LN2).exp()
        hi = nearest(S)
        lo = nearest(S - D(hi))
        rows.append("    %s, %s," % (hi.hex(), lo.hex()))
    lines += ["#define FS_EXP_TAB_N 64",
              "static __device__ const double fs_exp_tab[2 * FS_EXP_TAB_N] = {"] + rows + ["};", ""]
    ln2_hi = trunc_bits(LN2, 32)            # e * LN2_HI exact for |e| < 2^21
    ln2_lo = nearest(LN2 - D(ln2_hi))
    l1 = trunc_bits(LN2 / 64, 32)           # k * L1 exact for |k| < 2^21
    l2 = nearest(LN2 / 64 - D(l1))
    inv_l = nearest(D(64) / LN2)
    lines += ["#define FS_LN2_HI %s" % ln2_hi.hex(),
              "#define FS_LN2_LO %s" % ln2_lo.hex(),
              "#define FS_EXP_L1 %s" % l1.hex(),
              "#define FS_EXP_L2 %s" % l2.hex(),
              "#define FS_EXP_INV_L %s" % inv_l.hex(), ""]
    # Taylor coefficients 1/n! and (-1)^(n+1)/n, rounded once
    for n in range(2, 8):
        lines.append("#define FS_EXP_C%d %s" % (n, nearest(D(1) / D(math.factorial(n))).hex()))
    for n in range(2, 8):
        lines.append("#define FS_LOG_C%d %s" % (n, nearest(D((-1) ** (n + 1)) / D(n)).hex()))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fs_mathtab.h")
    with open(out, "w") as f:
        f.write("\n".join(lines) + "\n")
    return out


if __name__ == "__main__":
    print(main())
