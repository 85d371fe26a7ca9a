"""Writes bsg_crmath_tables.h: the constants and tables of the float-float
exp and log in bsg_crmath.h, computed in exact rational arithmetic from
60-digit decimal values of ln 2, 2^(j/32) and ln(256/k).

    python gen_crmath_tables.py        # rewrites bsg_crmath_tables.h here

Every float is written as a hex literal, so the header is exact."""
import decimal
import os
from fractions import Fraction

decimal.getcontext().prec = 60
D = decimal.Decimal
HERE = os.path.dirname(os.path.abspath(__file__))


def round_bits(v: Fraction, bits: int) -> Fraction:
    """v rounded to `bits` significant bits, ties to even."""
    if v == 0:
        return Fraction(0)
    a = abs(v)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if Fraction(2) ** e > a:
        e -= 1
    scale = Fraction(2) ** (bits - 1 - e)
    return round(v * scale) / scale


def f32(v: Fraction) -> Fraction:
    return round_bits(v, 24)


def hexf(v: Fraction) -> str:
    x = float(v)
    assert Fraction(x) == v, "not representable"
    return x.hex() + "f" if x != 0 else "0.0f"


def split2(v: Fraction):
    hi = f32(v)
    return hi, f32(v - hi)


def main():
    ln2 = Fraction(D(2).ln())
    L = ln2 / 32
    L1 = round_bits(L, 12)       # n * L1 exact for |n| < 2^12
    L2 = f32(L - L1)
    L3 = f32(L - L1 - L2)
    inv_l = f32(1 / L)
    LN2H = round_bits(ln2, 16)   # e * LN2H exact for |e| <= 2^8
    LN2M = f32(ln2 - LN2H)
    LN2L = f32(ln2 - LN2H - LN2M)
    exp_tab = [split2(Fraction(D(2) ** (D(j) / D(32)))) for j in range(32)]
    # log: m in [1, 2) indexed by its top 8 fraction bits i; for i >= 128
    # the argument is halved (m/2 in [0.75, 1)).  c_i = k_i / 256 with k_i
    # the integer nearest 256 / (the interval's midpoint), and ln(256/k_i).
    log_tab = []
    for i in range(256):
        mid = 1 + (Fraction(i) + Fraction(1, 2)) / 256
        if i >= 128:
            mid /= 2
        k = round(256 / mid)
        hi, lo = split2(Fraction((D(256) / D(k)).ln()))
        log_tab.append((Fraction(k, 256), hi, lo))

    out = []
    w = out.append
    w("// bsg_crmath_tables.h -- written by gen_crmath_tables.py; do not edit.")
    w("// Constants and tables of the float-float exp and log in bsg_crmath.h.")
    w("#pragma once")
    w("")
    w("// ln2/32 = kL1 + kL2 + kL3 (kL1 has 12 significant bits), and 32/ln2")
    w(f"#define BSG_CR_L1 {hexf(L1)}")
    w(f"#define BSG_CR_L2 {hexf(L2)}")
    w(f"#define BSG_CR_L3 {hexf(L3)}")
    w(f"#define BSG_CR_INV_L {hexf(inv_l)}")
    w("// ln2 = kLN2H + kLN2M + kLN2L (kLN2H has 16 significant bits)")
    w(f"#define BSG_CR_LN2H {hexf(LN2H)}")
    w(f"#define BSG_CR_LN2M {hexf(LN2M)}")
    w(f"#define BSG_CR_LN2L {hexf(LN2L)}")
    w("")
    w("// 2^(j/32) = hi + lo, j = 0..31")
    w("#define BSG_CR_EXP_TABLE \\")
    for j, (hi, lo) in enumerate(exp_tab):
        w(f"    {{{hexf(hi)}, {hexf(lo)}}}" + (", \\" if j < 31 else ""))
    w("")
    w("// {c = k/256, ln(256/k) hi, lo, 0} by the top 8 fraction bits of m in [1, 2)")
    w("#define BSG_CR_LOG_TABLE \\")
    for i, (c, hi, lo) in enumerate(log_tab):
        w(f"    {{{hexf(c)}, {hexf(hi)}, {hexf(lo)}, 0.0f}}" + (", \\" if i < 255 else ""))
    w("")
    with open(os.path.join(HERE, "bsg_crmath_tables.h"), "w") as f:
        f.write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
