"""Writes bsg_swmath_tables.h: the tables of the table-driven Box-Muller
transform and exponential in bsg_swmath.h, computed from 70-digit decimal
values of ln 2, ln F, sin, cos and 2^(j/64) and rounded once to double.

    python gen_swmath_tables.py      # rewrites bsg_swmath_tables.h here

Every double is written as a hex literal, so the header is exact."""
import decimal
import os
from fractions import Fraction

decimal.getcontext().prec = 70
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


def f64(v) -> float:
    x = round_bits(Fraction(v), 53)
    d = float(x)
    assert Fraction(d) == x, "not representable"
    return d


def hexd(v) -> str:
    d = f64(v)
    return d.hex() if d != 0 else "0.0"


def atan_inv(x: int) -> D:
    """atan(1/x) by its Taylor series."""
    s, term, k, x2 = D(0), D(1) / D(x), 0, D(x) * D(x)
    while abs(term) > D(10) ** -75:
        s += term / (2 * k + 1) if k % 2 == 0 else -term / (2 * k + 1)
        term /= x2
        k += 1
    return s


PI = 16 * atan_inv(5) - 4 * atan_inv(239)  # Machin's formula


def sin_cos(x: D):
    """sin x and cos x by their Taylor series (|x| <= 2 pi)."""
    s, c = D(0), D(0)
    term, n = D(1), 0  # term = x^n / n!
    while n < 200:
        if n % 4 == 0:
            c += term
        elif n % 4 == 1:
            s += term
        elif n % 4 == 2:
            c -= term
        else:
            s -= term
        n += 1
        term = term * x / n
        if n > 10 and abs(term) < D(10) ** -75:
            break
    tiny = D(10) ** -60  # the zeros of sin and cos at multiples of pi / 2
    return (D(0) if abs(s) < tiny else s), (D(0) if abs(c) < tiny else c)


def main():
    ln2 = D(2).ln()
    out = []
    w = out.append
    w("// bsg_swmath_tables.h -- written by gen_swmath_tables.py; do not edit.")
    w("// Tables of the table-driven Box-Muller transform and exp in bsg_swmath.h.")
    w("#pragma once")
    w("")
    w("// 2 pi 2^-53: the angle of one unit of the 53-bit uniform grid")
    w(f"#define BSG_SW_TWO_PI_ULP {hexd(2 * PI / D(2) ** 53)}")
    w("")
    w("// {-2/F, -2 ln F} for F = 1 + j/128, j = 0..128; ln(F/2) for j >= 64")
    w("#define BSG_SW_LOG_TABLE \\")
    for j in range(129):
        F = D(1) + D(j) / D(128)
        inv = Fraction(-256, 128 + j)
        val = D(-2) * (F / 2 if j >= 64 else F).ln()
        w(f"    {{{hexd(inv)}, {hexd(val)}}}" + (", \\" if j < 128 else ""))
    w("")
    w("// 2 i ln 2, i = 0..63")
    w("#define BSG_SW_EXP2_TABLE \\")
    for i in range(64):
        w(f"    {hexd(2 * i * ln2)}" + (", \\" if i < 63 else ""))
    w("")
    w("// exp: 64/ln 2, and ln2/64 = L1 + L2")
    L = ln2 / 64
    L1 = f64(L)
    w(f"#define BSG_SW_INV_L {hexd(1 / L)}")
    w(f"#define BSG_SW_L1 {hexd(L)}")
    w(f"#define BSG_SW_L2 {hexd(Fraction(L) - Fraction(L1))}")
    w("")
    w("// 2^(j/64), j = 0..63")
    w("#define BSG_SW_EXP_TABLE \\")
    for j in range(64):
        w(f"    {hexd((D(j) / D(64) * ln2).exp())}" + (", \\" if j < 63 else ""))
    w("")
    w("// {sin, cos}(2 pi j / 256), j = 0..255")
    w("#define BSG_SW_ANGLE_TABLE \\")
    for j in range(256):
        s, c = sin_cos(2 * PI * D(j) / D(256))
        w(f"    {{{hexd(s)}, {hexd(c)}}}" + (", \\" if j < 255 else ""))
    w("")
    with open(os.path.join(HERE, "bsg_swmath_tables.h"), "w") as f:
        f.write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
