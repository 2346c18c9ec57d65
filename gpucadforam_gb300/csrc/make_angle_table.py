"""Writes angle_table.h: sin and cos of the angles k / 32 rad, k = -101 .. 101
(the range [-3.156, 3.156] covers every angle reduced to [-pi, pi]), each as an
unevaluated pair of floats (hi = the float nearest the value, lo = the float
nearest the remainder), so hi + lo carries about 48 bits; and the Taylor
coefficients of sin(pi u) (odd powers 1..9) and cos(pi u) (even powers 2..10),
rounded to float, for |u| <= 1/4.

The values are computed from their Taylor series in decimal arithmetic at 40
significant digits (standard library only), so the table does not depend on any
platform's libm.  Run from this directory:  python make_angle_table.py
"""
from __future__ import annotations

import decimal
import os
import struct

STEP_INV = 32
K = 101
D = decimal.Decimal
decimal.getcontext().prec = 40


def taylor_sin_cos(x: decimal.Decimal) -> tuple[decimal.Decimal, decimal.Decimal]:
    s, c = D(0), D(0)
    term = D(1)  # x^n / n!
    n = 0
    while True:
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
        if abs(term) < D(10) ** -45:
            return s, c


def f32(v: float) -> float:
    return struct.unpack("<f", struct.pack("<f", v))[0]


def split(v: decimal.Decimal) -> tuple[float, float]:
    hi = f32(float(v))
    lo = f32(float(v - D(hi)))
    return hi, lo


def lit(v: float) -> str:
    if v == 0.0:
        return "0.0f"
    mant, exp = v.hex().split("p")
    return mant.rstrip("0").rstrip(".") + "p" + exp + "f"


def pi_decimal() -> decimal.Decimal:
    # Machin's formula: pi = 16 atan(1/5) - 4 atan(1/239)
    def atan_inv(n: int) -> decimal.Decimal:
        x = D(1) / n
        x2 = x * x
        term, total, k = x, x, 1
        while abs(term) > D(10) ** -45:
            term = -term * x2
            k += 2
            total += term / k
        return total

    return 16 * atan_inv(5) - 4 * atan_inv(239)


def render() -> str:
    pi = pi_decimal()
    coef = []
    fact = D(1)
    for n in range(1, 11):
        fact *= n
        sign = -1 if (n // 2) % 2 else 1
        coef.append((n, f32(float(sign * pi ** n / fact))))
    rows = []
    for k in range(-K, K + 1):
        s, c = taylor_sin_cos(D(k) / D(STEP_INV))
        sh, sl = split(s)
        ch, cl = split(c)
        rows.append(f"    {{{lit(sh)}, {lit(sl)}, {lit(ch)}, {lit(cl)}}},  // k = {k}")
    out = [
        "// Generated by make_angle_table.py: sin and cos of k / 32 rad for k = -101 .. 101,\n",
        "// each as {sin hi, sin lo, cos hi, cos lo} (hi + lo to about 48 bits).\n",
        "// Data only; shared by the graded-lattice kernels and the CPU oracle.\n",
        "#pragma once\n\n",
        f"#define GCM_ANGLE_STEP_INV {STEP_INV}\n#define GCM_ANGLE_K {K}\n\n",
        "// sin(pi u) = sum over odd n of GCM_SINPI_Cn u^n, cos(pi u) = 1 + sum over even n\n",
        "// of GCM_COSPI_Cn u^n: (-1)^floor(n/2) pi^n / n!, rounded to float\n",
    ]
    for n, v in coef:
        name = "SINPI" if n % 2 else "COSPI"
        out.append(f"#define GCM_{name}_C{n} {lit(v)}\n")
    out.append("\n#define GCM_ANGLE_TABLE_ROWS \\\n")
    out.append(" \\\n".join(r.replace("  // ", "  /* ") + " */" for r in rows))
    out.append("\n")
    return "".join(out)


HEADER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "angle_table.h")


def main() -> None:
    with open(HEADER, "w") as f:
        f.write(render())


if __name__ == "__main__":
    main()
