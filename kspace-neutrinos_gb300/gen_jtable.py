#!/usr/bin/env python3
"""Generate csrc/jfit_table.h: the fitting function of J(x) (delta_tot_table.c:417-428),

    J(x) = (1 + 0.0168 x^2 + 0.0407 x^4) / (1 + 2.1734 x^2 + 1.6787 x^4.1811 + 0.1467 x^8),

as piecewise polynomials for the GPU integrand.  For x in [2^E0, 2^E1) the octave and the
top SUB_BITS mantissa bits select a piece [lo, hi); on it J is the degree-DEG
interpolant at Chebyshev points in u = (x - c) / h (c, h: centre and half-width).  h is a
power of two, so the monomial coefficients in u are stored scaled by h^-j, exactly:
the device evaluates the polynomial in t = x - c (one subtraction and DEG FMAs).
Computed in 40-digit arithmetic (mpmath); the largest relative error of the FP64
evaluation (Horner in t) over 400 points per piece of a sample of pieces is printed and
stays near 2e-16 -- below the ~1e-15 error of evaluating x^4.1811 as exp(4.1811 log x)
in FP64 for large x.  Outside [2^E0, 2^E1)
the device evaluates the formula directly (below 2^E0 the x^4.1811 term is below 1e-25
relative and is dropped).

    python gen_jtable.py          # writes csrc/jfit_table.h
"""
import os

import mpmath as mp

HERE = os.path.dirname(os.path.abspath(__file__))
E0, E1 = -20, 13
SUB_BITS = 6
DEG = 7
mp.mp.dps = 40


def J(x):
    x = mp.mpf(x)
    if x <= 0:
        return mp.mpf(1)
    x2 = x * x
    return (1 + mp.mpf("0.0168") * x2 + mp.mpf("0.0407") * x2 * x2) / (
        1 + mp.mpf("2.1734") * x2 + mp.mpf("1.6787") * mp.e ** (mp.mpf("4.1811") * mp.log(x)) +
        mp.mpf("0.1467") * x2 ** 4)


def piece(lo, hi):
    c = (lo + hi) / 2
    h = (hi - lo) / 2
    n = DEG + 1
    us = [mp.cos(mp.pi * (k + mp.mpf(1) / 2) / n) for k in range(n)]
    A = mp.matrix([[u ** j for j in range(n)] for u in us])
    coef = mp.lu_solve(A, mp.matrix([J(c + h * u) for u in us]))
    return c, h, [coef[j] for j in range(n)]


def main():
    sub = 1 << SUB_BITS
    rows = []
    worst = 0.0
    for e in range(E0, E1):
        for s in range(sub):
            lo = mp.mpf(2) ** e * (1 + mp.mpf(s) / sub)
            hi = mp.mpf(2) ** e * (1 + mp.mpf(s + 1) / sub)
            c, h, coef = piece(lo, hi)
            cd, ih = float(c), float(1 / h)
            assert ih == 2.0 ** round(mp.log(ih, 2))  # a power of two: the scaling is exact
            cf = [float(v) * ih ** j for j, v in enumerate(coef)]
            rows.append([cd] + cf)
            if s % 7 == 0 and (e - E0) % 3 == 0:  # spot check in FP64 arithmetic
                for t in range(400):
                    x = float(lo + (hi - lo) * mp.mpf(t) / 400)
                    tt = x - cd
                    v = 0.0
                    for cj in reversed(cf):
                        v = v * tt + cj
                    worst = max(worst, abs(float((v - J(x)) / J(x))))
    out = os.path.join(HERE, "csrc", "jfit_table.h")
    with open(out, "w") as f:
        f.write("/* Generated by kspace-neutrinos_gb300/gen_jtable.py: the J(x) fitting function of\n"
                " * delta_tot_table.c:417-428 as piecewise polynomials.  Piece p = (octave - E0) * 2^SUB_BITS\n"
                " * + top SUB_BITS mantissa bits of x covers [lo, hi); entry: centre c, then DEG+1\n"
                " * monomial coefficients in t = x - c.\n"
                " * Largest relative error of the FP64 evaluation in the generator's check: %.2e */\n" % worst)
        f.write("#ifndef KSP_JFIT_TABLE_H\n#define KSP_JFIT_TABLE_H\n")
        f.write("#define KSP_JFIT_E0 (%d)\n#define KSP_JFIT_E1 (%d)\n#define KSP_JFIT_SUB_BITS %d\n#define KSP_JFIT_DEG %d\n"
                % (E0, E1, SUB_BITS, DEG))
        f.write("#define KSP_JFIT_STRIDE %d\n#define KSP_JFIT_PIECES %d\n" % (DEG + 2, len(rows)))
        f.write("#define KSP_JFIT_TABLE_INIT { \\\n")
        for r in rows:
            f.write("    " + ", ".join("%.17g" % v for v in r) + ", \\\n")
        f.write("}\n#endif\n")
    print("wrote", out, "pieces", len(rows), "worst relative error %.3e" % worst)


if __name__ == "__main__":
    main()
