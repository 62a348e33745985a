#!/usr/bin/env python3
"""Compute the 61-point Gauss-Kronrod rule (30-point Gauss + 31 Kronrod nodes) from
its mathematical definition and write it as a C header.

Method (Kronrod 1965; see also Laurie 1997, Math. Comp. 66):
  * the 30 Gauss-Legendre nodes are the zeros of P_30;
  * the 31 added nodes are the zeros of the Stieltjes polynomial E_31, the monic
    degree-31 polynomial orthogonal to every polynomial of degree <= 30 under the
    (sign-changing) weight P_30(x) on [-1, 1];
  * the 61 Kronrod weights make the rule exact for all polynomials of degree <= 91;
    they are obtained by solving the moment equations sum_i w_i P_j(x_i) = 2 delta_j0
    (j = 0..60) in 120-digit arithmetic.

The rule is the one QUADPACK's QAG uses for key 6 / GSL_INTEG_GAUSS61 (Piessens et
al. 1983), which the kspace-neutrinos integrator calls (delta_tot_table.c:404,597;
omega_nu_single.c:147,223).  Nothing here is copied from a table: every digit is
computed below and checked (exactness on x^0..x^91, interlacing, positivity).

Usage: python gen_kronrod.py csrc/gk61_table.h ../oracle/kronrod61.h (run from this directory)
"""
import sys
import mpmath as mp

mp.mp.dps = 120
N = 30  # Gauss order


def legendre_coeffs(n):
    """Monomial coefficients (index = power) of P_n, exact rationals via mpf."""
    p0 = [mp.mpf(1)]
    p1 = [mp.mpf(0), mp.mpf(1)]
    if n == 0:
        return p0
    for k in range(1, n):
        # (k+1) P_{k+1} = (2k+1) x P_k - k P_{k-1}
        nxt = [mp.mpf(0)] * (k + 2)
        for i, c in enumerate(p1):
            nxt[i + 1] += (2 * k + 1) * c
        for i, c in enumerate(p0):
            nxt[i] -= k * c
        nxt = [c / (k + 1) for c in nxt]
        p0, p1 = p1, nxt
    return p1


def poly_eval(c, x):
    r = mp.mpf(0)
    for a in reversed(c):
        r = r * x + a
    return r


def poly_deriv(c):
    return [i * c[i] for i in range(1, len(c))]


def moment(m):
    """Integral of x^m over [-1, 1]."""
    return mp.mpf(0) if m % 2 else mp.mpf(2) / (m + 1)


def main(outs):
    P = legendre_coeffs(N)
    dP = poly_deriv(P)
    # Gauss nodes: Newton from Chebyshev-like initial guesses.
    gauss = []
    for i in range(1, N + 1):
        x = mp.cos(mp.pi * (i - mp.mpf(1) / 4) / (N + mp.mpf(1) / 2))
        for _ in range(200):
            dx = poly_eval(P, x) / poly_eval(dP, x)
            x -= dx
            if abs(dx) < mp.mpf(10) ** (-110):
                break
        gauss.append(x)
    gauss = sorted(gauss, reverse=True)
    gw = [2 / ((1 - x * x) * poly_eval(dP, x) ** 2) for x in gauss]

    # Stieltjes polynomial E = x^31 + sum_{i<31} a_i x^i with
    # integral E(x) P_30(x) x^k dx = 0, k = 0..30.  Only odd powers survive
    # (E_31 is odd), which keeps the linear system well posed.
    odd_pows = [p for p in range(0, 31) if p % 2 == 1]
    rows, rhs = [], []
    for k in range(0, 31):
        # integral x^(p+k) P(x) dx = sum_j P_j moment(p+k+j)
        def ip(p):
            return mp.fsum(P[j] * moment(p + k + j) for j in range(len(P)))
        row = [ip(p) for p in odd_pows]
        val = -ip(31)
        if all(abs(r) < mp.mpf(10) ** (-100) for r in row) and abs(val) < mp.mpf(10) ** (-100):
            continue  # parity makes half of the conditions trivially zero
        rows.append(row)
        rhs.append(val)
    A = mp.matrix(rows)
    b = mp.matrix(rhs)
    sol = mp.lu_solve(A, b)
    E = [mp.mpf(0)] * 32
    E[31] = mp.mpf(1)
    for p, a in zip(odd_pows, sol):
        E[p] = a
    dE = poly_deriv(E)
    # Kronrod nodes interlace the Gauss nodes: one in each gap and one beyond each end.
    brackets = [mp.mpf(1)] + gauss + [mp.mpf(-1)]
    kron = []
    for lo_i in range(len(brackets) - 1):
        hi, lo = brackets[lo_i], brackets[lo_i + 1]
        # bisection + Newton polish (robust, no reliance on solver heuristics)
        a, bb = lo, hi
        fa = poly_eval(E, a)
        for _ in range(400):
            m = (a + bb) / 2
            fm = poly_eval(E, m)
            if (fm < 0) == (fa < 0):
                a, fa = m, fm
            else:
                bb = m
            if bb - a < mp.mpf(10) ** (-60):
                break
        x = (a + bb) / 2
        for _ in range(20):
            x -= poly_eval(E, x) / poly_eval(dE, x)
        kron.append(x)
    assert len(kron) == 31
    allx = sorted(gauss + kron, reverse=True)  # 61 nodes, descending
    assert len(allx) == 61
    # weights from the moment equations with Legendre test functions
    M = mp.matrix(61, 61)
    rhs = mp.matrix(61, 1)
    for j in range(61):
        Pj = legendre_coeffs(j)
        for i, x in enumerate(allx):
            M[j, i] = poly_eval(Pj, x)
        rhs[j] = 2 if j == 0 else 0
    w = mp.lu_solve(M, rhs)
    w = [w[i] for i in range(61)]
    # checks: exactness for monomials up to degree 91, positivity, symmetry
    for d in range(0, 92):
        s = mp.fsum(wi * xi ** d for wi, xi in zip(w, allx))
        assert abs(s - moment(d)) < mp.mpf(10) ** (-80), (d, s)
    s93 = mp.fsum(wi * xi ** 92 for wi, xi in zip(w, allx))
    assert abs(s93 - moment(92)) > mp.mpf(10) ** (-40)  # degree 92 is not exact
    assert all(wi > 0 for wi in w)
    for i in range(30):
        assert abs(allx[i] + allx[60 - i]) < mp.mpf(10) ** (-90)
        assert abs(w[i] - w[60 - i]) < mp.mpf(10) ** (-90)
    # Positive half, descending: xk[0..29] > 0, xk[30] = 0 (centre).
    xk = allx[:31]
    wk = w[:31]
    gauss_set = set(mp.nstr(x, 60) for x in gauss)
    is_gauss = [1 if mp.nstr(x, 60) in gauss_set else 0 for x in xk]
    assert sum(is_gauss) == 15 and is_gauss[30] == 0
    wg_for = []
    for x, flag in zip(xk, is_gauss):
        if flag:
            idx = [mp.nstr(g, 60) for g in gauss].index(mp.nstr(x, 60))
            wg_for.append(gw[idx])
        else:
            wg_for.append(mp.mpf(0))
    # Gauss rule exactness (degree 59)
    for d in range(0, 60, 2):
        s = mp.fsum(gw[i] * gauss[i] ** d for i in range(N))
        assert abs(s - moment(d)) < mp.mpf(10) ** (-80)

    lines = []
    lines.append("/* Generated by kspace-neutrinos_gb300/gen_kronrod.py: 61-point Gauss-Kronrod rule on [-1,1],")
    lines.append(" * computed from the Kronrod construction in 120-digit arithmetic (see the script).")
    lines.append(" * KSP_GK61_XK[i]: i=0..29 positive nodes in descending order, i=30 the centre (0).")
    lines.append(" * KSP_GK61_WK[i]: Kronrod weight of +/-XK[i]; KSP_GK61_WG[i]: weight of the embedded")
    lines.append(" * 30-point Gauss rule at +/-XK[i] (0 where XK[i] is a Kronrod-only node). */")
    lines.append("#ifndef KSP_GK61_TABLE_H")
    lines.append("#define KSP_GK61_TABLE_H")
    lines.append("#define KSP_GK61_NHALF 30")
    for name, arr in (("KSP_GK61_XK", xk), ("KSP_GK61_WK", wk), ("KSP_GK61_WG", wg_for)):
        lines.append("#define %s_INIT { \\" % name)
        for i, v in enumerate(arr):
            sep = "," if i < 30 else ""
            lines.append("    %s%s \\" % (mp.nstr(v, 22, strip_zeros=False) if v != 0 else "0.0", sep))
        lines.append("}")
    lines.append("#endif")
    text = "\n".join(lines) + "\n"
    for o in outs:
        with open(o, "w") as f:
            f.write(text)


if __name__ == "__main__":
    main(sys.argv[1:] or ["kronrod61.h"])
