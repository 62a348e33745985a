"""The 61-point Gauss-Kronrod table (generated from its definition by
kspace-neutrinos_gb300/gen_kronrod.py) integrates polynomials up to degree 91
exactly; the CUDA and oracle copies are identical."""
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def table(path):
    s = open(path).read()

    def arr(n):
        body = re.search(n + r"_INIT \{(.*?)\}", s, re.S).group(1)
        return np.array([float(x) for x in re.findall(r"[-+0-9.eE]+", body.replace("\\", " "))])
    return arr("KSP_GK61_XK"), arr("KSP_GK61_WK"), arr("KSP_GK61_WG")


def test_copies_identical():
    a = open(os.path.join(ROOT, "kspace-neutrinos_gb300", "csrc", "gk61_table.h")).read()
    b = open(os.path.join(ROOT, "oracle", "kronrod61.h")).read()
    assert a == b


def test_exactness():
    xk, wk, wg = table(os.path.join(ROOT, "oracle", "kronrod61.h"))
    x = np.concatenate([-xk[:30], xk[:30], [0.0]])
    w = np.concatenate([wk[:30], wk[:30], [wk[30]]])
    g = np.concatenate([wg[:30], wg[:30], [0.0]])
    from math import fsum
    for d in range(0, 92, 2):
        assert abs(fsum(w * x ** d) - 2.0 / (d + 1)) < 1e-14
    for d in range(0, 60, 2):
        assert abs(fsum(g * x ** d) - 2.0 / (d + 1)) < 1e-14
    gx, gw = np.polynomial.legendre.leggauss(30)
    assert np.allclose(np.sort(x[g > 0]), np.sort(gx), atol=1e-15)
