"""The tabulated J(x) of kspace-neutrinos_gb300/csrc/jfit_table.h (used by the GPU
integrand) against the fitting formula of delta_tot_table.c:417-428 in 40-digit
arithmetic, with the same piece selection (octave and top mantissa bits) as
ksp_jfit.cuh."""
import os
import re
import struct

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "kspace-neutrinos_gb300", "csrc", "jfit_table.h")


def load():
    text = open(HDR).read()
    macros = dict(re.findall(r"#define (KSP_JFIT_\w+) \(?(-?\d+)\)?\n", text))
    body = text[text.index("KSP_JFIT_TABLE_INIT {") + len("KSP_JFIT_TABLE_INIT {"):text.rindex("}")]
    vals = np.array([float(v) for v in re.findall(r"[-+0-9.eE]+", body.replace("\\", " "))])
    m = {k: int(v) for k, v in macros.items()}
    return m, vals.reshape(m["KSP_JFIT_PIECES"], m["KSP_JFIT_STRIDE"])


def J_exact(x):
    mp.mp.dps = 40
    x = mp.mpf(x)
    x2 = x * x
    return (1 + mp.mpf("0.0168") * x2 + mp.mpf("0.0407") * x2 * x2) / (
        1 + mp.mpf("2.1734") * x2 + mp.mpf("1.6787") * mp.e ** (mp.mpf("4.1811") * mp.log(x)) +
        mp.mpf("0.1467") * x2 ** 4)


def J_tab(x, m, T):
    bits = struct.unpack("<q", struct.pack("<d", x))[0]
    e = ((bits >> 52) & 0x7ff) - 1023
    assert m["KSP_JFIT_E0"] <= e < m["KSP_JFIT_E1"]
    sb = m["KSP_JFIT_SUB_BITS"]
    sub = (bits >> (52 - sb)) & ((1 << sb) - 1)
    p = T[((e - m["KSP_JFIT_E0"]) << sb) | sub]
    t = x - p[0]  # coefficients of the polynomial in x - centre
    v = 0.0
    for c in reversed(p[1:]):
        v = v * t + c
    return v


def test_table_matches_formula():
    m, T = load()
    rng = np.random.default_rng(0)
    xs = np.exp(rng.uniform(np.log(2.0 ** m["KSP_JFIT_E0"]), np.log(2.0 ** m["KSP_JFIT_E1"]), 3000))
    # piece edges and their neighbours
    nsub = 1 << m["KSP_JFIT_SUB_BITS"]
    edges = [2.0 ** e * (1 + s / nsub) for e in range(m["KSP_JFIT_E0"], m["KSP_JFIT_E1"]) for s in range(0, nsub, 5)]
    worst = 0.0
    for x in list(xs) + edges + [np.nextafter(x, 0) for x in edges[1:]]:
        ex = J_exact(x)
        worst = max(worst, abs(float((J_tab(float(x), m, T) - ex) / ex)))
    assert worst < 5e-16, worst
