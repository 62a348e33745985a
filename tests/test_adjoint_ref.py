"""The FP64 reference adjoint (tests/adjoint_ref.py + the oracle's ko_dnu_diff) against
central finite differences of the FP64 reference step (relative step 1e-6)."""
import ctypes as C
import math

import numpy as np
import pytest

import adjoint_ref
import cases
import workloads as W


def build(oracle, N=32, nb=32, Na=14, masses=(0.05, 0.05, 0.05), seed=0):
    c = cases.make_case(N, nb, Na, 0.5, masses, seed=seed)
    bg, s = cases.oracle_state(oracle, c)
    adjoint_ref.bind(oracle)
    # integrator state: delta_nu_init / delta_nu_last from the reference's init path
    dc0 = np.sqrt(W.spectrum(c["kphys"]))
    P = C.POINTER(C.c_double)
    assert oracle.L.ko_delta_tot_init(s, c["nk"], np.ascontiguousarray(c["kphys"]).ctypes.data_as(P),
                                      dc0.ctypes.data_as(P), 0.5) == 0
    st = oracle.get_state(s)
    vec = (st["nu_init"][:c["nk"]].copy(), st["nu_last"][:c["nk"]].copy(), c["kphys"].copy())
    a = 0.51
    ref = adjoint_ref.StepRef(oracle, bg, s, N, nb, c["L"], a, c["count"], c["kphys"], c["scalefact"])
    rng = np.random.default_rng(seed)
    wb = rng.random(c["nk"])
    x = c["grid"].astype(np.complex128)
    return c, ref, vec, x, wb


def test_reference_adjoint_matches_fd(oracle):
    c, ref, vec, x, wb = build(oracle)
    D = c["delta_tot"]
    mJ = np.array(c["MNu"])
    adj = ref.adjoint(x, D, mJ, wb)
    f = adj["f"]
    rng = np.random.default_rng(1)
    # history entries: normwise relative error over the sample (per-entry FD noise at a
    # 1e-6 step is ~1e-8 of the largest entry)
    scale = np.abs(adj["Dbar"]).max()
    errs = []
    for _ in range(16):
        b, j = rng.integers(c["nk"]), rng.integers(D.shape[1])
        fd = ref.fd_history(x, D, mJ, wb, f, b, j)
        errs.append(abs(fd - adj["Dbar"][b, j]))
    assert max(errs) <= 1e-5 * scale, (max(errs), scale)
    # mass
    fd = ref.fd_mass(x, D, mJ, wb, f)
    assert abs(fd / adj["mbar"][0] - 1) < 1e-5
    # grid modes (not the DC)
    xb = adj["xbar"].ravel()
    for _ in range(16):
        idx = int(rng.integers(1, x.size))
        for part in (0, 1):
            v = x.ravel()[idx].real if part == 0 else x.ravel()[idx].imag
            if abs(v) < 1e-30:
                continue
            fd = ref.fd_mode(x, D, mJ, wb, f, idx, part)
            got = xb[idx].real if part == 0 else xb[idx].imag
            assert abs(fd - got) <= 1e-5 * abs(fd), (idx, part, fd, got)
