"""The reference-named drop-in interface, driven from C by a minimal PM loop
(tests/dropin/pm_harness.c), against the oracle running the same sequence."""
import math
import os
import subprocess

import numpy as np
import pytest

import cases
import workloads as W

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def write_transfer(path, logk, T):
    with open(path, "w") as f:  # CAMB columns: k T_cdm T_b T_g T_rnu T_nu T_tot T_nonu
        for lk, t in zip(logk, T):
            f.write("%.17g 1 1 1 1 %.17g 1 1\n" % (math.exp(lk), t))


def write_state(path, sf, dt):
    with open(path, "w") as f:  # delta_tot_table.c:320-324
        for i in range(len(sf)):
            f.write("# %.17e " % sf[i] + " ".join("%.17e" % v for v in dt[:, i]) + " \n")


def test_pm_harness_matches_oracle(gpu, oracle, tmp_path):
    N, nb, L = 32, 32, 512.0
    c = cases.make_case(N, nb, 10, 0.5, (0.1, 0.1, 0.1))
    exe = str(tmp_path / "pm_harness")
    pkg = os.path.join(ROOT, "kspace-neutrinos_gb300")
    subprocess.run(["gcc", "-O2", "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "oracle", "shim"),
                    "-o", exe, os.path.join(ROOT, "tests", "dropin", "pm_harness.c"),
                    os.path.join(pkg, "dropin", "kspace_dropin.c"),
                    os.path.join(pkg, "dropin", "kspace_delta_tot_table.c"), "-L" + pkg, "-lkspace_gb300",
                    "-Wl,-rpath," + pkg, "-lm"], check=True)
    tf = str(tmp_path / "transfer.dat")
    sf_path = str(tmp_path / "state.txt")
    write_transfer(tf, c["logk"], c["T"])
    write_state(sf_path, c["scalefact"], c["delta_tot"])
    gin, gout = str(tmp_path / "g.in"), str(tmp_path / "g.out")
    c["grid"].tofile(gin)
    avals = ["0.51", "0.512", "0.52"]
    r = subprocess.run([exe, tf, sf_path, gin, gout, str(tmp_path), str(N), str(nb), str(L), str(c["TimeMax"])] + avals,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.fromfile(gout, dtype=np.complex64).reshape(c["grid"].shape)
    # the oracle on the same inputs (state read with the file's rounding)
    rows = [l.split() for l in open(sf_path)]
    sf = np.array([float(r[1]) for r in rows])
    dt = np.array([[float(v) for v in r[2:]] for r in rows]).T
    bg = oracle.bg((0.1, 0.1, 0.1), Omega0=0.3, UnitTime_in_s=W.UNIT_TIME)
    s = oracle.state(bg, nb, 0.01, c["TimeMax"], Omega0=0.3, UnitTime_in_s=W.UNIT_TIME,
                     UnitLength_in_cm=W.UNIT_LENGTH_MPC)
    oracle.set_transfer(s, c["logk"], c["T"])
    oracle.set_nu_state(s, sf, dt)
    g = c["grid"].copy()
    for a in avals:
        st, out = oracle.add_nu_power_to_rhogrid(s, float(a), L, g, N)
        assert st == 0
    rel = np.abs(got - g) / np.maximum(np.abs(g), 1e-30)
    assert rel.max() < 1e-6, rel.max()
    # snapshot files: state rows and P_nu
    so = oracle.get_state(s)
    saved = [l.split() for l in open(tmp_path / "delta_tot_nu.txt")]
    assert len(saved) == so["ia"]
    last = np.array([float(v) for v in saved[-1][2:]])
    assert cases.rel_err(last, so["delta_tot"][:c["nk"], so["ia"] - 1]) < 1e-6  # printed with %le
    pn = np.loadtxt(tmp_path / "powerspec_nu_001.txt")
    assert pn.shape == (c["nk"], 2)
    assert cases.rel_err(pn[:, 1], so["nu_last"][:c["nk"]] ** 2) < 1e-5  # printed with %g
    assert os.path.exists(tmp_path / "powerspec_tot_001.txt")
