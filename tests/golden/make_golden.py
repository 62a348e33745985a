#!/usr/bin/env python3
"""Generate the golden fixtures in this directory by running the reference C itself
(oracle/_ref/libkspace_ref.so, built from the reference sources) on
  * the reference test suite's own inputs (testdata/, camb_linear/), reproducing the
    sequences of delta_tot_table_test.c (test_delta_tot_init, test_get_delta_nu_update,
    test_reproduce_linear), delta_pow_test.c and transfer_init_test.c;
  * a small synthetic end-to-end add_nu_power_to_rhogrid through the reference's global
    interface (interface_common.c / interface_gadget.c).
Only this script reads the reference tree; the fixtures (.npz) travel with the tests.

    python tests/golden/make_golden.py [/path/to/reference]
"""
import ctypes as C
import math
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, os.path.join(ROOT, "kspace-neutrinos_gb300"))
from oracle_lib import RefLib, _p, build_oracle  # noqa: E402
import workloads as W  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
KPC = 3.085678e21
UT_KPC = KPC / 1e5


def read_powerspec(path, with_k=True):
    with open(path) as f:
        toks = f.read().split()
    scale = float(toks[0])
    n = int(toks[1])
    vals = np.array([float(t) for t in toks[2:]])
    if with_k:
        vals = vals.reshape(n, 2)
    return scale, n, vals


def testdata_fixture(R):
    """delta_tot_table_test.c:368-455 set-up, then :127-152 and :193-228."""
    _, n, nu = read_powerspec(os.path.join(REF, "testdata/powerspec_nu_004.txt"))
    logkk = nu[:, 0].copy()          # k, not log k (the test keeps k)
    dnu_file = np.sqrt(nu[:, 1])
    _, n2, cdm = read_powerspec(os.path.join(REF, "testdata/powerspec_cdm_004.txt"), with_k=False)
    assert n2 == n
    MNu = np.array([0.15, 0.15, 0.15])
    om = R.omnu(MNu, 0.01, 0.7)
    OmegaNua3 = R.L.ref_get_omega_nu(om, 0.01) * 0.01 ** 3
    OmegaMa = 0.2793 - R.L.ref_get_omega_nu(om, 1) + OmegaNua3
    fnu = OmegaNua3 / OmegaMa
    dcdm = (cdm - fnu * dnu_file) / (1. - fnu)
    tr = R.L.ref_transfer_new()
    st = R.L.ref_transfer_read(tr, 512000, KPC, KPC * 1e3, os.path.join(REF, "testdata/ics_transfer_99.dat").encode())
    assert st == 0
    nt = R.L.ref_transfer_get(tr, None, None)
    t_logk = np.zeros(nt)
    t_T = np.zeros(nt)
    R.L.ref_transfer_get(tr, _p(t_logk), _p(t_T))
    R.L.ref_set_hubble(om, 0.2793, 1 - 0.2793, UT_KPC, 1)
    out = {"MNu": MNu, "keff": logkk, "dnu_file": dnu_file, "dcdm": dcdm, "t_logk": t_logk, "t_T": t_T}
    # test_delta_tot_init (fresh start at a=0.01)
    d = R.L.ref_dtot_new()
    assert R.L.ref_allocate_delta_tot_table(d, n, 0.01, 1, 0.2793, om, UT_KPC, KPC) == 0
    assert R.L.ref_delta_tot_init(d, n, _p(logkk), _p(dcdm), tr, 0.01) == 0
    s = R.dtot_state(d)
    out["init_fresh_nu_init"] = s["nu_init"][:n].copy()
    out["init_fresh_nu_last"] = s["nu_last"][:n].copy()
    out["init_fresh_row0"] = s["delta_tot"][:n, 0].copy()
    R.L.ref_dtot_free(d)
    # the saved table (read_all_nu_state) and test_get_delta_nu_update
    d = R.L.ref_dtot_new()
    assert R.L.ref_allocate_delta_tot_table(d, n, 0.01, 1, 0.2793, om, UT_KPC, KPC) == 0
    tmp = tempfile.mkdtemp()
    src = os.path.join(REF, "testdata/delta_tot_nu.txt")
    assert R.L.ref_read_all_nu_state(d, src.encode()) == 0
    s = R.dtot_state(d)
    ia = s["ia"]
    out["table_scalefact"] = s["scalefact"][:ia].copy()
    out["table"] = s["delta_tot"][:n, :ia].copy()
    assert R.L.ref_delta_tot_init(d, n, _p(logkk), _p(dcdm), tr, 0.33333333) == 0
    s = R.dtot_state(d)
    out["resume_nu_init"] = s["nu_init"][:n].copy()
    out["resume_nu_last"] = s["nu_last"][:n].copy()
    dnu = np.zeros(n)
    assert R.L.ref_get_delta_nu_update(d, 0.33333333, n, _p(logkk), _p(dcdm), _p(dnu), tr) == 0
    out["update1_dnu"] = dnu.copy()
    out["update1_ia"] = np.array(R.dtot_state(d)["ia"])
    R.L.ref_dtot_set_ia(d, R.dtot_state(d)["ia"] - 1)
    assert R.L.ref_get_delta_nu_update(d, 0.33333333, n, _p(logkk), _p(dcdm), _p(dnu), tr) == 0
    out["update2_dnu"] = dnu.copy()
    out["update2_ia"] = np.array(R.dtot_state(d)["ia"])
    R.L.ref_dtot_free(d)
    # delta_pow_test.c:47-111: ratio table and interpolated values
    lk = np.log(logkk)
    ratio = dnu_file / cdm
    dp = R.L.ref_dpow_new()
    assert R.L.ref_init_delta_pow(dp, _p(lk), _p(ratio), n, 1.0) == 0
    qs = np.concatenate([lk[::5][:10], (lk[1:-1:5][:50] + lk[2::5][:50]) / 2, [lk[0] - 0.01, lk[-1] + 0.01]])
    vals = np.zeros(len(qs))
    for i, q in enumerate(qs):
        v = C.c_double()
        assert R.L.ref_get_dnudcdm_powerspec(dp, q, C.byref(v)) == 0
        vals[i] = v.value
    out["dpow_logk"] = lk
    out["dpow_ratio"] = ratio
    out["dpow_query"] = qs
    out["dpow_value"] = vals
    return out


def camb_fixture(R):
    """delta_tot_table_test.c:315-363 (99 steps driven by CAMB delta_cdm)."""
    NREAD = 200

    def load(tfile, mfile, kmin):
        dc, dn, ks = [], [], []
        with open(tfile) as f:
            for line in f:
                if line.startswith("#"):
                    continue
                v = line.split()
                if len(v) < 8:
                    break
                k, T_nu, T_tot, T_cdm = float(v[0]), float(v[5]), float(v[6]), float(v[7])
                if k > kmin:
                    dc.append((T_cdm / T_tot) ** 2)
                    dn.append((T_nu / T_tot) ** 2)
                if len(dc) == NREAD:
                    break
        c = 0
        with open(mfile) as f:
            for line in f:
                if line.startswith("#"):
                    continue
                v = line.split()
                k, Pk = float(v[0]), float(v[1])
                if k > kmin:
                    dc[c] = math.sqrt(dc[c] * Pk * 1000.0 ** 3)
                    dn[c] = math.sqrt(dn[c] * Pk * 1000.0 ** 3)
                    ks.append(k / 1000.0)
                    c += 1
                if c == NREAD:
                    break
        return np.array(dc), np.array(dn), np.array(ks)

    MNu = np.array([0.15, 0.15, 0.15])
    om = R.omnu(MNu, 0.01, 0.7)
    R.L.ref_set_hubble(om, 0.2793, 1 - 0.2793, UT_KPC, 1)
    tr = R.L.ref_transfer_new()
    cl = os.path.join(REF, "camb_linear")
    assert R.L.ref_transfer_read(tr, 512000, KPC, KPC * 1e3, os.path.join(cl, "ics_transfer_0.01.dat").encode()) == 0
    nt = R.L.ref_transfer_get(tr, None, None)
    t_logk = np.zeros(nt)
    t_T = np.zeros(nt)
    R.L.ref_transfer_get(tr, _p(t_logk), _p(t_T))
    kmin = 2 * math.pi / 512.
    dc0, dn0, ks0 = load(os.path.join(cl, "ics_transfer_0.01.dat"), os.path.join(cl, "ics_matterpow_0.01.dat"), kmin)
    d = R.L.ref_dtot_new()
    assert R.L.ref_allocate_delta_tot_table(d, NREAD, 0.01, 1, 0.2793, om, UT_KPC, KPC) == 0
    assert R.L.ref_delta_tot_init(d, NREAD, _p(ks0), _p(dc0), tr, 0.01) == 0
    steps = []
    for i in range(99):
        a = 0.01 + i * 0.01
        name = "%g" % a
        dc, dn, ks = load(os.path.join(cl, "ics_transfer_%s.dat" % name), os.path.join(cl, "ics_matterpow_%s.dat" % name),
                          kmin)
        out = np.zeros(NREAD)
        assert R.L.ref_get_delta_nu_update(d, a, NREAD, _p(ks), _p(dc), _p(out), tr) == 0
        steps.append((a, ks, dc, dn, out.copy(), R.dtot_state(d)["ia"]))
    return {"MNu": MNu, "t_logk": t_logk, "t_T": t_T, "k0": ks0, "dcdm0": dc0,
            "a": np.array([s[0] for s in steps]), "keff": np.array([s[1] for s in steps]),
            "dcdm": np.array([s[2] for s in steps]), "dnu_camb": np.array([s[3] for s in steps]),
            "dnu_ref": np.array([s[4] for s in steps]), "ia": np.array([s[5] for s in steps])}


def e2e_fixture(R):
    """add_nu_power_to_rhogrid through the reference's global interface on a 16^3 grid."""
    N, L = 16, 512.0
    MNu = np.array([0.1, 0.1, 0.1])
    nb = 16
    count, keff_grid = W.geometry(N, nb)
    m = count > 0
    kphys = keff_grid[m] * 2 * math.pi / L
    Na = 8
    sf, dt = W.history(kphys, Na, 0.5)
    logk, T = W.transfer_table(0.3)
    tmp = tempfile.mkdtemp()
    tf = os.path.join(tmp, "transfer.dat")
    with open(tf, "w") as f:  # CAMB column layout read by transfer_init.c:34,65
        for lk_, t_ in zip(logk, T):
            f.write("%.17g 1 1 1 1 %.17g 1 1\n" % (math.exp(lk_), t_))
    R.L.ref_set_kspace_params(tf.encode(), 0.01, W.UNIT_LENGTH_MPC, _p(MNu), 0, 0.0, 0.0)
    assert R.L.ref_InitOmegaNu(0.7, 2.7255) == 0
    R.L.ref_set_hubble_global(0.3, 0.7, W.UNIT_TIME, 1, 0.7, 2.7255)
    TimeMax = 0.01 + (Na + 12) / 100.0
    assert R.L.ref_allocate_kspace_memory(nb, L, W.UNIT_TIME, W.UNIT_LENGTH_MPC, 0.3, None, TimeMax) == 0
    flat = np.ascontiguousarray(dt)
    assert R.L.ref_set_nu_state(_p(sf), _p(flat), flat.shape[0], flat.shape[1]) == 0
    g0 = W.make_grid(N, L, seed=7)
    g = g0.copy()
    outs = []
    for a in (0.51, 0.512, 0.52):
        assert R.L.ref_add_nu_power_to_rhogrid(a, L, g.ctypes.data, N, 0, N) == 0
        outs.append(g.copy())
    sfo = np.zeros(64)
    dto = np.zeros(64 * 64)
    return {"N": np.array(N), "L": np.array(L), "nbins": np.array(nb), "MNu": MNu, "scalefact": sf, "delta_tot": dt,
            "t_logk": logk, "t_T": T, "TimeMax": np.array(TimeMax), "grid0": g0, "a": np.array([0.51, 0.512, 0.52]),
            "grids": np.array(outs), "kphys": kphys}


def main():
    build_oracle()
    R = RefLib()
    np.savez_compressed(os.path.join(HERE, "ref_testdata.npz"), **testdata_fixture(R))
    np.savez_compressed(os.path.join(HERE, "ref_camb_linear.npz"), **camb_fixture(R))
    np.savez_compressed(os.path.join(HERE, "ref_e2e_n16.npz"), **e2e_fixture(R))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
