#!/usr/bin/env python3
"""Generate the golden fixtures in this directory by running the reference C itself
(oracle/_ref/libkspace_ref.so, built from the reference sources) on
  * the reference test suite's own inputs (testdata/, camb_linear/), reproducing the
    sequences of delta_tot_table_test.c (test_delta_tot_init, test_get_delta_nu_update,
    test_reproduce_linear), delta_pow_test.c and transfer_init_test.c;
  * a small synthetic end-to-end add_nu_power_to_rhogrid through the reference's global
    interface (interface_common.c / interface_gadget.c).
Only this script reads the reference tree; the fixtures (.npz) travel with the tests.

    python tests/golden/make_golden.py /path/to/reference-sources
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
from oracle_lib import REF_NU2_SO, REF_SO, RefLib, _p, build_oracle  # noqa: E402
import workloads as W  # noqa: E402

if len(sys.argv) < 2 or not os.path.isfile(os.path.join(sys.argv[1], "delta_tot_table.c")):
    sys.exit("usage: make_golden.py /path/to/reference-sources (the kspace-neutrinos source tree)")
REF = sys.argv[1]
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
    # get_delta_nu per mass and get_delta_nu_combined on the resumed rows, at the last
    # stored time (beyond it the reference's spline is out of range)
    a_last = math.exp(s["scalefact"][s["ia"] - 1])
    out["resume_a_last"] = np.array(a_last)
    for tag, m in (("m015", 0.15), ("m005", 0.05)):
        v = np.zeros(n)
        assert R.L.ref_get_delta_nu(d, a_last, _p(logkk), _p(v), m) == 0
        out["resume_getdnu_" + tag] = v
    v = np.zeros(n)
    assert R.L.ref_get_delta_nu_combined(d, a_last, _p(logkk), _p(v)) == 0
    out["resume_getdnu_combined"] = v
    dnu = np.zeros(n)
    assert R.L.ref_get_delta_nu_update(d, 0.33333333, n, _p(logkk), _p(dcdm), _p(dnu), tr) == 0
    out["update1_dnu"] = dnu.copy()
    out["update1_ia"] = np.array(R.dtot_state(d)["ia"])
    R.L.ref_dtot_set_ia(d, R.dtot_state(d)["ia"] - 1)
    assert R.L.ref_get_delta_nu_update(d, 0.33333333, n, _p(logkk), _p(dcdm), _p(dnu), tr) == 0
    out["update2_dnu"] = dnu.copy()
    out["update2_ia"] = np.array(R.dtot_state(d)["ia"])
    # update_delta_tot: a new row at a = 0.345, then that row overwritten at a = 0.35
    dnu_u = dnu * 1.01
    assert R.L.ref_update_delta_tot(d, 0.345, _p(dcdm), _p(dnu_u), 0) == 0
    st_ = R.dtot_state(d)
    out["update_new_ia"] = np.array(st_["ia"])
    out["update_new_row"] = st_["delta_tot"][:n, st_["ia"] - 1].copy()
    assert R.L.ref_update_delta_tot(d, 0.35, _p(dcdm * 1.02), _p(dnu_u), 1) == 0
    st_ = R.dtot_state(d)
    out["update_over_ia"] = np.array(st_["ia"])
    out["update_over_row"] = st_["delta_tot"][:n, st_["ia"] - 1].copy()
    out["update_over_loga"] = np.array(st_["scalefact"][st_["ia"] - 1])
    R.L.ref_dtot_free(d)
    # test_allocate_delta_tot_table (delta_tot_table_test.c:57-80): massless neutrinos, a
    # table in other units (UnitTime = UnitLength = 1), the host H(a) unchanged
    om0 = R.omnu(np.zeros(3), 0.01, 0.7)
    d = R.L.ref_dtot_new()
    assert R.L.ref_allocate_delta_tot_table(d, 300, 0.01, 1, 0.2793, om0, 1.0, 1.0) == 0
    dnu0 = np.zeros(n)
    assert R.L.ref_get_delta_nu_update(d, 0.02, n, _p(logkk), _p(dcdm), _p(dnu0), tr) == 0
    out["massless_dnu"] = dnu0
    out["massless_ia"] = np.array(R.dtot_state(d)["ia"])
    R.L.ref_dtot_free(d)
    # specialJ (fit and truncated series), nufrac_low, fslength (test host H(a))
    xs = np.concatenate([[0.0, 1e-3, 0.1, 0.3, 0.5, 1, 2, 5, 20, 100]])
    out["sj_x"] = xs
    sj = []
    for qc, nfl in ((-1.0, 0.0), (1e-2, 0.5), (0.5, 0.2), (1.0, 0.5), (3.0, 0.1)):
        sj.append([qc, nfl] + [R.L.ref_specialJ(x, qc, nfl) for x in xs])
    out["sj_table"] = np.array(sj)
    qcs = np.array([0.0, 0.1, 0.5, 1.0, 2.0, 3.0, 10.0])
    nf = []
    for q in qcs:
        v = C.c_double()
        assert R.L.ref_nufrac_low(q, C.byref(v)) == 0
        nf.append(v.value)
    out["nufrac_qc"] = qcs
    out["nufrac_val"] = np.array(nf)
    iv = np.array([[math.log(0.5), 0.0], [math.log(0.1), math.log(0.5)], [math.log(0.01), math.log(0.3)],
                   [math.log(0.02), math.log(0.021)], [0.0, -1.0]])
    fs = []
    for lo_, hi_ in iv:
        v = C.c_double()
        assert R.L.ref_fslength(lo_, hi_, 299792., C.byref(v)) == 0
        fs.append(v.value)
    out["fsl_intervals"] = iv
    out["fsl_val"] = np.array(fs)
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


def _write_transfer(path, logk, T):
    with open(path, "w") as f:  # CAMB column layout read by transfer_init.c:34,65
        for lk_, t_ in zip(logk, T):
            f.write("%.17g 1 1 1 1 %.17g 1 1\n" % (math.exp(lk_), t_))


def _read(path):
    with open(path) as f:
        return f.read()


def _global_setup(R, MNu, nb, L, Na, a_end, hybrid=(0, 0.0, 0.0), extra_rows=12):
    """kspace_params, InitOmegaNu, allocate_kspace_memory and a synthetic history through
    the reference's global interface (interface_common.c:77-102,166-188)."""
    count, keff_grid = W.geometry(16, nb)
    m = count > 0
    kphys = keff_grid[m] * 2 * math.pi / L
    sf, dt = W.history(kphys, Na, a_end)
    logk, T = W.transfer_table(float(sum(MNu)))
    tmp = tempfile.mkdtemp()
    tf = os.path.join(tmp, "transfer.dat")
    _write_transfer(tf, logk, T)
    R.L.ref_set_kspace_params(tf.encode(), 0.01, W.UNIT_LENGTH_MPC, _p(np.asarray(MNu, np.float64)), hybrid[0],
                              hybrid[1], hybrid[2])
    assert R.L.ref_InitOmegaNu(0.7, 2.7255) == 0
    R.L.ref_set_hubble_global(0.3, 0.7, W.UNIT_TIME, 1, 0.7, 2.7255)
    TimeMax = 0.01 + (Na + extra_rows) / 100.0
    assert R.L.ref_allocate_kspace_memory(nb, L, W.UNIT_TIME, W.UNIT_LENGTH_MPC, 0.3, None, TimeMax) == 0
    flat = np.ascontiguousarray(dt)
    assert R.L.ref_set_nu_state(_p(sf), _p(flat), flat.shape[0], flat.shape[1]) == 0
    return dict(count=count, keff_grid=keff_grid, kphys=kphys, scalefact=sf, delta_tot=dt, t_logk=logk, t_T=T,
                TimeMax=np.array(TimeMax), tmp=tmp)


def _power_from_cdm(R, st, L, a_end, times):
    """compute_neutrino_power_from_cdm (interface_common.c:106-123) on all nb bins, the
    empty ones (Nmodes = 0) included, with P_cdm = P(k) (a/a_end)^2."""
    count = st["count"]
    nb = len(count)
    kin = st["keff_grid"] * 2 * math.pi / L
    P0 = W.spectrum(np.where(count > 0, kin, 0.05))
    Nmodes = count.astype(np.int64)
    out = {"pc_keff_in": kin, "pc_nmodes": Nmodes, "pc_times": np.array(times)}
    lk, ra, nr, nbo, ia = [], [], [], [], []
    for a in times:
        P = P0 * (a / a_end) ** 2
        logk = np.zeros(nb)
        ratio = np.zeros(nb)
        norm = C.c_double()
        n = C.c_int()
        assert R.L.ref_compute_neutrino_power_from_cdm(a, _p(kin), _p(P), Nmodes.ctypes.data_as(C.POINTER(C.c_long)),
                                                       nb, _p(logk), _p(ratio), C.byref(norm), C.byref(n)) == 0
        lk.append(logk)
        ra.append(ratio)
        nr.append(norm.value)
        nbo.append(n.value)
        ia.append(R.dtot_state(R.L.ref_global_dtot())["ia"])
    out.update(pc_logk=np.array(lk), pc_ratio=np.array(ra), pc_norm=np.array(nr), pc_nbins=np.array(nbo),
               pc_ia=np.array(ia))
    return out


def interface_fixture():
    """MP-Gadget-style entry (compute_neutrino_power_from_cdm) through the global
    interface, then the snapshot writers: save_neutrino_power (delta_tot_table.c:356-374
    via interface_common.c:41-52) and save_nu_state twice, the second renaming the first
    file to .bak (delta_tot_table.c:327-352)."""
    R = RefLib(REF_NU2_SO)
    MNu, nb, L, Na, a_end = (0.1, 0.1, 0.1), 16, 512.0, 8, 0.5
    st = _global_setup(R, MNu, nb, L, Na, a_end)
    out = {"MNu": np.array(MNu), "nbins": np.array(nb), "L": np.array(L), "Na": np.array(Na), "a_end": np.array(a_end)}
    out.update({k: v for k, v in st.items() if k != "tmp"})
    out.update(_power_from_cdm(R, st, L, a_end, [0.51, 0.512, 0.53]))
    d = st["tmp"]
    ret = C.c_int()
    assert R.L.ref_save_neutrino_power(0.53, 3, d.encode(), C.byref(ret)) == 0 and ret.value == 0
    out["save_nu_power_txt"] = np.array(_read(os.path.join(d, "powerspec_nu_003.txt")))
    sfile = os.path.join(d, "delta_tot_nu.txt")
    assert R.L.ref_save_nu_state(sfile.encode()) == 0
    first = _read(sfile)
    more = _power_from_cdm(R, st, L, a_end, [0.55])
    out.update({"second_" + k: v for k, v in more.items()})
    assert R.L.ref_save_nu_state(sfile.encode()) == 0
    out["save_state_txt"] = np.array(_read(sfile))
    out["save_state_bak_txt"] = np.array(_read(sfile + ".bak"))
    assert out["save_state_bak_txt"] == np.array(first)
    return out


def hybrid_fixture():
    """Hybrid neutrinos (omega_nu_single.c:214-279; specialJ's truncated series,
    delta_tot_table.c:431-463, and the particle fraction and looser tolerance of
    get_delta_nu, :539-548) through the global interface."""
    R = RefLib(REF_NU2_SO)
    MNu, nb, L, Na, a_end = (0.15, 0.15, 0.15), 16, 512.0, 8, 0.5
    vcrit, nu_crit_time = 1000.0, 0.3
    st = _global_setup(R, MNu, nb, L, Na, a_end, hybrid=(1, vcrit, nu_crit_time))
    out = {"MNu": np.array(MNu), "nbins": np.array(nb), "L": np.array(L), "Na": np.array(Na), "a_end": np.array(a_end),
           "vcrit": np.array(vcrit), "nu_crit_time": np.array(nu_crit_time)}
    out.update({k: v for k, v in st.items() if k != "tmp"})
    av = np.array([0.02, 0.1, 0.29, 0.299999, 0.300001, 0.31, 0.5, 0.51, 0.8, 1.0])
    out["bg_a"] = av
    out["bg_omega_nu"] = np.array([R.L.ref_OmegaNu(a) for a in av])
    out["bg_omega_nu_nopart"] = np.array([R.L.ref_OmegaNu_nopart(a) for a in av])
    out["bg_particle_active"] = np.array([R.L.ref_particle_nu_active(a) for a in av])
    out.update(_power_from_cdm(R, st, L, a_end, [0.51, 0.512, 0.53]))
    return out


def gadget_saves_fixture():
    """add_nu_power_to_rhogrid on a 16^3 grid (library built for a Gadget-2 neutrino run,
    -DKSPACE_NEUTRINOS_2), then save_total_power (interface_gadget.c:196-224, the
    get_delta_tot branch) and save_neutrino_power."""
    R = RefLib(REF_NU2_SO)
    MNu, nb, L, Na, a_end = (0.1, 0.1, 0.1), 16, 512.0, 8, 0.5
    st = _global_setup(R, MNu, nb, L, Na, a_end)
    out = {"MNu": np.array(MNu), "nbins": np.array(nb), "L": np.array(L), "Na": np.array(Na), "a_end": np.array(a_end)}
    out.update({k: v for k, v in st.items() if k != "tmp"})
    g0 = W.make_grid(16, L, seed=11)
    g = g0.copy()
    av = [0.51, 0.512, 0.52]
    grids = []
    for a in av:
        assert R.L.ref_add_nu_power_to_rhogrid(a, L, g.ctypes.data, 16, 0, 16) == 0
        grids.append(g.copy())
    d = st["tmp"]
    ret = C.c_int()
    assert R.L.ref_save_total_power(0.52, 2, d.encode(), C.byref(ret)) == 0 and ret.value == 0
    assert R.L.ref_save_neutrino_power(0.52, 2, d.encode(), C.byref(ret)) == 0 and ret.value == 0
    out.update(grid0=g0, a=np.array(av), grids=np.array(grids),
               save_total_txt=np.array(_read(os.path.join(d, "powerspec_tot_002.txt"))),
               save_nu_power_txt=np.array(_read(os.path.join(d, "powerspec_nu_002.txt"))))
    return out


def total_power_fixture(N, seeds=(21, 22), times=(0.4, 0.6)):
    """compute_total_power_spectrum + save_total_power of a run without the integrator
    (interface_gadget.c:114-144,196-224, library built without KSPACE_NEUTRINOS_2, as
    gadget-2 patch 0004 calls it), twice on one N^3 grid size in a fresh process, as a
    simulation calls it at two snapshots.  Its k column is what the reference writes:
    keff and delta_cdm_last share storage there (3/2*pmgrid is pmgrid in integer
    arithmetic, :118-119), so the stored log k is log(delta_cdm * 2 pi / BoxSize)."""
    R = RefLib(REF_SO)
    out = {"N": np.array(N)}
    L = 512.0
    for j, (seed, Time) in enumerate(zip(seeds, times)):
        g = W.make_grid(N, L, seed=seed)
        d = tempfile.mkdtemp()
        assert R.L.ref_compute_total_power_spectrum(Time, L, g.ctypes.data, N, 0, N) == 0
        ret = C.c_int()
        assert R.L.ref_save_total_power(Time, 7, d.encode(), C.byref(ret)) == 0 and ret.value == 0
        out["grid%d" % j] = g
        out["time%d" % j] = np.array(Time)
        out["txt%d" % j] = np.array(_read(os.path.join(d, "powerspec_tot_007.txt")))
    return out


SUBPROCESS_FIXTURES = {
    "ref_interface.npz": interface_fixture,
    "ref_hybrid.npz": hybrid_fixture,
    "ref_gadget_saves_n16.npz": gadget_saves_fixture,
    "ref_total_power_n16.npz": lambda: total_power_fixture(16),
    "ref_total_power_n32.npz": lambda: total_power_fixture(32),
}


def main():
    build_oracle()
    if len(sys.argv) > 3 and sys.argv[2] == "--fixture":
        # the global-interface fixtures each need a fresh process (the reference keeps
        # its state in process globals, interface_common.c:17-26)
        name = sys.argv[3]
        np.savez_compressed(os.path.join(HERE, name), **SUBPROCESS_FIXTURES[name]())
        return
    R = RefLib()
    np.savez_compressed(os.path.join(HERE, "ref_testdata.npz"), **testdata_fixture(R))
    np.savez_compressed(os.path.join(HERE, "ref_camb_linear.npz"), **camb_fixture(R))
    np.savez_compressed(os.path.join(HERE, "ref_e2e_n16.npz"), **e2e_fixture(R))
    import subprocess
    for name in SUBPROCESS_FIXTURES:
        subprocess.run([sys.executable, os.path.abspath(__file__), REF, "--fixture", name], check=True)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
