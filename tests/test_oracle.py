"""The CPU oracle, pinned: the reference test suite's known answers, the golden
fixtures produced by the reference C itself (tests/golden/make_golden.py), and -- where
the reference sources were available to build oracle/_ref -- direct comparison."""
import math
import os

import numpy as np
import pytest

import cases
import workloads as W

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KPC = 3.085678e21
UT_KPC = KPC / 1e5
T_CMB0 = 2.7255


def kT():
    return 8.61734e-5 * (4 / 11.) ** (1 / 3.) * 1.00328 * T_CMB0


# ---------------------------------------------------------------- known answers
def test_specialJ_known_answers(oracle):
    J = oracle.L.ko_specialJ
    # delta_tot_table_test.c:159-169 (Mathematica values)
    assert J(0, -1, 0) == 1
    assert abs(J(1, -1, 0) - 0.2117) < 1e-3
    assert abs(J(2, -1, 0) - 0.0223807) < 1e-3
    assert abs(J(0.5, -1, 0) - 0.614729) < 1e-3
    assert abs(J(0.3, -1, 0) - 0.829763) < 1e-3
    assert abs(J(0, 1, 0) - 0.940437) < 1e-4
    assert abs(J(0.5, 1e-2, 0.5) - 0.614729 / 0.5) < 1e-3
    assert abs(J(0.5, 1, 0.5) - 0.556557 / 0.5) < 1e-4
    assert abs(J(1, 0.1, 0.5) - 0.211662 / 0.5) < 1e-4


def test_fslength_known_answers(oracle):
    import ctypes as C
    # delta_tot_table_test.c:183-191: Omega0=0.2793, h=0.7, kpc units
    bg = oracle.bg((0.15, 0.15, 0.15), Omega0=0.2793, UnitTime_in_s=UT_KPC)
    st = C.c_int(0)
    f1 = oracle.L.ko_fslength(bg, math.log(0.5), math.log(1), 299792., C.byref(st))
    f2 = oracle.L.ko_fslength(bg, math.log(0.1), math.log(0.5), 299792., C.byref(st))
    assert abs(f1 / 1272.92 / (0.45 / kT()) - 1) < 1e-5
    assert abs(f2 / 5427.8 / (0.6 / kT()) - 1) < 1e-5
    oracle.L.ko_bg_free(bg)


def test_omega_nu_known_answers(oracle):
    # omega_nu_single_test.c:37-65,112-169
    bg = oracle.bg((0.5, 0.5, 0.0))
    rhocrit, kb, deg, mnu = oracle.bg_info(bg)
    assert abs(rhocrit - 1.8784e-29 * 0.49) < 5e-5 * rhocrit
    om1 = oracle.L.ko_omega_nu_single(bg, 1, 0)
    assert abs(om1 / 0.5 ** 3 - oracle.L.ko_omega_nu_single(bg, 0.5, 0)) < 5e-5 * om1
    assert om1 / 0.01 ** 3 < oracle.L.ko_omega_nu_single(bg, 0.01, 0)
    assert abs(om1 - 0.5 / 93.14 / 0.49) < 1e-4 * om1
    assert oracle.L.ko_omega_nu_single(bg, 0.1, 1) == oracle.L.ko_omega_nu_single(bg, 0.1, 0)
    m0 = oracle.L.ko_omega_nu_single(bg, 1, 2)
    assert m0 / 0.5 ** 4 == oracle.L.ko_omega_nu_single(bg, 0.5, 2)
    assert oracle.L.ko_omega_nu_single(bg, 1e-4, 0) > oracle.L.ko_omega_nu_single(bg, 1, 0) / 1e-4 ** 3
    oracle.L.ko_bg_free(bg)
    bg = oracle.bg((0.2, 0.2, 0.2))
    assert oracle.bg_info(bg)[2] == [3, 0, 0]
    oracle.L.ko_bg_free(bg)
    bg = oracle.bg((0.2, 0.1, 0.3))
    assert oracle.bg_info(bg)[2] == [1, 1, 1]
    tot = sum(oracle.L.ko_omega_nu_single(bg, 0.5, i) for i in range(3))
    assert abs(oracle.L.ko_omega_nu(bg, 0.5) - tot) < 1e-6 * tot
    oracle.L.ko_bg_free(bg)
    assert oracle.L.ko_nufrac_low(0) == 0
    assert abs(oracle.L.ko_nufrac_low(1) / 0.0595634 - 1) < 1e-5
    assert abs(oracle.L.ko_nufrac_low(0.5) / 0.00941738 - 1) < 1e-5


def test_hybrid_known_answers(oracle):
    # omega_nu_single_test.c:171-187
    bg = oracle.bg((0.2, 0.2, 0.2))
    oracle.L.ko_bg_hybrid(bg, 700, 299792, 0.5)
    rhocrit, kb, deg, mnu = oracle.bg_info(bg)
    part = oracle.L.ko_nufrac_low(700 / 299792. * 0.2 / kb)
    assert abs(oracle.L.ko_particle_nu_fraction(bg, 0.50001, 0) / part - 1) < 1e-5
    assert oracle.L.ko_particle_nu_fraction(bg, 0.49999, 0) == 0
    r = oracle.L.ko_omega_nu_nopart(bg, 0.499999) * (1 - part) / oracle.L.ko_omega_nu_nopart(bg, 0.500001)
    assert abs(r - 1) < 1e-4
    r = oracle.L.ko_omega_nu_single(bg, 0.499999, 0) * (1 - part) / oracle.L.ko_omega_nu_single(bg, 0.500001, 0)
    assert abs(r - 1) < 1e-4
    oracle.L.ko_bg_free(bg)


def powerspectrum_test_field():
    """The 4^3 input of powerspectrum_test.c:21-35 (ones on the first 8 rows of the
    padded in-place array, field[0]=2) and its r2c transform (FFTW2 forward,
    unnormalised: numpy's rfftn is the same transform)."""
    f = np.zeros((4, 4, 4))
    padded = np.zeros(4 * 4 * 6)
    for i in range(32):
        padded[6 * (i // 4) + i % 4] = 1
    padded[0] = 2
    f = padded.reshape(4, 4, 6)[:, :, :4]
    return np.fft.rfftn(f).astype(np.complex64)


def test_powerspectrum_known_answers(oracle):
    g = powerspectrum_test_field()
    nk, p, c, k = oracle.total_powerspectrum(g, 4, 15)
    # powerspectrum_test.c:38-45
    assert nk == 9
    assert abs(k[2] - 1.73205) < 1e-5
    assert c[1] == 12 and c[0] == 6 and c[nk - 1] == 1
    assert abs(p[0] - 0.254834) < 1e-5 * 0.04
    assert abs(p[1] - 0.00212722) < 1e-5 * 0.005
    assert abs(p[2] - 0.00323766) < 1e-5 * 0.003


# ---------------------------------------------------------------- golden fixtures
def _testdata():
    return np.load(os.path.join(GOLD, "ref_testdata.npz"))


def _td_state(oracle, z, TimeMax=1.0):
    bg = oracle.bg(tuple(z["MNu"]), Omega0=0.2793, UnitTime_in_s=UT_KPC)
    n = len(z["keff"])
    s = oracle.state(bg, n, 0.01, TimeMax, Omega0=0.2793, UnitTime_in_s=UT_KPC, UnitLength_in_cm=KPC)
    oracle.set_transfer(s, z["t_logk"], z["t_T"])
    return bg, s


def test_golden_transfer_table():
    z = _testdata()
    # transfer_init_test.c:226-237: 271 rows above pi/BoxSize, fixed first values
    assert len(z["t_logk"]) == 271
    assert abs(z["t_T"][0] - 0.508479) < 1e-6
    assert abs(z["t_T"][30] - 0.0122563) < 1e-6
    assert z["t_logk"][0] > math.log(math.pi / 512000)


def test_golden_delta_tot_init(oracle):
    z = _testdata()
    bg, s = _td_state(oracle, z)
    n = len(z["keff"])
    assert oracle.L.ko_delta_tot_init(s, n, cases.np.ascontiguousarray(z["keff"]).ctypes.data_as(
        cases.np.ctypeslib.ctypes.POINTER(cases.np.ctypeslib.ctypes.c_double)),
        np.ascontiguousarray(z["dcdm"]).ctypes.data_as(np.ctypeslib.ctypes.POINTER(np.ctypeslib.ctypes.c_double)),
        0.01) == 0
    st = oracle.get_state(s)
    assert cases.rel_err(st["nu_init"][:n], z["init_fresh_nu_init"]) < 1e-14
    assert cases.rel_err(st["nu_last"][:n], z["init_fresh_nu_last"]) < 1e-14
    assert cases.rel_err(st["delta_tot"][:n, 0], z["init_fresh_row0"]) < 1e-14
    # delta_tot_table_test.c:143-150
    assert np.all(np.abs(st["nu_last"][:n] / st["nu_init"][:n] - 1) < 1e-4)


def test_golden_get_delta_nu_update(oracle):
    z = _testdata()
    bg, s = _td_state(oracle, z)
    oracle.set_nu_state(s, z["table_scalefact"], z["table"])
    st, d1 = oracle.get_delta_nu_update(s, 0.33333333, z["keff"], z["dcdm"])
    assert st == 0
    assert oracle.get_state(s)["ia"] == int(z["update1_ia"])
    assert cases.rel_err(d1, z["update1_dnu"]) < 1e-13
    # delta_tot_table_test.c:216-218: against the saved P_nu within 1e-2
    assert np.all(np.abs(d1 / z["dnu_file"] - 1) < 1e-2)
    oracle.L.ko_state_set_ia(s, oracle.get_state(s)["ia"] - 1)
    st, d2 = oracle.get_delta_nu_update(s, 0.33333333, z["keff"], z["dcdm"])
    assert st == 0 and oracle.get_state(s)["ia"] == int(z["update2_ia"])
    assert cases.rel_err(d2, z["update2_dnu"]) < 1e-13
    assert np.all(np.abs(d2 / z["dnu_file"] - 1) < 3e-2)


def test_golden_delta_pow(oracle):
    z = _testdata()
    lk, r = z["dpow_logk"], z["dpow_ratio"]
    import ctypes as C
    P = C.POINTER(C.c_double)
    lkp = np.ascontiguousarray(lk)
    rp = np.ascontiguousarray(r)
    got = np.array([oracle.L.ko_dnudcdm(lkp.ctypes.data_as(P), rp.ctypes.data_as(P), len(lk), 1.0, q, None)
                    for q in z["dpow_query"]])
    assert np.array_equal(got[:10], z["dpow_value"][:10])  # exact at the nodes (delta_pow_test.c:26-27)
    assert cases.rel_err(got, z["dpow_value"]) < 1e-15


def test_golden_camb_linear(oracle):
    """test_reproduce_linear (delta_tot_table_test.c:315-363): 99 steps; the oracle
    matches the reference step by step, and both track CAMB within the test's bounds."""
    z = np.load(os.path.join(GOLD, "ref_camb_linear.npz"))
    bg = oracle.bg(tuple(z["MNu"]), Omega0=0.2793, UnitTime_in_s=UT_KPC)
    s = oracle.state(bg, 200, 0.01, 1.0, Omega0=0.2793, UnitTime_in_s=UT_KPC, UnitLength_in_cm=KPC)
    oracle.set_transfer(s, z["t_logk"], z["t_T"])
    import ctypes as C
    P = C.POINTER(C.c_double)
    k0 = np.ascontiguousarray(z["k0"])
    d0 = np.ascontiguousarray(z["dcdm0"])
    assert oracle.L.ko_delta_tot_init(s, 200, k0.ctypes.data_as(P), d0.ctypes.data_as(P), 0.01) == 0
    worst = 0.0
    for i in range(99):
        st, d = oracle.get_delta_nu_update(s, float(z["a"][i]), z["keff"][i], z["dcdm"][i])
        assert st == 0
        assert oracle.get_state(s)["ia"] == int(z["ia"][i]) == i + 1
        worst = max(worst, cases.rel_err(d, z["dnu_ref"][i]))
        acc = 0.05 if i < 8 else (2e-2 if i < 22 else 1.2e-2)
        assert np.all(np.abs(z["dnu_camb"][i] - d) < acc * d)
    assert worst < 1e-12, worst


# ---------------------------------------------------------------- direct comparison
def test_oracle_matches_reference_build(oracle, reflib):
    """Binning and a full integrator update, restatement vs the reference C."""
    R = reflib
    for N, nb in ((16, 15), (32, 16), (48, 40)):
        g = W.make_grid(N, seed=3)
        n1, p1, c1, k1 = oracle.total_powerspectrum(g, N, nb)
        n2, p2, c2, k2 = R.total_powerspectrum(g, N, nb)
        assert n1 == n2 and np.array_equal(c1, c2)
        assert cases.rel_err(p1, p2) < 1e-14 and cases.rel_err(k1, k2) < 1e-14
    z = _testdata()
    bg, s = _td_state(oracle, z)
    oracle.set_nu_state(s, z["table_scalefact"], z["table"])
    st, d = oracle.get_delta_nu_update(s, 0.33333333, z["keff"], z["dcdm"])
    assert cases.rel_err(d, z["update1_dnu"]) < 1e-13


def test_e2e_golden_oracle(oracle):
    """The 16^3 end-to-end fixture: the oracle's add_nu_power_to_rhogrid reproduces the
    reference's corrected grids (three calls: commit, discard, commit)."""
    z = np.load(os.path.join(GOLD, "ref_e2e_n16.npz"))
    N, L, nb = int(z["N"]), float(z["L"]), int(z["nbins"])
    bg = oracle.bg(tuple(z["MNu"]), Omega0=0.3, UnitTime_in_s=W.UNIT_TIME)
    s = oracle.state(bg, nb, 0.01, float(z["TimeMax"]), Omega0=0.3, UnitTime_in_s=W.UNIT_TIME,
                     UnitLength_in_cm=W.UNIT_LENGTH_MPC)
    oracle.set_transfer(s, z["t_logk"], z["t_T"])
    oracle.set_nu_state(s, z["scalefact"], z["delta_tot"])
    g = z["grid0"].copy()
    for a, ref in zip(z["a"], z["grids"]):
        st, out = oracle.add_nu_power_to_rhogrid(s, float(a), L, g, N)
        assert st == 0
        rel = np.abs(g - ref) / np.maximum(np.abs(ref), 1e-30)
        assert rel.max() < 1e-6


@pytest.mark.parametrize("Na", [40, 256])
def test_fs_table_fixed_order_vs_qag(oracle, Na):
    """The cumulative fixed-order fslength table, as the GPU computes it (4-point
    Gauss-Legendre per segment, or 2-point where the knots are closer than 1.5e-3 in
    log a: the 256-row history), changes delta_nu by far less than the 1e-10 bar."""
    c = cases.make_case(64, 48, Na, 1.0, (0.02, 0.03, 0.06), grid=False, extra_rows=12 + Na // 4)
    res = []
    for mode in (0, 2, 3):
        bg, s = cases.oracle_state(oracle, c, fs_mode=mode)
        st, d = oracle.get_delta_nu_update(s, 1.01, c["kphys"], np.sqrt(W.spectrum(c["kphys"])))
        assert st == 0
        res.append(d)
    assert cases.rel_err(res[1], res[0]) < 1e-11
    assert cases.rel_err(res[2], res[0]) < 1e-11
