"""GPU against the outputs of the reference C itself (tests/golden/*.npz, made by
tests/golden/make_golden.py from the reference test suite's inputs)."""
import math
import os

import numpy as np
import pytest

import cases
import workloads as W

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KPC = 3.085678e21
UT_KPC = KPC / 1e5
TOL_DNU = 1e-10


def _inst(kg, MNu, nk, TimeMax, t_logk, t_T, Omega0=0.2793, UL=KPC, UT=UT_KPC):
    k = kg.KspaceNeutrinos()
    k.init_omega_nu(MNu, 0.01, 0.7)
    k.set_hubble(Omega0, 1 - Omega0, UT, True)
    k.alloc_table(nk, 0.01, TimeMax, Omega0, UT, UL)
    k.set_transfer(t_logk, t_T)
    return k


def test_testdata_init_and_updates(gpu):
    z = np.load(os.path.join(GOLD, "ref_testdata.npz"))
    n = len(z["keff"])
    # fresh start (delta_tot_table_test.c:127-152)
    k = _inst(gpu, tuple(z["MNu"]), n, 1.0, z["t_logk"], z["t_T"])
    d = k.get_delta_nu_update(0.01, z["keff"], z["dcdm"])
    v = k.vectors()
    assert cases.rel_err(v["delta_nu_init"][:n], z["init_fresh_nu_init"]) < 1e-13
    assert cases.rel_err(d, z["init_fresh_nu_last"]) < TOL_DNU
    sf, dt = k.get_nu_state()
    assert cases.rel_err(dt[:, 0], z["init_fresh_row0"]) < 1e-13
    k.close()
    # resume from the saved table (delta_tot_table_test.c:193-228)
    k = _inst(gpu, tuple(z["MNu"]), n, 1.0, z["t_logk"], z["t_T"])
    k.set_nu_state(z["table_scalefact"], z["table"])
    d1 = k.get_delta_nu_update(0.33333333, z["keff"], z["dcdm"])
    assert k.table_info()["ia"] == int(z["update1_ia"])
    assert cases.rel_err(d1, z["update1_dnu"]) < TOL_DNU, cases.rel_err(d1, z["update1_dnu"])
    v = k.vectors()
    assert cases.rel_err(v["delta_nu_init"][:n], z["resume_nu_init"]) < 1e-13
    sf, dt = k.get_nu_state()
    k.set_nu_state(sf[:-1], dt[:, :-1])  # the test's d_tot.ia-- (line 220)
    d2 = k.get_delta_nu_update(0.33333333, z["keff"], z["dcdm"])
    assert k.table_info()["ia"] == int(z["update2_ia"])
    assert cases.rel_err(d2, z["update2_dnu"]) < TOL_DNU
    k.close()


def test_camb_linear_99_steps(gpu):
    """test_reproduce_linear: 99 sequential updates; GPU vs the reference within 1e-10,
    and against CAMB within the reference test's tolerances."""
    z = np.load(os.path.join(GOLD, "ref_camb_linear.npz"))
    k = _inst(gpu, tuple(z["MNu"]), 200, 1.0, z["t_logk"], z["t_T"])
    worst = 0.0
    for i in range(99):
        d = k.get_delta_nu_update(float(z["a"][i]), z["keff"][i], z["dcdm"][i])
        assert k.table_info()["ia"] == int(z["ia"][i])
        worst = max(worst, cases.rel_err(d, z["dnu_ref"][i]))
        acc = 0.05 if i < 8 else (2e-2 if i < 22 else 1.2e-2)
        assert np.all(np.abs(z["dnu_camb"][i] - d) < acc * d)
    assert worst < TOL_DNU, worst
    k.close()


def test_e2e_n16_against_reference(gpu):
    import torch
    z = np.load(os.path.join(GOLD, "ref_e2e_n16.npz"))
    N, L, nb = int(z["N"]), float(z["L"]), int(z["nbins"])
    k = _inst(gpu, tuple(z["MNu"]), nb, float(z["TimeMax"]), z["t_logk"], z["t_T"], Omega0=0.3,
              UL=W.UNIT_LENGTH_MPC, UT=W.UNIT_TIME)
    k.set_nu_state(z["scalefact"], z["delta_tot"])
    g = torch.as_tensor(z["grid0"]).cuda()
    for a, ref in zip(z["a"], z["grids"]):
        k.add_nu_power_to_rhogrid(float(a), L, g, N)
        got = g.cpu().numpy()
        rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30)
        assert rel.max() < 1e-6, rel.max()
    k.close()
