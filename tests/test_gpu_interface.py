"""The library against outputs of the reference C itself through its global interface
(tests/golden/ref_interface.npz, ref_hybrid.npz, ref_gadget_saves_n16.npz,
ref_total_power_n*.npz, made by tests/golden/make_golden.py):

* compute_neutrino_power_from_cdm (interface_common.c:106-123), the MP-Gadget entry,
  including its skipping of empty bins;
* the snapshot files: save_nu_state with its .bak rotation (delta_tot_table.c:304-352),
  save_neutrino_power (:356-374), save_total_power in a neutrino run and in a run
  without the integrator (interface_gadget.c:114-144,196-224);
* hybrid neutrinos: Omega_nu with and without particles, particle_nu_active, and
  delta_nu through the truncated specialJ series and the looser QAG tolerance
  (omega_nu_single.c:214-279, delta_tot_table.c:431-463,539-548).

Tolerances: delta_nu/delta_cdm 1e-10 relative; the grid 1e-6; numbers in the text files
as printed (%g: 6 significant digits, %le: 7), compared to 1e-5 relative after parsing;
Omega_nu 1e-9 (the Fermi-Dirac tables are integrated to a relative 1e-9 on both
sides)."""
import math
import os

import numpy as np
import pytest

import cases
import workloads as W

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
LIGHT_KMS = 2.99792458e10 / 1e5
TOL_DNU = 1e-10


def _gold(name):
    return np.load(os.path.join(GOLD, name))


def _inst(kg, z, hybrid=False):
    """allocate_kspace_memory's sequence (interface_common.c:77-102) with the same inputs."""
    k = kg.KspaceNeutrinos()
    k.init_omega_nu(tuple(z["MNu"]), 0.01, 0.7)
    if hybrid:
        k.init_hybrid_nu(float(z["vcrit"]), LIGHT_KMS, float(z["nu_crit_time"]))
    k.set_hubble(0.3, 0.7, W.UNIT_TIME, True)
    k.alloc_table(int(z["nbins"]), 0.01, float(z["TimeMax"]), 0.3, W.UNIT_TIME, W.UNIT_LENGTH_MPC)
    k.set_transfer(z["t_logk"], z["t_T"])
    k.set_nu_state(z["scalefact"], z["delta_tot"])
    return k


def _power_from_cdm(k, z, times, prefix="pc_"):
    """The inputs of the fixture's compute_neutrino_power_from_cdm calls, and the checks."""
    kin, nm = z["pc_keff_in"], z["pc_nmodes"]
    P0 = W.spectrum(np.where(nm > 0, kin, 0.05))
    a_end = float(z["a_end"])
    for j, a in enumerate(times):
        logk, ratio, norm = k.compute_neutrino_power_from_cdm(a, kin, P0 * (a / a_end) ** 2, nm)
        n = int(z[prefix + "nbins"][j])
        assert len(logk) == n
        assert k.table_info()["ia"] == int(z[prefix + "ia"][j])
        assert cases.rel_err(logk, z[prefix + "logk"][j][:n]) < 1e-15
        assert cases.rel_err(ratio, z[prefix + "ratio"][j][:n]) < TOL_DNU, (a, cases.rel_err(ratio, z[prefix + "ratio"][j][:n]))
        assert abs(norm / z[prefix + "norm"][j] - 1) < 1e-12


def _same_text(got, want, rtol=1e-5):
    """Line for line: the same tokens, numbers equal to the printed precision."""
    gl, wl = got.splitlines(), want.splitlines()
    assert len(gl) == len(wl)
    for g, w in zip(gl, wl):
        gt, wt = g.split(" "), w.split(" ")
        assert len(gt) == len(wt), (g, w)
        for a, b in zip(gt, wt):
            if a == b:
                continue
            fa, fb = float(a), float(b)
            assert abs(fa - fb) <= rtol * abs(fb), (g, w)


def test_compute_neutrino_power_from_cdm(gpu):
    z = _gold("ref_interface.npz")
    assert (z["pc_nmodes"] == 0).any()  # the empty bins are skipped
    k = _inst(gpu, z)
    _power_from_cdm(k, z, list(z["pc_times"]))
    k.close()


def test_snapshot_files_and_bak_rotation(gpu, tmp_path):
    z = _gold("ref_interface.npz")
    k = _inst(gpu, z)
    _power_from_cdm(k, z, list(z["pc_times"]))
    assert k.save_nu_power(0.53, 3, str(tmp_path)) == 0
    _same_text(open(tmp_path / "powerspec_nu_003.txt").read(), str(z["save_nu_power_txt"]))
    sfile = str(tmp_path / "delta_tot_nu.txt")
    k.save_nu_state(sfile)
    first = open(sfile).read()
    _power_from_cdm(k, z, [0.55], prefix="second_pc_")
    k.save_nu_state(sfile)
    # the first file moved to .bak, the new one in its place (delta_tot_table.c:335-348)
    assert open(sfile + ".bak").read() == first
    _same_text(open(sfile + ".bak").read(), str(z["save_state_bak_txt"]), rtol=2e-6)
    _same_text(open(sfile).read(), str(z["save_state_txt"]), rtol=2e-6)
    # and it resumes: read back into a fresh context, the same rows to printed precision
    k2 = _inst(gpu, z)
    k2.read_nu_state(sfile)
    sf1, dt1 = k.get_nu_state()
    sf2, dt2 = k2.get_nu_state()
    assert len(sf2) == len(sf1) and cases.rel_err(dt2, dt1) < 1e-6
    k.close()
    k2.close()


def test_gadget_step_and_total_power_neutrino_run(gpu, tmp_path):
    import torch
    z = _gold("ref_gadget_saves_n16.npz")
    k = _inst(gpu, z)
    g = torch.as_tensor(z["grid0"]).cuda()
    for a, ref in zip(z["a"], z["grids"]):
        k.add_nu_power_to_rhogrid(float(a), float(z["L"]), g, 16)
        got = g.cpu().numpy()
        assert (np.abs(got - ref) / np.maximum(np.abs(ref), 1e-30)).max() < 1e-6
    assert k.save_total_power(0.52, 2, str(tmp_path)) == 0
    _same_text(open(tmp_path / "powerspec_tot_002.txt").read(), str(z["save_total_txt"]))
    assert k.save_nu_power(0.52, 2, str(tmp_path)) == 0
    _same_text(open(tmp_path / "powerspec_nu_002.txt").read(), str(z["save_nu_power_txt"]))
    k.close()


@pytest.mark.parametrize("N", [16, 32])
def test_total_power_without_integrator(gpu, tmp_path, N):
    """A run without the neutrino module: no InitOmegaNu, no table (gadget-2 patch 0004),
    two snapshots.  The files match the reference's, the k column included (see
    save_total_power)."""
    z = _gold("ref_total_power_n%d.npz" % N)
    k = gpu.KspaceNeutrinos()
    for j in range(2):
        t = float(z["time%d" % j])
        k.compute_total_power_spectrum(t, 512.0, z["grid%d" % j], N)
        assert k.save_total_power(t, 7, str(tmp_path)) == 0
        _same_text(open(tmp_path / "powerspec_tot_007.txt").read(), str(z["txt%d" % j]))
    k.close()


def test_hybrid_neutrinos(gpu):
    z = _gold("ref_hybrid.npz")
    k = _inst(gpu, z, hybrid=True)
    for a, om, omn, act in zip(z["bg_a"], z["bg_omega_nu"], z["bg_omega_nu_nopart"], z["bg_particle_active"]):
        assert abs(k.OmegaNu(float(a)) / om - 1) < 1e-9
        assert abs(k.OmegaNu_nopart(float(a)) / omn - 1) < 1e-9
        assert k.particle_nu_active(float(a)) == int(act)
    assert k.particle_nu_active(0.51) == 1  # the steps below run with particles on
    _power_from_cdm(k, z, list(z["pc_times"]))
    k.close()


def test_integrals_at_the_calls_k(gpu, oracle):
    """get_delta_nu_update integrates at the k passed in each call (delta_tot_table.c:224,
    526, 593), not at the k stored when the table was initialised."""
    c = cases.make_case(32, 32, 12, 0.5, (0.1, 0.1, 0.1), grid=False)
    bg, s = cases.oracle_state(oracle, c)
    k = cases.gpu_instance(gpu, c)
    dcdm = np.sqrt(W.spectrum(c["kphys"]))
    for a, kscale in ((0.51, 1.0), (0.512, 1.03), (0.53, 0.97)):
        kk = c["kphys"] * kscale
        st, d_o = oracle.get_delta_nu_update(s, a, kk, dcdm)
        assert st == 0
        d_g = k.get_delta_nu_update(a, kk, dcdm)
        assert cases.rel_err(d_g, d_o) < TOL_DNU, (a, cases.rel_err(d_g, d_o))
    k.close()
