"""The integrator-level drop-in (include/kspace_delta_tot_table.h: delta_tot_table.h,
delta_pow.h, omega_nu_single.h, transfer_init.h) driven from C through the sequences
of the reference's delta_tot_table_test.c (tests/dropin/dtt_harness.c), against the
reference's own outputs on the same inputs (tests/golden/ref_testdata.npz, made by
tests/golden/make_golden.py from the reference sources).

Tolerances: delta_nu 1e-10 relative (the task's bar); quantities the reference forms
in one or two steps from the inputs (delta_nu_init, the first row) 1e-13; the fitted
J 1e-13; its truncated series and nufrac_low 1e-12; fslength 1e-9 (the reference's own
adaptive rule at relative tolerance 1e-6 against a converged fixed rule)."""
import math
import os
import subprocess

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def build_harness(tmp_path):
    exe = str(tmp_path / "dtt_harness")
    pkg = os.path.join(ROOT, "kspace-neutrinos_gb300")
    subprocess.run(["gcc", "-O2", "-Wall", "-I" + os.path.join(ROOT, "include"), "-o", exe,
                    os.path.join(ROOT, "tests", "dropin", "dtt_harness.c"),
                    os.path.join(pkg, "dropin", "kspace_delta_tot_table.c"), "-L" + pkg, "-lkspace_gb300",
                    "-Wl,-rpath," + pkg, "-lm"], check=True)
    return exe


def write_state(path, sf, dt):
    with open(path, "w") as f:  # the layout of delta_tot_table.c:320-324, full precision
        for i in range(len(sf)):
            f.write("# %.17e " % sf[i] + " ".join("%.17e" % v for v in dt[:, i]) + " \n")


def parse(out):
    vals, checks = {}, {}
    for line in out.splitlines():
        t = line.split()
        if not t:
            continue
        if t[0] == "check":
            checks[t[1]] = int(t[2])
        elif t[0] not in ("done", "terminated"):
            vals[t[0]] = np.array([float(x) for x in t[2:2 + int(t[1])]])
    return vals, checks


@pytest.fixture(scope="module")
def harness_run(tmp_path_factory):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    tmp = tmp_path_factory.mktemp("dtt")
    exe = build_harness(tmp)
    z = np.load(os.path.join(GOLD, "ref_testdata.npz"))
    n, tn = len(z["keff"]), len(z["t_logk"])
    for name, arr in (("keff.bin", z["keff"]), ("dcdm.bin", z["dcdm"]), ("tlogk.bin", z["t_logk"]),
                      ("tT.bin", z["t_T"])):
        np.ascontiguousarray(arr, dtype=np.float64).tofile(str(tmp / name))
    write_state(str(tmp / "delta_tot_nu.txt"), z["table_scalefact"], z["table"])
    r = subprocess.run([exe, str(tmp), str(n), str(tn), str(tmp)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    vals, checks = parse(r.stdout)
    return z, vals, checks, tmp


def test_reference_test_assertions(harness_run):
    """Every assertion of delta_tot_table_test.c holds through the drop-in."""
    _, _, checks, _ = harness_run
    assert len(checks) >= 12
    assert all(v == 1 for v in checks.values()), checks


def test_fresh_init(harness_run):
    z, v, _, _ = harness_run
    assert cases.rel_err(v["init_fresh_nu_init"], z["init_fresh_nu_init"]) < 1e-13
    assert cases.rel_err(v["init_fresh_row0"], z["init_fresh_row0"]) < 1e-13
    assert cases.rel_err(v["init_fresh_nu_last"], z["init_fresh_nu_last"]) < 1e-10


def test_resume_and_updates(harness_run):
    z, v, _, _ = harness_run
    assert cases.rel_err(v["resume_nu_init"], z["resume_nu_init"]) < 1e-13
    assert cases.rel_err(v["resume_nu_last"], z["resume_nu_last"]) < 1e-10
    assert int(v["update1_ia"][0]) == int(z["update1_ia"])
    assert cases.rel_err(v["update1_dnu"], z["update1_dnu"]) < 1e-10
    assert int(v["update2_ia"][0]) == int(z["update2_ia"])
    assert cases.rel_err(v["update2_dnu"], z["update2_dnu"]) < 1e-10


def test_get_delta_nu_single_mass_and_combined(harness_run):
    z, v, _, _ = harness_run
    for tag in ("m015", "m005", "combined"):
        assert cases.rel_err(v["resume_getdnu_" + tag], z["resume_getdnu_" + tag]) < 1e-10, tag


def test_update_delta_tot(harness_run):
    z, v, _, _ = harness_run
    assert int(v["update_new_ia"][0]) == int(z["update_new_ia"])
    assert cases.rel_err(v["update_new_row"], z["update_new_row"]) < 1e-10
    assert int(v["update_over_ia"][0]) == int(z["update_over_ia"])
    assert cases.rel_err(v["update_over_row"], z["update_over_row"]) < 1e-10
    assert v["update_over_loga"][0] == float(z["update_over_loga"])


def test_massless_neutrinos_other_units(harness_run):
    """test_allocate_delta_tot_table: zero masses, a table in units other than the
    host's H(a) (the host function is then tabulated on the GPU)."""
    z, v, _, _ = harness_run
    assert int(v["massless_ia"][0]) == int(z["massless_ia"])
    assert cases.rel_err(v["massless_dnu"], z["massless_dnu"]) < 1e-10


def test_special_functions(harness_run):
    z, v, _, _ = harness_run
    sj = z["sj_table"]
    for j in range(sj.shape[0]):
        got = v["sj_row%d" % j]
        assert np.array_equal(got[:2], sj[j, :2])
        tol = 1e-13 if sj[j, 0] <= 0 else 1e-12
        assert cases.rel_err(got[2:], sj[j, 2:]) < tol, (j, got[2:], sj[j, 2:])
    assert cases.rel_err(v["nufrac_val"], z["nufrac_val"]) < 1e-12
    assert cases.rel_err(v["fsl_val"][:4], z["fsl_val"][:4]) < 1e-9
    assert v["fsl_val"][4] == 0.0 == z["fsl_val"][4]


def test_state_files(harness_run):
    """The state written by save_all_nu_state reads back (checked in C) and keeps the
    reference's line layout; save_nu_power writes the reference's header."""
    z, v, _, tmp = harness_run
    assert v["roundtrip_combined_rel"][0] < 1e-5  # rows printed with 7 significant digits
    lines = open(tmp / "saved_delta_tot_nu.txt").read().splitlines()
    assert len(lines) == int(z["update_over_ia"])
    for ln in lines:
        assert ln.startswith("# ") and ln.endswith(" ")
        toks = ln[2:].split(" ")[:-1]
        assert len(toks) == len(z["keff"]) + 1
        assert all("e" in t and len(t.split("e")[0].split(".")[1]) == 6 for t in toks)
    pn = open(tmp / "powerspec_nu_004.txt").read().splitlines()
    assert pn[:3] == ["# k P_nu(k)", "# a = 0.35", "# nbins = %d" % len(z["keff"])]
    assert os.path.exists(str(tmp / "saved_delta_tot_nu.txt.bak"))


def test_delta_pow(harness_run):
    _, v, _, _ = harness_run
    # linear interpolation in log k, clamped at both ends (delta_pow.c:19-37), times norm
    assert np.allclose(v["dpow_vals"], [2 * 2.0, 2 * 2.5, 2 * 2.0, 2 * 1.0], rtol=0, atol=1e-15)
