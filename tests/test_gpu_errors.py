"""Error paths: each failure the reference reports through terminate(code, ...) comes
back from the library as that code (KspaceError.code in Python), made on the host --
no GPU fault is provoked.  The context stays usable afterwards.

  2002 nk differs from the stored table          delta_tot_table.c:203-204
  2003 fewer than two bins                        :205-206
  2023 no history although the run starts late   :91-92
  2024 scale factor before the transfer time     :94-95
  2006 a short row in the state file             :281
  2007 a state file starting at another a        :291-292
  2001/2004 NaN in the history or a NaN grid mode: the integral of a NaN integrand
       stops either in QAG (GSL error -> the reference's handler, terminate(2001),
       delta_tot_table.c:70-73,101) or at the NaN check after it (2004, :239-244),
       depending on how the NaN meets QAG's comparisons; the oracle (the reference's
       source built without -ffast-math) gives 2001 for the history and 2004 for the
       grid.  The reference as built by its own Makefile (-ffast-math) compiles both
       isnan checks away and returns without an error.
     5 NaN correction factor                      interface_gadget.c:183-184
  A step that fails in the integrator leaves the grid as it was (the multiply does not
  run; the reference terminates before it).
"""
import math

import numpy as np
import pytest

import cases
import workloads as W

pytestmark = pytest.mark.gpu


def _case():
    return cases.make_case(32, 32, 10, 0.5, (0.1, 0.1, 0.1), grid=False)


def _code(gpu, fn):
    with pytest.raises(gpu.KspaceError) as e:
        fn()
    return e.value.code


def test_bin_count_errors(gpu, oracle):
    c = _case()
    dcdm = np.sqrt(W.spectrum(c["kphys"]))
    k = cases.gpu_instance(gpu, c)
    k.get_delta_nu_update(0.51, c["kphys"], dcdm)
    assert _code(gpu, lambda: k.get_delta_nu_update(0.52, c["kphys"][:-1], dcdm[:-1])) == 2002
    # the context is still usable
    d = k.get_delta_nu_update(0.52, c["kphys"], dcdm)
    bg, s = cases.oracle_state(oracle, c)
    oracle.get_delta_nu_update(s, 0.51, c["kphys"], dcdm)
    st, d_o = oracle.get_delta_nu_update(s, 0.52, c["kphys"], dcdm)
    assert cases.rel_err(d, d_o) < 1e-10
    k.close()
    k = cases.gpu_instance(gpu, c)
    assert _code(gpu, lambda: k.get_delta_nu_update(0.51, c["kphys"][:1], dcdm[:1])) == 2003
    k.close()


def test_time_errors(gpu):
    c = _case()
    dcdm = np.sqrt(W.spectrum(c["kphys"]))
    k = gpu.make_instance(c["MNu"], 0.01, 0.7, 0.3, c["nbins"], c["TimeMax"], c["logk"], c["T"],
                          UnitLength_in_cm=cases.UL)
    # a fresh table (no history) at a late time: the resume file was not read
    assert _code(gpu, lambda: k.get_delta_nu_update(0.5, c["kphys"], dcdm)) == 2023
    # before the transfer function's time
    assert _code(gpu, lambda: k.get_delta_nu_update(0.005, c["kphys"], dcdm)) == 2024
    # a first call at the transfer time works
    d = k.get_delta_nu_update(0.01, c["kphys"], dcdm)
    assert np.all(np.isfinite(d))
    k.close()


def test_state_file_errors(gpu, tmp_path):
    c = _case()
    k = cases.gpu_instance(gpu, c)
    sf, dt = c["scalefact"], c["delta_tot"]
    short = tmp_path / "short.txt"
    with open(short, "w") as f:
        for i in range(len(sf)):
            vals = dt[:, i] if i != 3 else dt[:-2, i]  # row 3 is cut short
            f.write("# %le " % sf[i] + " ".join("%le" % v for v in vals) + " \n")
    assert _code(gpu, lambda: k.read_nu_state(str(short))) == 2006
    late = tmp_path / "late.txt"
    with open(late, "w") as f:
        for i in range(1, len(sf)):  # starts one row later than the transfer time
            f.write("# %le " % sf[i] + " ".join("%le" % v for v in dt[:, i]) + " \n")
    assert _code(gpu, lambda: k.read_nu_state(str(late))) == 2007
    k.close()


def test_nan_history_stops(gpu, oracle):
    c = _case()
    dt = c["delta_tot"].copy()
    dt[5, 4] = np.nan
    dcdm = np.sqrt(W.spectrum(c["kphys"]))
    k = gpu.make_instance(c["MNu"], 0.01, 0.7, 0.3, c["nbins"], c["TimeMax"], c["logk"], c["T"],
                          UnitLength_in_cm=cases.UL)
    k.set_nu_state(c["scalefact"], dt)
    assert _code(gpu, lambda: k.get_delta_nu_update(0.51, c["kphys"], dcdm)) in (2001, 2004)
    k.close()
    c2 = dict(c)
    c2["delta_tot"] = dt
    bg, s = cases.oracle_state(oracle, c2)
    st, _ = oracle.get_delta_nu_update(s, 0.51, c["kphys"], dcdm)
    assert st in (2001, 2004)


def test_nan_grid_mode(gpu, oracle):
    import torch
    c = cases.make_case(16, 16, 6, 0.5, (0.1, 0.1, 0.1))
    g = c["grid"].copy()
    g[3, 5, 2] = np.complex64(complex(np.nan, 0.0))
    bg, s = cases.oracle_state(oracle, c)
    st, _ = oracle.add_nu_power_to_rhogrid(s, 0.51, c["L"], g.copy(), 16)
    k = cases.gpu_instance(gpu, c)
    code = _code(gpu, lambda: k.add_nu_power_to_rhogrid(0.51, c["L"], torch.as_tensor(g).cuda(), 16))
    assert code in (2001, 2004) and st in (2001, 2004), (code, st)
    k.close()


def test_failed_step_leaves_grid(gpu):
    """An integrator error inside add_nu_power_to_rhogrid (a NaN in the history) stops the
    step before the multiply, as the reference's terminate does: the grid comes back bit
    for bit as it went in, from device memory and from host memory.  (delta_nu_last is NaN
    after such a step, as in the reference, where set_nu_state does not reset it:
    interface_common.c:166-179, delta_tot_table.c:225-228.)  A fresh context with the good
    history then steps the untouched grid normally."""
    import torch
    c = cases.make_case(16, 16, 6, 0.5, (0.1, 0.1, 0.1))
    dt = c["delta_tot"].copy()
    dt[2, 3] = np.nan
    k = cases.gpu_instance(gpu, c)
    k.set_nu_state(c["scalefact"], dt)
    g0 = c["grid"].copy()
    gd = torch.as_tensor(g0).cuda()
    assert _code(gpu, lambda: k.add_nu_power_to_rhogrid(0.51, c["L"], gd, 16)) in (2001, 2004)
    assert np.array_equal(gd.cpu().numpy(), g0)
    gh = g0.copy()
    assert _code(gpu, lambda: k.add_nu_power_to_rhogrid(0.51, c["L"], gh, 16)) in (2001, 2004)
    assert np.array_equal(gh, g0)
    k.close()
    k = cases.gpu_instance(gpu, c)
    k.add_nu_power_to_rhogrid(0.51, c["L"], gd, 16)
    assert not np.array_equal(gd.cpu().numpy(), g0)
    k.close()


def test_nan_correction_factor_gives_5(gpu):
    import torch
    c = cases.make_case(16, 16, 6, 0.5, (0.1, 0.1, 0.1))
    k = cases.gpu_instance(gpu, c)
    nb = c["nbins"]
    nk = c["nk"]
    logk = np.log(c["kphys"])
    ratio = np.full(nk, 0.01)
    ratio[nk // 2] = np.nan
    g = torch.as_tensor(c["grid"]).cuda()
    assert _code(gpu, lambda: k.apply_delta_pow(c["L"], g, 16, nb, logk, ratio, 0.01)) == 5
    ratio[nk // 2] = 0.01
    k.apply_delta_pow(c["L"], g, 16, nb, logk, ratio, 0.01)  # still usable
    k.close()


_EXPIRED_WAIT = r"""
import ctypes, os, sys
sys.path[:0] = [sys.argv[1], sys.argv[1] + "/tests", sys.argv[1] + "/kspace-neutrinos_gb300"]
import torch
import cases, kspace_gpu as kg
import workloads as W
rt = None
for name in ("libcudart.so.13", "libcudart.so"):
    try:
        rt = ctypes.CDLL(name)
        break
    except OSError:
        pass
N, nb = 64, 48
g = torch.as_tensor(W.make_grid(N, seed=4)).cuda()
k = kg.KspaceNeutrinos()
k.init_omega_nu((0.1, 0.1, 0.1), 0.01, 0.7)
k.alloc_table(nb, 0.01, 1.0, 0.3, cases.UT, cases.UL)
try:
    k.total_powerspectrum(N, g, nb)
    print("status 0")
except kg.KspaceError as e:
    print("status", e.code)
torch.cuda.synchronize()
print("pending", rt.cudaPeekAtLastError() if rt else 0)
x = torch.arange(10, device="cuda", dtype=torch.float64).sum().item()  # the device is still usable
print("after", x)
k.close()
"""


def test_expired_bounded_wait_returns_timeout(gpu):
    """The first bounded wait of the binning pass given no polls (KSPACE_GPU_TEST_FIRST_WAIT=0,
    read once per process): the wait reports expiry, the warps stop, the group's leader
    waits (bounded) for its copies still in flight, the kernel returns and the call gives
    KSPACE_ERR_TIMEOUT (10005); no trap, no pending CUDA error, the device stays usable."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, KSPACE_GPU_TEST_FIRST_WAIT="0")
    r = subprocess.run([sys.executable, "-c", _EXPIRED_WAIT, root], capture_output=True, text=True, timeout=600,
                       env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "status 10005" in r.stdout, r.stdout
    assert "pending 0" in r.stdout, r.stdout
    assert "after 45.0" in r.stdout, r.stdout
