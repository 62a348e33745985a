"""The warp-pipelined grid passes -- the default binning (K1) and correction (K3)
kernels -- over their tile shapes and both binning variants, against the oracle:
whole grids and slab ranges, grid sizes whose 16-mode rows straddle grid rows or
leave a partial last tile, and low-k regions that take the cooperative path.

Bars: mode counts bit-exact; the exact binning variant within 1e-12 of the oracle's
double sums (it carries the reference's double product and sums as float pairs); the
lean variant (FP32 run sums) within the 1e-6 bar for P(k); the corrected grid within
1e-6 relative."""
import math

import numpy as np
import pytest

import cases
import workloads as W

pytestmark = pytest.mark.gpu

L_BOX = 512.0
SHAPES = [(256, 2), (256, 3), (128, 2), (128, 3)]  # rows per CTA (32 per warp), stages per warp
TOL_EXACT = 1e-12
TOL_LEAN = 1e-6


def _instance(gpu, nb):
    k = gpu.KspaceNeutrinos()
    k.init_omega_nu((0.1, 0.1, 0.1), 0.01, 0.7)
    k.alloc_table(max(nb, 16), 0.01, 1.0, 0.3, cases.UT, cases.UL)
    return k


@pytest.mark.parametrize("N,nb", [(16, 15), (64, 48), (96, 80), (128, 128), (256, 200), (64, 1000), (100, 2500)])
def test_binning_stream_variants(gpu, oracle, N, nb):
    import torch
    g = W.make_grid(N, seed=100 + N)
    nk_o, p_o, c_o, _ = oracle.total_powerspectrum(g, N, nb)
    k = _instance(gpu, nb)
    gd = torch.as_tensor(g).cuda()
    worst = {3: 0.0, 4: 0.0, 5: 0.0, 6: 0.0}
    for rows, stages in SHAPES:
        for tma, tol in ((3, TOL_EXACT), (4, TOL_LEAN), (5, TOL_EXACT), (6, TOL_LEAN)):
            k.set_tuning(tma=tma, rows=rows, stages=stages)
            nk_g, p_g, c_g, _ = k.total_powerspectrum(N, gd, nb)
            assert nk_g == nk_o
            assert np.array_equal(c_g, c_o)
            err = cases.rel_err(p_g, p_o)
            worst[tma] = max(worst[tma], err)
            assert err < tol, (rows, stages, tma, err)
    # the CTA-tiled kernel of the same pass agrees too
    k.set_tuning(tma=1, rows=128, stages=2)
    _, p_1, _, _ = k.total_powerspectrum(N, gd, nb)
    assert cases.rel_err(p_1, p_o) < TOL_EXACT
    k.close()
    print("N=%d worst P error: exact %.2e / %.2e, lean %.2e / %.2e" % (N, worst[3], worst[5], worst[4], worst[6]))


@pytest.mark.parametrize("N,nb,cuts", [(96, 64, (0, 37, 96)), (128, 100, (0, 1, 64, 127, 128))])
def test_binning_stream_slabs(gpu, oracle, N, nb, cuts):
    """Per-slab bin sums through the allocation-free entry point (the same kernel)."""
    import torch
    lib = gpu.load_library()
    g = W.make_grid(N, seed=7 + N)
    for s0, s1 in zip(cuts[:-1], cuts[1:]):
        gs = np.ascontiguousarray(g[s0:s1])
        po, _, _, fo = oracle.total_powerspectrum(gs, N, nb, startslab=s0, nslab=s1 - s0, partial=True)
        gd = torch.as_tensor(gs).cuda()
        sums = np.full(nb + 1, np.nan)
        st = lib.kspace_gpu_bin_power_noalloc(N, gd.data_ptr(), nb, s0, s1 - s0, sums.ctypes.data, None)
        assert st == 0, st
        assert np.array_equal(sums[:nb] == 0, po == 0)
        m = po != 0
        assert cases.rel_err(sums[:nb][m], po[m]) < TOL_EXACT, (s0, s1)
        if s0 == 0:
            assert sums[nb] == fo


def _table(N, nb):
    count, keff = W.geometry(N, nb)
    kph = keff[count > 0] * 2 * math.pi / L_BOX
    ratio = 0.4 / (1.0 + (kph / 0.05) ** 2) + 0.01 * np.sin(7 * np.log(kph))
    return np.log(kph), ratio, 0.37


@pytest.mark.parametrize("N,nb", [(16, 15), (64, 48), (96, 80), (128, 100), (64, 1000)])
def test_correction_stream_variants(gpu, oracle, N, nb):
    import torch
    logk, ratio, norm = _table(N, nb)
    g = W.make_grid(N, seed=300 + N)
    go = g.copy()
    assert oracle.apply_correction(go, N, 0, N, L_BOX, logk, ratio, norm) == 0
    k = _instance(gpu, nb)
    for tma, (rows, stages) in [(3, s) for s in SHAPES] + [(1, (128, 2))]:
        k.set_tuning(tma=tma, rows=rows, stages=stages)
        gd = torch.as_tensor(g).cuda()
        k.apply_delta_pow(L_BOX, gd, N, nb, logk, ratio, norm)
        gg = gd.cpu().numpy()
        rel = np.abs(gg - go) / np.maximum(np.abs(go), 1e-30)
        assert rel.max() < 1e-6, (tma, rows, stages, rel.max())
    # slab ranges
    k.set_tuning(tma=3, rows=256, stages=2)
    cuts = (0, 5, N // 2, N)
    for s0, s1 in zip(cuts[:-1], cuts[1:]):
        gs = np.ascontiguousarray(g[s0:s1])
        gos = gs.copy()
        assert oracle.apply_correction(gos, N, s0, s1 - s0, L_BOX, logk, ratio, norm) == 0
        gd = torch.as_tensor(gs).cuda()
        k.apply_delta_pow(L_BOX, gd, N, nb, logk, ratio, norm, slabstart_y=s0, nslab_y=s1 - s0)
        rel = np.abs(gd.cpu().numpy() - gos) / np.maximum(np.abs(gos), 1e-30)
        assert rel.max() < 1e-6, (s0, s1, rel.max())
    k.close()


def test_binning_rows_warp_groups(gpu, oracle):
    """N=560: rows of 281 modes are 17 runs, a two-row tile is 34 runs, so tiles go to
    groups of two warps sharing a stage ring (the N >= 1024 shape, at a size the oracle
    bins in seconds)."""
    import torch
    N, nb = 560, 120
    g = W.make_grid(N, seed=11)
    nk_o, p_o, c_o, _ = oracle.total_powerspectrum(g, N, nb)
    k = _instance(gpu, nb)
    gd = torch.as_tensor(g).cuda()
    del g
    for rows, stages in ((256, 2), (128, 3)):
        for tma, tol in ((5, TOL_EXACT), (6, TOL_LEAN)):
            k.set_tuning(tma=tma, rows=rows, stages=stages)
            nk_g, p_g, c_g, _ = k.total_powerspectrum(N, gd, nb)
            assert nk_g == nk_o and np.array_equal(c_g, c_o)
            assert cases.rel_err(p_g, p_o) < tol, (rows, stages, tma)
    k.close()


@pytest.mark.parametrize("N,nb,Na", [(16, 16, 6), (64, 48, 24), (96, 80, 20)])
def test_full_step_host_grid_chunks(gpu, N, nb, Na):
    """A host grid moves in slab chunks (upload behind the binning pass, download behind
    the correction pass); the step must equal the same step on a device grid: the same
    correction table (to rounding of the per-chunk bin sums) and the same grid."""
    import torch
    c = cases.make_case(N, nb, Na, 0.5, (0.1, 0.1, 0.1))
    k_dev = cases.gpu_instance(gpu, c)
    k_host = cases.gpu_instance(gpu, c)
    g_dev = torch.as_tensor(c["grid"]).cuda()
    g_host = c["grid"].copy()
    for a in (0.51, 0.512, 0.53):
        k_dev.add_nu_power_to_rhogrid(a, c["L"], g_dev, N)
        k_host.add_nu_power_to_rhogrid(a, c["L"], g_host, N)
        l_dev, l_host = k_dev.last_correction(), k_host.last_correction()
        assert l_dev["nk"] == l_host["nk"]
        assert cases.rel_err(l_host["ratio"], l_dev["ratio"]) < 1e-12
        gd = g_dev.cpu().numpy()
        rel = np.abs(g_host - gd) / np.maximum(np.abs(gd), 1e-30)
        assert rel.max() < 1e-6, rel.max()
        g_host[...] = gd  # continue both from the same grid
    k_dev.close()
    k_host.close()


_ROW_KERNEL = r"""
import json, sys
sys.path[:0] = [sys.argv[1], sys.argv[1] + "/tests", sys.argv[1] + "/kspace-neutrinos_gb300"]
import torch
import cases, kspace_gpu as kg
import workloads as W
out = []
for N, nb in ((64, 48), (96, 80), (128, 128)):
    g = W.make_grid(N, seed=300 + N)
    k = kg.KspaceNeutrinos()
    k.init_omega_nu((0.1, 0.1, 0.1), 0.01, 0.7)
    k.alloc_table(max(nb, 16), 0.01, 1.0, 0.3, cases.UT, cases.UL)
    gd = torch.as_tensor(g).cuda()
    for tma in (5, 6):
        k.set_tuning(tma=tma)
        nk, p, c, _ = k.total_powerspectrum(N, gd, nb)
        out.append([N, nb, tma, int(nk), p.tolist(), c.tolist()])
    k.close()
print(json.dumps(out))
"""


def test_row_kernel_without_mirrors(gpu, oracle):
    """The row-aligned binning kernel (k_bin_rows with the run table, and its lean variant):
    the pass for grids of more than 32 runs per row (N > 1086), and with
    KSPACE_GPU_MIRROR=0 (read once per process, hence a child process), against the
    oracle: counts bit for bit, exact P(k) within 1e-12, lean within 1e-6."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, KSPACE_GPU_MIRROR="0")
    r = subprocess.run([sys.executable, "-c", _ROW_KERNEL, root], capture_output=True, text=True, timeout=600,
                       env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert len(res) == 6
    for N, nb, tma, nk, p, c in res:
        g = W.make_grid(N, seed=300 + N)
        nk_o, p_o, c_o, _ = oracle.total_powerspectrum(g, N, nb)
        assert nk == nk_o and np.array_equal(np.asarray(c), c_o)
        assert cases.rel_err(np.asarray(p), p_o) < (TOL_EXACT if tma == 5 else TOL_LEAN), (N, tma)
