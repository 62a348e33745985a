"""Seeded synthetic inputs with the shapes and value distributions of the benchmark
configurations (no public dataset is involved).

Grid: an r2c k-space density grid ``[nslab][N][N/2+1]`` complex64 (FFTW2 slab layout,
z fastest, powerspectrum.c:57-59).  Each mode has Re, Im ~ N(0, P(|k|)/2) with
P(k) = 2e4 (k/0.02) / (1 + (k/0.02)^2.8) (Mpc/h)^3, k = 2 pi |n| / L.  The kz=0 and
kz=N/2 planes are made Hermitian (F(-n) = conj F(n)); self-conjugate modes are real with
variance P.  The DC mode is F(0) = L^{3/2}, so that the estimator P_b L^3 / |F(0)|^2
of the reference (interface_gadget.c:96-97) returns P(k) in expectation.

History: rows at log-spaced a_j from TimeTransfer to a_end with
delta_tot(k_b, a_j) = sqrt(P(k_b)) a_j / a_end on the non-empty bins of the grid.
Transfer table: 300 log-spaced k in [1e-4, 50] h/Mpc, T_nu/T_nonu = 1/(1+(k/k_fs)^2),
k_fs = 0.05 (sum M_nu / 0.1 eV) h/Mpc.
"""
import math

import numpy as np

UNIT_LENGTH_MPC = 3.085678e24          # cm per internal length unit (Mpc/h)
UNIT_TIME = UNIT_LENGTH_MPC / 1e5      # s


def spectrum(k):
    k = np.asarray(k, dtype=np.float64)
    x = k / 0.02
    return 2e4 * x / (1.0 + x ** 2.8)


def kval(n, N):
    n = np.asarray(n)
    return np.where(n <= N // 2, n, n - N)


def _hermitian_plane(plane):
    """Make an N x N plane Hermitian: P[-x,-y] = conj P[x,y]; self-conjugate real."""
    N = plane.shape[0]
    x = np.arange(N)[:, None]
    y = np.arange(N)[None, :]
    px = (-x) % N
    py = (-y) % N
    idx = (x * N + y).ravel()
    pidx = (px * N + py).ravel()
    flat = plane.reshape(-1).copy()
    canon = idx < pidx
    selfc = idx == pidx
    out = flat.copy()
    out[pidx[canon]] = np.conj(flat[idx[canon]])
    out[selfc] = (flat[selfc].real * math.sqrt(2.0)).astype(np.float32)
    return out.reshape(N, N)


def make_grid(N, L=512.0, seed=0, slab0=0, nslab=None):
    """Host (numpy) grid generator; returns complex64 [nslab, N, N/2+1]."""
    if nslab is None:
        nslab = N
    rng = np.random.default_rng(seed)
    nz = N // 2 + 1
    g = np.empty((N, N, nz), dtype=np.complex64)
    kx = kval(np.arange(N), N).astype(np.float64)
    kz = np.arange(nz, dtype=np.float64)
    kxy2 = kx[:, None] ** 2 + kx[None, :] ** 2
    for i in range(N):  # slab by slab to bound temporary memory
        k = 2 * math.pi / L * np.sqrt(kxy2[i][:, None] + kz[None, :] ** 2)
        amp = np.sqrt(spectrum(np.where(k > 0, k, 1.0)) / 2.0)
        re = rng.standard_normal((N, nz)) * amp
        im = rng.standard_normal((N, nz)) * amp
        g[i] = (re + 1j * im).astype(np.complex64)
    for z in (0, N // 2):
        g[:, :, z] = _hermitian_plane(g[:, :, z])
    g[0, 0, 0] = np.complex64(L ** 1.5)
    return np.ascontiguousarray(g[slab0:slab0 + nslab])


def make_grid_torch(N, L=512.0, seed=0, device="cuda"):
    """Device (torch) generator with the same distribution (a different random stream).
    Returns a complex64 tensor [N, N, N/2+1]."""
    import torch
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    nz = N // 2 + 1
    g = torch.empty((N, N, nz), dtype=torch.complex64, device=device)
    kx = torch.as_tensor(kval(np.arange(N), N), dtype=torch.float64, device=device)
    kz = torch.arange(nz, dtype=torch.float64, device=device)
    kxy2 = kx[:, None] ** 2 + kx[None, :] ** 2
    step = max(1, (1 << 26) // (N * nz))
    for i0 in range(0, N, step):
        i1 = min(N, i0 + step)
        k = 2 * math.pi / L * torch.sqrt(kxy2[i0:i1, :, None] + kz[None, None, :] ** 2)
        x = torch.where(k > 0, k, torch.ones_like(k)) / 0.02
        amp = torch.sqrt(2e4 * x / (1.0 + x ** 2.8) / 2.0)
        re = torch.randn(k.shape, generator=gen, device=device, dtype=torch.float64) * amp
        im = torch.randn(k.shape, generator=gen, device=device, dtype=torch.float64) * amp
        g[i0:i1] = torch.complex(re.float(), im.float())
    for z in (0, N // 2):
        plane = g[:, :, z].cpu().numpy()
        g[:, :, z] = torch.as_tensor(_hermitian_plane(plane), device=device)
    g[0, 0, 0] = complex(L ** 1.5, 0.0)
    return g


def geometry(N, nrbins, slab0=0, nslab=None):
    """Mode counts and mean |k| (grid units) per bin, as total_powerspectrum would
    compute them (powerspectrum.c:40,56-89), from a histogram over integer k^2.
    Returns (count[nrbins] int64, keff[nrbins] float64 (0 where empty))."""
    if nslab is None:
        nslab = N
    nz = N // 2 + 1
    kx = kval(np.arange(slab0, slab0 + nslab), N).astype(np.int64)
    ky = kval(np.arange(N), N).astype(np.int64)
    kxy2 = (kx[:, None] ** 2 + ky[None, :] ** 2).ravel()
    h2 = np.bincount(kxy2)
    k2max = 3 * (N // 2) ** 2
    hist = np.zeros(k2max + 1, dtype=np.int64)
    nzv = np.nonzero(h2)[0]
    for z in range(nz):
        w = 1 if (z == 0 or z == N // 2) else 2
        hist[nzv + z * z] += w * h2[nzv]
    hist[0] = 0  # the DC mode is not binned
    k2 = np.nonzero(hist)[0]
    binsperunit = (nrbins - 1) / math.log(math.sqrt(3) * N / 2.0)
    kk = np.sqrt(k2.astype(np.float64))
    b = np.floor(binsperunit * np.log(kk)).astype(np.int64)
    count = np.zeros(nrbins, dtype=np.int64)
    np.add.at(count, b, hist[k2])
    ksum = np.zeros(nrbins)
    np.add.at(ksum, b, hist[k2] * kk)
    keff = np.where(count > 0, ksum / np.maximum(count, 1), 0.0)
    return count, keff


def transfer_table(sum_mnu, n=300, kmin=1e-4, kmax=50.0):
    logk = np.linspace(math.log(kmin), math.log(kmax), n)
    kfs = 0.05 * (sum_mnu / 0.1)
    T = 1.0 / (1.0 + (np.exp(logk) / kfs) ** 2)
    return logk, T


def history(k_phys, Na, a_end, a0=0.01):
    """(scalefact[Na] = log a_j, delta_tot[nk][Na])."""
    a = np.exp(np.linspace(math.log(a0), math.log(a_end), Na))
    sf = np.log(a)
    sf[0] = math.log(a0)
    dt = np.sqrt(spectrum(k_phys))[:, None] * (a[None, :] / a_end)
    return sf, np.ascontiguousarray(dt)


CONFIGS = {
    # name: grid N, bins, history rows, history end, masses
    "cfg0_n128": dict(N=128, nbins=128, Na=32, a_end=0.5, MNu=(0.1, 0.1, 0.1), L=512.0),
    "cfg1_n512": dict(N=512, nbins=256, Na=256, a_end=1.0, MNu=(0.1, 0.1, 0.1), L=512.0),
    "cfg2_n1024": dict(N=1024, nbins=512, Na=512, a_end=1.0, MNu=(0.02, 0.03, 0.06), L=512.0),
    "cfg3_n256": dict(N=256, nbins=128, Na=128, a_end=1.0, MNu=(0.05, 0.05, 0.05), L=512.0),
    # a smaller grid with the N=1024 workload's kernel shapes (two warps per row-pair tile in
    # the binning pass), for full ncu captures that stay within a few GB of device memory
    "prof_n768": dict(N=768, nbins=384, Na=256, a_end=1.0, MNu=(0.02, 0.03, 0.06), L=512.0),
    # profiling case: grid larger than L2 (227 MB) but small enough for multi-pass captures
    "prof_n384": dict(N=384, nbins=192, Na=64, a_end=1.0, MNu=(0.1, 0.1, 0.1), L=512.0),
}

# Batched integration: independent instances with their own cosmology, masses, history
# length and k bins, plus grids bound to some of them.
BATCH = dict(M=4096, grids=16, grid_N=(64, 96, 128, 192, 256), nbins_grid=128, a_end=1.0, L=512.0)


def batch_instances(M, seed=0, a_end=1.0, Na_range=(16, 512), nk_range=(64, 512)):
    """Per-instance parameters: sum M_nu ~ U(0.03, 0.6) eV as 3 degenerate states,
    Omega0 ~ U(0.25, 0.35), h ~ U(0.6, 0.75), history length Na ~ U{16..512} log-spaced
    rows from a = 0.01 to a_end, nk ~ U{64..512} bins log-spaced over 0.005-5 h/Mpc."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(M):
        s = float(rng.uniform(0.03, 0.6))
        Na = int(rng.integers(Na_range[0], Na_range[1] + 1))
        nk = int(rng.integers(nk_range[0], nk_range[1] + 1))
        out.append(dict(MNu=(s / 3, s / 3, s / 3), Omega0=float(rng.uniform(0.25, 0.35)),
                        h=float(rng.uniform(0.6, 0.75)), Na=Na, nk=nk, a_end=a_end,
                        k=np.exp(np.linspace(math.log(0.005), math.log(5.0), nk))))
    return out


def batch_grid_sizes(G, seed=0, choices=(64, 96, 128, 192, 256)):
    rng = np.random.default_rng(seed + 7)
    return [int(x) for x in rng.choice(choices, size=G)]
