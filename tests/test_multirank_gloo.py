"""Slab-decomposed step on two CPU ranks (torch.distributed, gloo): each rank bins its
slabs, the per-bin sums (nb doubles + |F(0)|^2) are all-reduced -- the one exchange of
the path (powerspectrum.c:91-95) -- the integrator runs replicated, and each rank
corrects its own slabs.  The result must equal the single-rank step: mode counts bit
for bit, power and grid to rounding."""
import math
import os
import socket

import numpy as np
import pytest

import cases
import workloads as W


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out_dir, N, nb, L):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle_lib import Oracle
    O = Oracle()
    c = cases.make_case(N, nb, 10, 0.5, (0.1, 0.1, 0.1))
    slab0 = N * rank // world
    nslab = N * (rank + 1) // world - slab0
    g = np.ascontiguousarray(c["grid"][slab0:slab0 + nslab])
    power, count, ksum, f0 = O.total_powerspectrum(g, N, nb, startslab=slab0, nslab=nslab, partial=True)
    buf = torch.from_numpy(np.concatenate([power, ksum, [f0], count.astype(np.float64)]))
    dist.all_reduce(buf)
    b = buf.numpy()
    P, K, F0, C = b[:nb], b[nb:2 * nb], b[2 * nb], b[2 * nb + 1:].astype(np.int64)
    m = C > 0
    Pn = P[m] / F0 / C[m]
    keff = K[m] / C[m]
    # integrator (replicated on every rank) and the multiply of this rank's slabs
    bg, s = cases.oracle_state(O, c)
    dcdm = np.sqrt(Pn / L ** -3)
    kphys = keff * 2 * math.pi / L
    st, dnu = O.get_delta_nu_update(s, 0.51, kphys, dcdm)
    assert st == 0
    logk = np.log(kphys)
    ratio = dnu / dcdm
    import ctypes as Cc
    norm = Cc.c_double()
    bgL = O.L
    om_nop = bgL.ko_omega_nu_nopart(bg, 0.51)
    om = bgL.ko_omega_nu(bg, 0.51)
    Omeganonu = O.scalars(s)["Omeganonu"]
    kprefac = om_nop / (Omeganonu / 0.51 ** 3 + (om - om_nop))
    assert O.apply_correction(g, N, slab0, nslab, L, logk, ratio, kprefac) == 0
    np.save(os.path.join(out_dir, "slab%d.npy" % rank), g)
    np.save(os.path.join(out_dir, "counts%d.npy" % rank), C[m])
    np.save(os.path.join(out_dir, "power%d.npy" % rank), Pn)
    dist.destroy_process_group()


def test_two_ranks_equal_one(tmp_path, oracle):
    import torch.multiprocessing as mp
    N, nb, L = 32, 32, 512.0
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path), N, nb, L), nprocs=2, join=True)
    c = cases.make_case(N, nb, 10, 0.5, (0.1, 0.1, 0.1))
    nk, p1, c1, k1 = oracle.total_powerspectrum(c["grid"], N, nb)
    for r in range(2):
        assert np.array_equal(np.load(tmp_path / ("counts%d.npy" % r)), c1)
        assert cases.rel_err(np.load(tmp_path / ("power%d.npy" % r)), p1) < 1e-13
    bg, s = cases.oracle_state(oracle, c)
    g = c["grid"].copy()
    st, out = oracle.add_nu_power_to_rhogrid(s, 0.51, L, g, N)
    assert st == 0
    both = np.concatenate([np.load(tmp_path / "slab0.npy"), np.load(tmp_path / "slab1.npy")])
    rel = np.abs(both - g) / np.maximum(np.abs(g), 1e-30)
    assert rel.max() < 1e-6
