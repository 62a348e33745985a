"""The library's own multi-rank path: two processes (torch.distributed, gloo on the host),
each with its own GPU context and a disjoint slab range of the grid, the per-bin sums
exchanged through kspace_gpu_set_allreduce wrapping dist.all_reduce -- the one exchange
of the path (powerspectrum.c:91-95).  Both ranks' kernels run on the one GPU; they never
wait on each other (the exchange is on the host, between kernels).  The ranks' slabs
put together must equal the single-rank GPU step: mode counts bit for bit, P(k) and
delta_nu/delta_cdm to rounding, the grid within 1e-6."""
import os
import socket

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
N, NB, NA = 32, 32, 10


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out_dir, slab_cut):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (os.path.join(root, "kspace-neutrinos_gb300"), os.path.join(root, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch
    import torch.distributed as dist
    import kspace_gpu as kg
    import cases as cs
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    c = cs.make_case(N, NB, NA, 0.5, (0.1, 0.1, 0.1))
    slab0 = 0 if rank == 0 else slab_cut
    nslab = slab_cut if rank == 0 else N - slab_cut
    k = cs.gpu_instance(kg, c)
    calls = []

    def allreduce(buf):
        t = torch.from_numpy(buf.copy())
        dist.all_reduce(t)
        buf[:] = t.numpy()
        calls.append(len(buf))

    k.set_allreduce(allreduce)
    g = torch.as_tensor(np.ascontiguousarray(c["grid"][slab0:slab0 + nslab])).cuda()
    nk, power, count, keff = k.total_powerspectrum(N, g, NB, slab0, nslab)
    np.save(os.path.join(out_dir, "count%d.npy" % rank), count)
    np.save(os.path.join(out_dir, "power%d.npy" % rank), power)
    for a in (0.51, 0.512):
        k.add_nu_power_to_rhogrid(a, c["L"], g, N, slab0, nslab)
    lc = k.last_correction()
    np.save(os.path.join(out_dir, "ratio%d.npy" % rank), lc["ratio"])
    np.save(os.path.join(out_dir, "slab%d.npy" % rank), g.cpu().numpy())
    np.save(os.path.join(out_dir, "calls%d.npy" % rank), np.array(calls))
    k.close()
    dist.destroy_process_group()


@pytest.mark.parametrize("slab_cut", [16, 5])
def test_two_ranks_equal_one(gpu, tmp_path, slab_cut):
    import torch
    import torch.multiprocessing as mp
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path), slab_cut), nprocs=2, join=True)
    c = cases.make_case(N, NB, NA, 0.5, (0.1, 0.1, 0.1))
    k = cases.gpu_instance(gpu, c)
    g = torch.as_tensor(c["grid"]).cuda()
    nk, p1, c1, _ = k.total_powerspectrum(N, g, NB)
    for a in (0.51, 0.512):
        k.add_nu_power_to_rhogrid(a, c["L"], g, N)
    r1 = k.last_correction()["ratio"]
    g1 = g.cpu().numpy()
    k.close()
    for r in range(2):
        # one exchange of nb + 1 doubles per binning pass (three passes per rank)
        assert list(np.load(tmp_path / ("calls%d.npy" % r))) == [NB + 1] * 3
        assert np.array_equal(np.load(tmp_path / ("count%d.npy" % r)), c1)
        assert cases.rel_err(np.load(tmp_path / ("power%d.npy" % r)), p1) < 1e-12
        assert cases.rel_err(np.load(tmp_path / ("ratio%d.npy" % r)), r1) < 1e-10
    both = np.concatenate([np.load(tmp_path / "slab0.npy"), np.load(tmp_path / "slab1.npy")])
    rel = np.abs(both - g1) / np.maximum(np.abs(g1), 1e-30)
    assert rel.max() < 1e-6, rel.max()
