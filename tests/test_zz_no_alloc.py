"""kspace_gpu_bin_power_noalloc (the binning pass with its scratch in a fixed device
array, no allocation) against kspace_gpu_total_powerspectrum on the same grid, called
twice in a row through the C ABI, with host and device outputs."""
import ctypes as C

import numpy as np
import pytest

import workloads as W

pytestmark = pytest.mark.gpu

UL = W.UNIT_LENGTH_MPC


def _power_from_sums(sums, nb, count_full):
    m = count_full > 0
    return sums[:nb][m] / sums[nb] / count_full[m]


@pytest.mark.parametrize("N,nb", [(64, 48), (96, 64)])
def test_noalloc_matches_total_powerspectrum(gpu, N, nb):
    import torch
    L = gpu.load_library()
    grid = W.make_grid_torch(N, 512.0, seed=N)
    logk, T = W.transfer_table(0.3)
    k = gpu.make_instance((0.1, 0.1, 0.1), 0.01, 0.7, 0.3, nb, 1.0, logk, T, UnitLength_in_cm=UL)
    nk, power, count, keff = k.total_powerspectrum(N, grid, nb)
    count_full, _ = W.geometry(N, nb)
    assert nk == int((count_full > 0).sum())
    torch.cuda.synchronize()
    for _ in range(2):  # two calls in a row reuse the scratch
        sums = np.full(nb + 1, np.nan)
        st = L.kspace_gpu_bin_power_noalloc(N, grid.data_ptr(), nb, 0, N, sums.ctypes.data, None)
        assert st == 0, st
        p = _power_from_sums(sums, nb, count_full)
        assert np.max(np.abs(p / power - 1)) <= 1e-12
    # device output
    out = torch.full((nb + 1,), float("nan"), dtype=torch.float64, device="cuda")
    st = L.kspace_gpu_bin_power_noalloc(N, grid.data_ptr(), nb, 0, N, out.data_ptr(), None)
    assert st == 0, st
    p = _power_from_sums(out.cpu().numpy(), nb, count_full)
    assert np.max(np.abs(p / power - 1)) <= 1e-12
    # warmed up: a further call takes no device memory (free memory unchanged)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    st = L.kspace_gpu_bin_power_noalloc(N, grid.data_ptr(), nb, 0, N, out.data_ptr(), None)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert st == 0 and free1 == free0, (free0, free1)
    # beyond the fixed scratch: refused, nothing launched
    sums = np.zeros(5001)
    assert L.kspace_gpu_bin_power_noalloc(N, grid.data_ptr(), 5000, 0, N, sums.ctypes.data, None) == 10002
    k.close()
