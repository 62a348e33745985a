"""Batched integration against the single-instance path and the oracle.

Instances with different masses, cosmologies, history lengths and bin counts -- two of
them bound to grids of different sizes -- are advanced together through the batch ABI
(one captured CUDA graph per call) and, as twins with identical inputs, one at a time
through kspace_gpu_get_delta_nu_update / kspace_gpu_add_nu_power_to_rhogrid.  The
calls mix committed rows, dropped provisional rows and the same-scale-factor shortcut.
delta_nu must agree to 1e-12 relative (the bar for batching is 1e-10), the corrected
grids to 1e-6.  A tuning run in between (dry steps) must leave every state unchanged.
Three free instances (one, two and three mass states) are also driven through the
oracle's get_delta_nu_update with the same inputs: delta_nu within 1e-10.
"""
import math

import numpy as np
import pytest

import cases
import workloads as W

pytestmark = pytest.mark.gpu

UL, UT = W.UNIT_LENGTH_MPC, W.UNIT_TIME
L = 512.0


def make_params(M, seed):
    ps = W.batch_instances(M, seed=seed, Na_range=(16, 48), nk_range=(64, 96))
    if M > 5:
        ps[3]["MNu"] = (0.02, 0.03, 0.06)  # non-degenerate: three species
        ps[5]["MNu"] = (0.05, 0.05, 0.1)   # two species
    return ps


def build_instance(kg, p, nbins_grid=None, N=None):
    TimeMax = 0.01 + (p["Na"] + 20) / 100.0
    logk, T = W.transfer_table(float(sum(p["MNu"])))
    if N is None:
        kphys, nk_alloc = p["k"], p["nk"]
    else:
        count, keff = W.geometry(N, nbins_grid)
        kphys = keff[count > 0] * 2 * math.pi / L
        nk_alloc = nbins_grid
    k = kg.make_instance(p["MNu"], 0.01, p["h"], p["Omega0"], nk_alloc, TimeMax, logk, T, UnitLength_in_cm=UL)
    sf, dt = W.history(kphys, p["Na"], p["a_end"])
    k.set_nu_state(sf, dt)
    return k, kphys


def schedule(M):
    """Scale factors per call and instance: committed rows, dropped rows, same a."""
    base = np.array([1.0, 1.01, 1.014, 1.02, 1.02, 1.031])
    jit = np.where(np.arange(M) % 2 == 0, 0.0, 0.005)
    calls = [np.full(M, base[0])]
    for b in base[1:]:
        calls.append(b + jit)
    return calls


def oracle_instance(oracle, p):
    """The oracle state of instance p (the inputs build_instance gives the library)."""
    ut = UL / 1e5
    bg = oracle.bg(p["MNu"], a0=0.01, h=p["h"], Omega0=p["Omega0"], UnitTime_in_s=ut)
    s = oracle.state(bg, p["nk"], 0.01, 0.01 + (p["Na"] + 20) / 100.0, Omega0=p["Omega0"], UnitTime_in_s=ut,
                     UnitLength_in_cm=UL)
    logk, T = W.transfer_table(float(sum(p["MNu"])))
    oracle.set_transfer(s, logk, T)
    sf, dt = W.history(p["k"], p["Na"], p["a_end"])
    assert oracle.set_nu_state(s, sf, dt) == 0
    return s


def test_batch_matches_single_instances(gpu, oracle):
    import torch
    M = 18
    ps = make_params(M, seed=3)
    grid_N = {0: 32, 1: 48}
    nbins_grid = 24
    batch_insts, twins, kph = [], [], []
    for i, p in enumerate(ps):
        N = grid_N.get(i)
        k1, kp = build_instance(gpu, p, nbins_grid, N)
        k2, _ = build_instance(gpu, p, nbins_grid, N)
        batch_insts.append(k1)
        twins.append(k2)
        kph.append(kp)
    grids_b = {i: W.make_grid_torch(N, L, seed=10 + i) for i, N in grid_N.items()}
    grids_t = {i: g.clone() for i, g in grids_b.items()}
    B = gpu.KspaceBatch(batch_insts)
    for i, N in grid_N.items():
        B.bind_grid(i, grids_b[i], N, L)
    nk = np.array([0 if i in grid_N else len(kph[i]) for i in range(M)], dtype=np.int32)
    keff_pool = np.concatenate([kph[i] for i in range(M) if i not in grid_N])
    dcdm0 = np.concatenate([np.sqrt(W.spectrum(kph[i])) for i in range(M) if i not in grid_N])
    calls = schedule(M)
    oracle_ids = (2, 3, 5)  # one, three and two mass states
    ostates = {i: oracle_instance(oracle, ps[i]) for i in oracle_ids}
    worst_oracle = 0.0
    B.init(calls[0], nk, keff_pool, dcdm0)
    off = B.offsets
    assert list(B.nk[2:]) == [len(kph[i]) for i in range(2, M)]
    rng = np.random.default_rng(0)
    worst = 0.0
    for ci, a in enumerate(calls):
        if ci == 3:
            # tuning in the middle: dry steps only
            B.autotune(calls[4], np.ones(int(off[-1])), reps=1)
        # delta_cdm of this call: the generator's, with a small per-call change
        dcdm = np.zeros(int(off[-1]))
        for i in range(M):
            if i in grid_N:
                continue
            dcdm[off[i]:off[i + 1]] = np.sqrt(W.spectrum(kph[i])) * (1 + 0.01 * ci) * (
                1 + 1e-3 * rng.standard_normal(len(kph[i])))
        out = B.step(a, dcdm)
        assert not B.status().any(), B.status()
        torch.cuda.synchronize()
        for i in range(M):
            t = twins[i]
            if i in grid_N:
                N = grid_N[i]
                t.add_nu_power_to_rhogrid(a[i], L, grids_t[i], N)
                corr = t.last_correction()
                ratio_b = out[off[i]:off[i + 1]] / corr["dcdm"][:len(corr["ratio"])]
                got = out[off[i]:off[i + 1]]
                ref = corr["ratio"] * corr["dcdm"][:len(corr["ratio"])]
                assert cases.rel_err(ratio_b, corr["ratio"]) <= 1e-12
                torch.cuda.synchronize()
                d = (grids_b[i] - grids_t[i]).abs().max().item()
                assert d <= 1e-6 * grids_t[i].abs().max().item(), (ci, i, d)
            else:
                ref = t.get_delta_nu_update(a[i], kph[i], dcdm[off[i]:off[i + 1]])
                got = out[off[i]:off[i + 1]]
            nz = np.abs(ref) > 0
            err = cases.rel_err(got[nz], ref[nz]) if nz.any() else 0.0
            assert np.array_equal(got == 0, ref == 0)
            worst = max(worst, err)
            assert err <= 1e-12, (ci, i, err)
            if i in ostates:
                st, ro = oracle.get_delta_nu_update(ostates[i], a[i], kph[i], dcdm[off[i]:off[i + 1]])
                assert st == 0
                nzo = np.abs(ro) > 0
                eo = cases.rel_err(got[nzo], ro[nzo])
                worst_oracle = max(worst_oracle, eo)
                assert eo <= 1e-10, (ci, i, eo)
    # the twins' history tables equal the batch's
    for i in range(M):
        s1 = batch_insts[i].table_info()
        s2 = twins[i].table_info()
        assert s1 == s2
        v1, v2 = batch_insts[i].vectors(), twins[i].vectors()
        for key in v1:
            assert cases.rel_err(v1[key][:s1["nk"]], v2[key][:s1["nk"]]) <= 1e-12, key
    B.close()
    for k in batch_insts + twins:
        k.close()
    print("worst batch/single relative difference", worst, "batch/oracle", worst_oracle)


def test_batch_errors(gpu):
    ps = make_params(3, seed=5)
    insts = [build_instance(gpu, p)[0] for p in ps]
    B = gpu.KspaceBatch(insts)
    nk = np.array([p["nk"] for p in ps], dtype=np.int32)
    keff = np.concatenate([p["k"] for p in ps])
    dc = np.sqrt(W.spectrum(keff))
    a = np.full(3, 1.0)
    B.init(a, nk, keff, dc)
    # committing a row per call fills the shortest table first: its status is the
    # history-table-full code, the other instances keep stepping
    code = None
    for j in range(40):
        try:
            B.step(a + 0.01 * (j + 1), dc)
        except gpu.KspaceError as e:
            code = e.code
            break
    assert code == 2025
    st = B.status()
    assert set(st.tolist()) <= {0, 2025}
    assert st[int(np.argmin([p["Na"] for p in ps]))] == 2025
    B.close()
    for k in insts:
        k.close()
