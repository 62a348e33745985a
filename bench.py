#!/usr/bin/env python3
"""Benchmark of the linear-response neutrino force correction step on GB300.

One "step" = add_nu_power_to_rhogrid on a synthetic r2c grid: bin the grid into the
power spectrum (K1), advance delta_nu over the stored delta_tot history (K2), multiply
every mode by the neutrino correction (K3).  Default workload: the precision
configuration, an N=1024 grid (1024x1024x513 complex64, 4.3 GB), 512 log k bins, a
512-row history from a=0.01 to a=1.0, three neutrino mass states of 0.02, 0.03 and
0.06 eV, box 512 Mpc/h.  The N=512 configuration (512x512x257, 256 bins, 256-row
history, 3 x 0.1 eV) is measured too and reported under "n512".

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  value = grid modes processed per second (whole job) with the
grid resident in HBM; e2e = the same through the C ABI with the grid in pinned host
memory (host->device and device->host copies inside the timed region), beside the
plain copy bandwidth of the host link.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "kspace-neutrinos_gb300"))

import numpy as np  # noqa: E402

import workloads as W  # noqa: E402

METRIC = "k-modes/s & HBM GB/s per step, plain vs fwd+adjoint; batched solves/s; err vs FP64"
UNIT = "k-modes/s"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class NvmlClockSampler:
    """SM clock and clock-event (throttle) reasons polled every millisecond through NVML
    (the driver's libnvidia-ml) while running; a timed region of a few ms still gets
    samples.  Falls back to ClockSampler (nvidia-smi) where NVML cannot be opened."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, gpu_index=0):
        import ctypes
        self.C = ctypes
        self.samples = []
        self.stop = False
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        ids = [x for x in vis.split(",") if x.strip()]
        idx = int(ids[gpu_index]) if gpu_index < len(ids) and ids[gpu_index].strip().isdigit() else gpu_index
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        if self.lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(idx), ctypes.byref(self.h)) != 0:
            raise RuntimeError("no NVML handle")
        mx = ctypes.c_uint()
        self.max_mhz = float(mx.value) if self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, ctypes.byref(mx)) == 0 else None
        self.reason_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(self.lib, "nvmlDeviceGetCurrentClocksThrottleReasons")

    def _poll(self):
        C = self.C
        clk, rs = C.c_uint(), C.c_ulonglong()
        while not self.stop:
            if self.lib.nvmlDeviceGetClockInfo(self.h, 1, C.byref(clk)) == 0 and \
                    self.reason_fn(self.h, C.byref(rs)) == 0:
                self.samples.append((float(clk.value), int(rs.value)))
            time.sleep(0.001)

    def __enter__(self):
        self.t = threading.Thread(target=self._poll, daemon=True)
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop = True
        self.t.join(timeout=2)

    def summary(self):
        sm = [c for c, _ in self.samples]
        reasons = set()
        for _, r in self.samples:
            for bit, name in self.REASONS.items():
                if r & bit:
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": self.max_mhz,
                "reasons": sorted(reasons), "samples": len(sm), "source": "nvml, 1 ms polling"}


def clock_sampler(gpu_index=0):
    try:
        return NvmlClockSampler(gpu_index)
    except Exception:
        return ClockSampler(gpu_index)


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


_HOST_GRIDS = {}


def host_grid(N, L, seed):
    """The seeded numpy grid, generated once per process (4.3 GB at N=1024)."""
    key = (N, L, seed)
    if key not in _HOST_GRIDS:
        _HOST_GRIDS.clear()
        _HOST_GRIDS[key] = W.make_grid(N, L, seed=seed)
    return _HOST_GRIDS[key]


def bench_config(cfg):
    """The workload description printed by both arms (the same dict)."""
    N = cfg["N"]
    gbytes = 8 * N * N * (N // 2 + 1)
    return {"workload": cfg["name"], "N": N, "nbins": cfg["nbins"], "history_rows": cfg["Na"],
            "masses_eV": list(cfg["MNu"]), "box_mpc_h": cfg["L"], "grid_bytes": gbytes,
            "l2": ("grid (%.0f MB) larger than L2 (129 MB): no flush" % (gbytes / 1e6)) if gbytes >= 160e6 else
                  ("grid (%.0f MB) smaller than L2 (129 MB): L2 flushed (256 MB write) before each separately "
                   "timed step" % (gbytes / 1e6))}


def setup_workload(cfg, device_grid=True, seed=0):
    N, nb, L = cfg["N"], cfg["nbins"], cfg["L"]
    count, keff_grid = W.geometry(N, nb)
    m = count > 0
    kphys = keff_grid[m] * 2 * math.pi / L
    sf, dt = W.history(kphys, cfg["Na"], cfg["a_end"])
    logk, T = W.transfer_table(float(sum(cfg["MNu"])))
    return dict(kphys=kphys, sf=sf, dt=dt, logk=logk, T=T, nk=int(m.sum()))


def time_max(cfg, nsteps):
    """TimeMax sizing the history table (namax = ceil(100 (TimeMax - a0)) + 2,
    delta_tot_table.c:36) for the synthetic history plus the steps run."""
    return 0.01 + (cfg["Na"] + nsteps + 6) / 100.0


def step_times(cfg, w, steps):
    """Scale factors: the first call at a_end+0.01 commits a row; later calls advance
    by 0.001 (provisional row dropped), so each timed step does the same work."""
    a0 = cfg["a_end"] + 0.01
    return [a0 + 0.001 * i for i in range(steps)]


def plain_steps(k, cfg, grid, slab0, nslab, stream, a_list, warmup, steps, world=1):
    """Device-timed steps with the grid resident in HBM: returns (seconds, stage ms [4],
    launches per step).  A grid smaller than L2 is timed step by step after an L2 flush.
    The timed loop holds the calls alone; the per-stage times come from a separate pass
    of up to 5 more calls with the library's stage events on."""
    import torch
    N, L = cfg["N"], cfg["L"]
    for i in range(warmup):
        k.add_nu_power_to_rhogrid(a_list[i], L, grid, N, slab0, nslab)
    torch.cuda.synchronize()
    launches0 = k.launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    bytes_grid = 8 * grid.numel()
    flush = torch.empty(32 * 1024 * 1024, dtype=torch.float64, device="cuda") if bytes_grid < 160e6 else None
    if flush is None:
        ev0.record(stream)
        for i in range(steps):
            k.add_nu_power_to_rhogrid(a_list[warmup + i], L, grid, N, slab0, nslab)
        ev1.record(stream)
        torch.cuda.synchronize()
        t_dev = ev0.elapsed_time(ev1) / 1e3
    else:
        t_dev = 0.0
        for i in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            ev0.record(stream)
            k.add_nu_power_to_rhogrid(a_list[warmup + i], L, grid, N, slab0, nslab)
            ev1.record(stream)
            torch.cuda.synchronize()
            t_dev += ev0.elapsed_time(ev1) / 1e3
    launches = (k.launch_count() - launches0) / steps
    # stage times: later scale factors (each call still drops its provisional row)
    k.set_profiling(True)
    stage = np.zeros(4)
    n_stage = min(steps, 5)
    for j in range(n_stage):
        if flush is not None:
            with torch.cuda.stream(stream):
                flush.zero_()
        k.add_nu_power_to_rhogrid(a_list[-1] + 0.0005 + 0.001 * j, L, grid, N, slab0, nslab)
        stage += np.array(k.stage_times())
    k.set_profiling(False)
    return t_dev, stage / n_stage, launches


def link_bandwidth(nbytes, reps=3):
    """Plain pinned-memory copies of nbytes each way over the host link (cudaMemcpyAsync
    through torch), best of reps: the ceiling of an end-to-end step that moves the grid
    up and back."""
    import torch
    h = torch.empty(nbytes // 4, dtype=torch.float32, pin_memory=True)
    d = torch.empty(nbytes // 4, dtype=torch.float32, device="cuda")
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    best_up, best_down = 1e30, 1e30
    for _ in range(reps):
        torch.cuda.synchronize()
        ev0.record()
        d.copy_(h, non_blocking=True)
        ev1.record()
        torch.cuda.synchronize()
        best_up = min(best_up, ev0.elapsed_time(ev1) / 1e3)
        ev0.record()
        h.copy_(d, non_blocking=True)
        ev1.record()
        torch.cuda.synchronize()
        best_down = min(best_down, ev0.elapsed_time(ev1) / 1e3)
    del h, d
    return {"h2d_gbs": nbytes / best_up / 1e9, "d2h_gbs": nbytes / best_down / 1e9,
            "up_and_down_ms": 1e3 * (best_up + best_down)}


def run_gb300(args, cfg):
    import torch
    import kspace_gpu as kg
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    N, nb, L = cfg["N"], cfg["nbins"], cfg["L"]
    nz = N // 2 + 1
    slab0 = N * rank // world
    nslab = N * (rank + 1) // world - slab0
    wl = setup_workload(cfg)
    nsteps = args.warmup + args.steps
    TimeMax = time_max(cfg, 3 * nsteps + 4)
    k = kg.make_instance(cfg["MNu"], 0.01, 0.7, 0.3, nb, TimeMax, wl["logk"], wl["T"],
                         UnitLength_in_cm=W.UNIT_LENGTH_MPC, device=local)
    k.set_nu_state(wl["sf"], wl["dt"])
    stream = torch.cuda.Stream()
    k.set_stream(stream)
    if world > 1:
        import torch.distributed as dist

        def allreduce(buf):
            t = torch.from_numpy(buf.copy()).cuda()
            dist.all_reduce(t)
            buf[:] = t.cpu().numpy()
        k.set_allreduce(allreduce)
    full = W.make_grid_torch(N, L, seed=1, device="cuda")
    grid = full[slab0:slab0 + nslab].contiguous()
    del full
    G = nslab * N * nz
    bytes_grid = 8 * G
    a_list = step_times(cfg, None, nsteps)
    with clock_sampler(local) as clk:
        t_dev, stage, launches = plain_steps(k, cfg, grid, slab0, nslab, stream, a_list, args.warmup, args.steps,
                                             world)
    if world > 1:
        tt = torch.tensor([t_dev], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_dev = float(tt.item())
    ms_per_step = 1e3 * t_dev / args.steps
    value = N * N * nz * args.steps / t_dev
    # the same steps with the lean binning (tuning tma=6: FP32 run sums), for comparison;
    # the default reproduces the reference's float roundings, which delta_nu's 1e-10 bar
    # needs (errors of both in the `errors` key).  Scale factors keep increasing.
    a_next = a_list[-1] + 0.005  # past the stage pass's calls
    lean = None
    if rank == 0 and world == 1 and not args.no_extras:
        a_lean = [a_next + 0.001 * i for i in range(nsteps)]
        tma_default = int(os.environ.get("KSPACE_GPU_TMA", "5"))
        k.set_tuning(tma=6)
        t_l, stage_l, _ = plain_steps(k, cfg, grid, slab0, nslab, stream, a_lean, args.warmup, args.steps)
        k.set_tuning(tma=tma_default)
        ms_l = 1e3 * t_l / args.steps
        hbm_l, _ = peaks()
        lean = {"tuning": "tma=6 (FP32 run sums)", "ms_per_step": ms_l,
                "hbm_frac_step": 3 * bytes_grid / (ms_l * 1e-3) / 1e9 / hbm_l,
                "stage_ms": {"binning_K1": stage_l[0], "integrator_K2": stage_l[1], "correction_K3": stage_l[2]}}
        a_next = a_lean[-1] + 0.005
    # e2e through the C ABI with host buffers (pinned)
    host = torch.empty((nslab, N, nz), dtype=torch.complex64, pin_memory=True)
    host.copy_(grid.cpu())
    del grid
    torch.cuda.empty_cache()
    a_e2e = [a_next + 0.001 * i for i in range(args.warmup + args.steps)]
    for i in range(args.warmup):
        k.add_nu_power_to_rhogrid(a_e2e[i], L, host.numpy(), N, slab0, nslab)
    torch.cuda.synchronize()
    # each call returns with the corrected grid back in host memory; the per-call times
    # are kept as well, since the host link is shared with the other GPUs of the node and
    # a single call now and then takes several times the usual
    step_s = []
    t0 = time.perf_counter()
    for i in range(args.steps):
        t1 = time.perf_counter()
        k.add_nu_power_to_rhogrid(a_e2e[args.warmup + i], L, host.numpy(), N, slab0, nslab)
        step_s.append(time.perf_counter() - t1)
    t_e2e = time.perf_counter() - t0
    if world > 1:
        tt = torch.tensor([t_e2e], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_e2e = float(tt.item())
    e2e_value = N * N * nz * args.steps / t_e2e
    step_ms = sorted(1e3 * x for x in step_s)
    e2e_steps = {"median": step_ms[len(step_ms) // 2], "min": step_ms[0], "max": step_ms[-1],
                 "in_order": [round(1e3 * x, 2) for x in step_s]}
    del host
    link = link_bandwidth(bytes_grid) if rank == 0 else None
    # roofline of the dominant grid kernel
    hbm, peak_kind = peaks()
    k1_ms, k2_ms, k3_ms = stage[0], stage[1], stage[2]
    k1_gbs = bytes_grid / (k1_ms * 1e-3) / 1e9 if k1_ms > 0 else None
    k3_gbs = 2 * bytes_grid / (k3_ms * 1e-3) / 1e9 if k3_ms > 0 else None
    tma = int(os.environ.get("KSPACE_GPU_TMA", "5"))
    # the mirrored-row binning pass where a grid row is at most 32 runs of 17 modes
    mirror = tma >= 5 and os.environ.get("KSPACE_GPU_MIRROR", "1") != "0" and (nz + 16) // 17 <= 32
    k1_name = ("k_bin_mirror" if mirror else "k_bin_rows") if tma >= 5 else (
        "k_bin_stream" if tma >= 3 else "k_bin_power_tma")
    k3_name = "k_correct_stream" if tma >= 3 else "k_correct_tma"
    if k3_ms >= k1_ms:
        dom = {"kernel": k3_name + " (grid multiply)", "bytes": 2 * bytes_grid, "ms": k3_ms, "gbs": k3_gbs}
    else:
        dom = {"kernel": k1_name + " (binning)", "bytes": bytes_grid, "ms": k1_ms, "gbs": k1_gbs}
    traffic, traffic_note = None, None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            tj = json.load(f)
        ref_bytes = tj.get("captured_grid_bytes", 538968064)
        traffic = tj.get(dom["kernel"].split()[0])
        if traffic is not None and bytes_grid != ref_bytes:
            # captured on a smaller grid; DRAM bytes scale with the grid
            traffic = traffic * bytes_grid / ref_bytes
            traffic_note = "ncu capture at %d grid bytes scaled by the grid size" % ref_bytes
    except Exception:
        pass
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "strong" if world > 1 else "weak", "vs_baseline": None, "dtype": "c64 grid / f64 integrator",
        "data": "synthetic (seeded Gaussian modes with the configured P(k); no dataset)",
        "config": bench_config(cfg),
        "parallelism": "slabs over %d ranks" % world if world > 1 else "single GPU",
        "hbm_gbs_step": 3 * bytes_grid / (ms_per_step * 1e-3) / 1e9,
        "hbm_frac_step": 3 * bytes_grid / (ms_per_step * 1e-3) / 1e9 / hbm,
        "stage_ms": {"binning_K1": k1_ms, "integrator_K2": k2_ms, "correction_K3": k3_ms, "whole_call": stage[3]},
        "stage_gbs": {"K1": k1_gbs, "K3": k3_gbs},
        "stage_kernels": {"K1": k1_name, "K2": "k_dnu_qag_blk (+ k_dtot_coeffs, k_combine, k_finish)", "K3": k3_name},
        "stage_frac": {"K1": (k1_gbs / hbm) if k1_gbs else None, "K3": (k3_gbs / hbm) if k3_gbs else None},
        "roofline": {"bound": "hbm", "kernel": dom["kernel"], "achieved": dom["gbs"], "peak": hbm,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": (dom["gbs"] / hbm) if dom["gbs"] else None,
                     "traffic": traffic, "traffic_note": traffic_note, "algorithmic_bytes_per_launch": dom["bytes"]},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": bytes_grid,
                "d2h_bytes_per_step": bytes_grid, "ms_per_step": 1e3 * t_e2e / args.steps,
                "per_call_ms": e2e_steps, "value_at_median_call": N * N * nz / (1e-3 * e2e_steps["median"])},
        "gpu_launches": int(round(launches * args.steps)),
        "clocks": clk.summary(),
    }
    if link:
        res["e2e"]["link"] = link
        res["e2e"]["frac_of_link"] = link["up_and_down_ms"] / res["e2e"]["ms_per_step"]
        res["e2e"]["frac_of_link_at_median_call"] = link["up_and_down_ms"] / e2e_steps["median"]
    if rank == 0 and not args.no_cpu_baseline:
        res["cpu_baseline"] = cpu_baseline(cfg, wl, args.cpu_threads, sample_steps=1)
    k.close()
    if lean:
        res["lean_binning"] = lean
    if rank == 0 and world == 1 and not args.no_extras:
        res["errors"] = errors_vs_oracle(cfg, wl, args.cpu_threads or os.cpu_count() or 1)
        if cfg["name"] != "cfg1_n512":
            res["n512"] = n512_steps(args)
        res["fwd_adjoint"] = fwd_adjoint()
        b = run_batch(args, dict(W.BATCH))
        res["batch"] = {k_: b[k_] for k_ in ("config", "value", "unit", "ms_per_step", "e2e", "per_instance_calls",
                                             "agreement_vs_per_instance", "agreement_vs_oracle", "autotune")}
    if world > 1:
        dist.destroy_process_group()
    return res if rank == 0 else None


def n512_steps(args):
    """The N=512 configuration (512x512x257, 256 bins, 256-row history, 3 x 0.1 eV):
    device-timed steps and stage times, as for the main workload."""
    import torch
    import kspace_gpu as kg
    cfg = dict(W.CONFIGS["cfg1_n512"])
    cfg["name"] = "cfg1_n512"
    N, nb, L = cfg["N"], cfg["nbins"], cfg["L"]
    wl = setup_workload(cfg)
    nsteps = args.warmup + args.steps
    k = kg.make_instance(cfg["MNu"], 0.01, 0.7, 0.3, nb, time_max(cfg, 2 * nsteps + 2), wl["logk"], wl["T"],
                         UnitLength_in_cm=W.UNIT_LENGTH_MPC)
    k.set_nu_state(wl["sf"], wl["dt"])
    stream = torch.cuda.Stream()
    k.set_stream(stream)
    grid = W.make_grid_torch(N, L, seed=1, device="cuda")
    with clock_sampler(0) as clk:
        t_dev, stage, _ = plain_steps(k, cfg, grid, 0, N, stream, step_times(cfg, None, nsteps), args.warmup,
                                      args.steps)
    k.close()
    hbm, _ = peaks()
    gb = 8 * grid.numel()
    ms = 1e3 * t_dev / args.steps
    return {"config": bench_config(cfg), "value": N * N * (N // 2 + 1) / (ms * 1e-3), "unit": UNIT,
            "ms_per_step": ms, "hbm_frac_step": 3 * gb / (ms * 1e-3) / 1e9 / hbm,
            "stage_ms": {"binning_K1": stage[0], "integrator_K2": stage[1], "correction_K3": stage[2]},
            "stage_frac": {"K1": gb / (stage[0] * 1e-3) / 1e9 / hbm, "K3": 2 * gb / (stage[2] * 1e-3) / 1e9 / hbm},
            "clocks": clk.summary()}


def fwd_adjoint(steps=5, warmup=3):
    """The differentiation workload (N=256, 128 bins, 128-row history, sum M_nu=0.15 eV):
    device time of the plain step against the forward + adjoint step (store and
    recompute variants), grid resident in HBM."""
    import torch
    import kspace_gpu as kg
    cfg = dict(W.CONFIGS["cfg3_n256"])
    N, nb, L = cfg["N"], cfg["nbins"], cfg["L"]
    wl = setup_workload(cfg)
    k = kg.make_instance(cfg["MNu"], 0.01, 0.7, 0.3, nb, time_max(cfg, 2 * (steps + warmup) + 4), wl["logk"],
                         wl["T"], UnitLength_in_cm=W.UNIT_LENGTH_MPC)
    k.set_nu_state(wl["sf"], wl["dt"])
    grid = W.make_grid_torch(N, L, seed=3)
    work = grid.clone()
    a = cfg["a_end"] + 0.01
    k.add_nu_power_to_rhogrid(a, L, work, N)  # initialisation + one committed row
    nk = k.table_info()["nk"]

    def timed(fn, n):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(n):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / n

    state = {"a": a}

    def plain():
        state["a"] += 0.001
        work.copy_(grid)
        k.add_nu_power_to_rhogrid(state["a"], L, work, N)

    out = torch.empty_like(grid)
    pnu = torch.empty(nk, dtype=torch.float64, device="cuda")
    gin = torch.empty_like(grid)
    gbar = torch.randn(grid.shape, dtype=torch.complex64, device="cuda")
    pbar = torch.rand(nk, dtype=torch.float64, device="cuda")
    Dbar = torch.empty((nk, k.table_info()["ia"]), dtype=torch.float64, device="cuda")
    ad = state["a"] + 0.005

    def fa(recompute):
        def run():
            k.diff_forward(ad, L, grid, out, N, pnu, store_intervals=not recompute)
            k.diff_backward(gbar, grid, pbar, gin, Dbar, recompute=recompute)
        return run

    def copy_only():
        work.copy_(grid)

    for f in (plain, fa(False), fa(True)):
        for _ in range(warmup):
            f()
    t_copy = timed(copy_only, steps)
    t_plain = timed(plain, steps) - t_copy
    t_store = timed(fa(False), steps)
    t_rec = timed(fa(True), steps)
    k.close()
    return {"workload": "cfg3_n256 (N=256, 128 bins, 128-row history, sum M_nu=0.15 eV)",
            "plain_ms": 1e3 * t_plain, "fwd_adj_store_ms": 1e3 * t_store, "fwd_adj_recompute_ms": 1e3 * t_rec,
            "ratio_store": t_store / t_plain, "ratio_recompute": t_rec / t_plain,
            "timing": "host clock around synchronous calls, %d steps after %d warm-up" % (steps, warmup)}


def errors_vs_oracle(cfg, wl, threads):
    """One step on a fresh instance and on the oracle (the reference algorithm in C), and
    on the all-FP64 oracle (double |F|^2 and window, exact delta_nu integral): per-bin
    mode counts (bit for bit) and max relative differences of P(k), delta_nu,
    delta_nu/delta_cdm and the corrected grid.  The same step with the lean binning
    (tuning tma=6) against the reference oracle, under `lean_binning`."""
    import torch
    import kspace_gpu as kg
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Oracle
    O = Oracle()
    N, nb, L = cfg["N"], cfg["nbins"], cfg["L"]
    TimeMax = time_max(cfg, 4)
    a = cfg["a_end"] + 0.01
    g = host_grid(N, L, 1)

    def gpu_step(tma):
        k = kg.make_instance(cfg["MNu"], 0.01, 0.7, 0.3, nb, TimeMax, wl["logk"], wl["T"],
                             UnitLength_in_cm=W.UNIT_LENGTH_MPC)
        k.set_tuning(tma=tma)
        k.set_nu_state(wl["sf"], wl["dt"])
        gd = torch.as_tensor(g).cuda()
        nk_g, p_g, c_g, _ = k.total_powerspectrum(N, gd, nb)
        k.add_nu_power_to_rhogrid(a, L, gd, N)
        lc = k.last_correction()
        gg = gd.cpu().numpy()
        del gd
        k.close()
        torch.cuda.empty_cache()
        return nk_g, c_g, lc, gg

    def errs(lc, gg, out, go):
        m = out["ratio"] != 0
        dnu_g = lc["ratio"] * lc["dcdm"]
        return {
            "P_k": float(np.max(np.abs((lc["dcdm"] / out["dcdm"]) ** 2 - 1))),
            "delta_nu": float(np.max(np.abs(dnu_g[m] / out["dnu"][m] - 1))),
            "delta_nu_over_delta_cdm": float(np.max(np.abs(lc["ratio"][m] / out["ratio"][m] - 1))),
            "corrected_grid": float(np.max(np.abs(gg - go) / np.maximum(np.abs(go), 1e-30))),
        }

    tma_default = int(os.environ.get("KSPACE_GPU_TMA", "5"))
    nk_g, c_g, lc, gg = gpu_step(tma_default)
    nk_o, p_o, c_o, _ = O.total_powerspectrum(g, N, nb, nthreads=threads)
    res = {"counts_equal": bool(nk_g == nk_o and np.array_equal(c_g, c_o)), "nk": int(nk_o),
           "modes_binned": int(c_o.sum())}
    for name, exact in (("vs_reference_oracle", 0), ("vs_fp64_oracle", 1)):
        bg = O.bg(cfg["MNu"], a0=0.01, h=0.7, Omega0=0.3, UnitTime_in_s=W.UNIT_TIME)
        s = O.state(bg, nb, 0.01, TimeMax, Omega0=0.3, UnitTime_in_s=W.UNIT_TIME, UnitLength_in_cm=W.UNIT_LENGTH_MPC)
        O.set_transfer(s, wl["logk"], wl["T"])
        assert O.set_nu_state(s, wl["sf"], wl["dt"]) == 0
        O.L.ko_state_options(s, 0, exact)
        if exact:
            st, out, go = O.add_nu_power_to_rhogrid_fp64(s, a, L, g, N, nthreads=threads, nk_alloc=nb)
        else:
            go = g.copy()
            st, out = O.add_nu_power_to_rhogrid(s, a, L, go, N, nthreads=threads, nk_alloc=nb)
        assert st == 0, st
        res[name] = errs(lc, gg, out, go)
        if not exact:
            nk_l, c_l, lc_l, gg_l = gpu_step(6)
            res["lean_binning"] = {"tuning": "tma=6 (FP32 run sums)",
                                   "counts_equal": bool(nk_l == nk_o and np.array_equal(c_l, c_o)),
                                   "vs_reference_oracle": errs(lc_l, gg_l, out, go)}
            del gg_l
        del go
    res["bars"] = {"counts": "bit-exact", "P_k": 1e-6, "corrected_grid": 1e-6, "delta_nu": 1e-10}
    return res


def cpu_baseline(cfg, wl, threads, sample_steps=1):
    """The oracle port (the reference algorithm restated in C) on the host cores."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Oracle
    O = Oracle()
    threads = threads or os.cpu_count() or 1
    N, nb, L = cfg["N"], cfg["nbins"], cfg["L"]
    bg = O.bg(cfg["MNu"], a0=0.01, h=0.7, Omega0=0.3, UnitTime_in_s=W.UNIT_TIME)
    TimeMax = time_max(cfg, sample_steps + 2)
    s = O.state(bg, nb, 0.01, TimeMax, Omega0=0.3, UnitTime_in_s=W.UNIT_TIME, UnitLength_in_cm=W.UNIT_LENGTH_MPC)
    O.set_transfer(s, wl["logk"], wl["T"])
    assert O.set_nu_state(s, wl["sf"], wl["dt"]) == 0
    g = host_grid(N, L, 1).copy()
    # initialisation call (delta_nu_last) is not timed, as on the GPU
    st, _ = O.add_nu_power_to_rhogrid(s, cfg["a_end"] + 0.01, L, g, N, nthreads=threads, nk_alloc=nb)
    assert st == 0, st
    G = g.size
    t0 = time.perf_counter()
    stages = np.zeros(3)
    for i in range(sample_steps):
        st, out = O.add_nu_power_to_rhogrid(s, cfg["a_end"] + 0.011 + 0.001 * i, L, g, N, nthreads=threads,
                                            nk_alloc=nb)
        assert st == 0, st
        stages += out["t_stages"]
    dt = time.perf_counter() - t0
    return {"value": G * sample_steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d full step(s) of the same N=%d workload (grid binning and multiply split over %d threads "
                      "as MPI slabs; integrator once)" % (sample_steps, N, threads),
            "stage_s": {"binning": stages[0] / sample_steps, "integrator": stages[1] / sample_steps,
                        "multiply": stages[2] / sample_steps}}


def run_reference(args, cfg):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    wl = setup_workload(cfg)
    threads = args.cpu_threads or os.cpu_count() or 1
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Oracle
    O = Oracle()
    N, nb, L = cfg["N"], cfg["nbins"], cfg["L"]
    bg = O.bg(cfg["MNu"], a0=0.01, h=0.7, Omega0=0.3, UnitTime_in_s=W.UNIT_TIME)
    nsteps = args.warmup + args.steps
    TimeMax = time_max(cfg, nsteps)
    s = O.state(bg, nb, 0.01, TimeMax, Omega0=0.3, UnitTime_in_s=W.UNIT_TIME, UnitLength_in_cm=W.UNIT_LENGTH_MPC)
    O.set_transfer(s, wl["logk"], wl["T"])
    assert O.set_nu_state(s, wl["sf"], wl["dt"]) == 0
    g = host_grid(N, L, 1).copy()
    a_list = step_times(cfg, None, nsteps)
    for i in range(args.warmup):
        st, _ = O.add_nu_power_to_rhogrid(s, a_list[i], L, g, N, nthreads=threads, nk_alloc=nb)
        assert st == 0, st
    t0 = time.perf_counter()
    for i in range(args.steps):
        st, _ = O.add_nu_power_to_rhogrid(s, a_list[args.warmup + i], L, g, N, nthreads=threads, nk_alloc=nb)
        assert st == 0, st
    dt = time.perf_counter() - t0
    v = g.size * args.steps / dt
    return {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64 grid / f64 integrator", "data": "synthetic",
            "config": bench_config(cfg),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "the full N=%d step, %d timed steps, binning/multiply split over %d threads "
                                       "as MPI slabs" % (N, args.steps, threads)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def make_batch_sets(kg, M, G, seed, nsets, nbins_grid, L, extra_rows):
    """nsets identical sets of M free instances + G grid-bound instances."""
    import torch
    ps = W.batch_instances(M, seed=seed)
    Ns = W.batch_grid_sizes(G, seed=seed)
    gps = W.batch_instances(G, seed=seed + 1)
    sets = []
    for _ in range(nsets):
        insts, kph = [], []
        for p in ps:
            logk, T = W.transfer_table(float(sum(p["MNu"])))
            k = kg.make_instance(p["MNu"], 0.01, p["h"], p["Omega0"], p["nk"], 0.01 + (p["Na"] + extra_rows) / 100.0,
                                 logk, T, UnitLength_in_cm=W.UNIT_LENGTH_MPC)
            sf, dt = W.history(p["k"], p["Na"], p["a_end"])
            k.set_nu_state(sf, dt)
            insts.append(k)
            kph.append(p["k"])
        grids = []
        for j, (p, N) in enumerate(zip(gps, Ns)):
            count, keff = W.geometry(N, nbins_grid)
            kp = keff[count > 0] * 2 * math.pi / L
            logk, T = W.transfer_table(float(sum(p["MNu"])))
            k = kg.make_instance(p["MNu"], 0.01, p["h"], p["Omega0"], nbins_grid,
                                 0.01 + (p["Na"] + extra_rows) / 100.0, logk, T, UnitLength_in_cm=W.UNIT_LENGTH_MPC)
            sf, dt = W.history(kp, p["Na"], p["a_end"])
            k.set_nu_state(sf, dt)
            insts.append(k)
            kph.append(kp)
            grids.append(W.make_grid_torch(N, L, seed=100 + j))
        torch.cuda.synchronize()
        sets.append(dict(insts=insts, kph=kph, grids=grids, Ns=Ns))
    return sets, ps


def run_batch(args, cfg):
    """Batched integration: M independent instances + G grids advanced per call by one
    CUDA graph, against the same instances driven one call per instance."""
    import torch
    import kspace_gpu as kg
    torch.cuda.set_device(0)
    M, G, L, nbg = args.batch_m, cfg["grids"], cfg["L"], cfg["nbins_grid"]
    nsteps = args.warmup + args.steps
    t_setup = time.perf_counter()
    sets, ps = make_batch_sets(kg, M, G, 0, 2, nbg, L, nsteps + 8)
    t_setup = time.perf_counter() - t_setup
    A, T = sets
    MT = M + G
    B = kg.KspaceBatch(A["insts"])
    for j in range(G):
        B.bind_grid(M + j, A["grids"][j], A["Ns"][j], L)
    nk = np.array([len(A["kph"][i]) for i in range(M)] + [0] * G, dtype=np.int32)
    keff = np.concatenate(A["kph"][:M])
    dc0 = np.sqrt(W.spectrum(keff))
    a_end = cfg["a_end"]
    a_list = [a_end + 0.01 + 0.001 * i for i in range(nsteps)]
    # first call at the first step's a (delta_tot_init keeps the rows before it), as the
    # single-instance path does on its first get_delta_nu_update
    B.init(np.full(MT, a_list[0]), nk, keff, dc0)
    off = B.offsets
    nbins_total = int(off[-1])
    # per-step inputs: the generator's delta_cdm grown linearly with a
    dcdm_h = torch.empty(nbins_total, dtype=torch.float64, pin_memory=True)
    dnu_h = torch.empty(nbins_total, dtype=torch.float64, pin_memory=True)
    base = np.zeros(nbins_total)
    for i in range(M):
        base[off[i]:off[i + 1]] = np.sqrt(W.spectrum(A["kph"][i]))
    tune = None
    if args.autotune:
        dcdm_h.copy_(torch.from_numpy(base * a_list[0] / a_end))
        tune = B.autotune(np.full(MT, a_list[0]), dcdm_h, reps=2)
    dev_ms, host_s, outs = [], [], []
    with clock_sampler(0) as clk:
        for i in range(nsteps):
            dcdm_h.copy_(torch.from_numpy(base * a_list[i] / a_end))
            t0 = time.perf_counter()
            B.step(np.full(MT, a_list[i]), dcdm_h, dnu_h)
            t1 = time.perf_counter()
            if i >= args.warmup:
                dev_ms.append(B.last_ms())
                host_s.append(t1 - t0)
            outs.append(dnu_h.numpy().copy())
    t_dev = sum(dev_ms) / 1e3
    t_host = sum(host_s)
    # the same instances, one call per instance (the same scale factors and inputs)
    per_s = []
    worst = 0.0
    n_cmp = min(nsteps, args.warmup + 1)
    for i in range(n_cmp):
        d = base * a_list[i] / a_end
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = []
        for j in range(MT):
            k = T["insts"][j]
            if j < M:
                res.append(k.get_delta_nu_update(a_list[i], T["kph"][j], d[off[j]:off[j + 1]]))
            else:
                k.add_nu_power_to_rhogrid(a_list[i], L, T["grids"][j - M], T["Ns"][j - M])
                res.append(None)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        if i >= args.warmup:
            per_s.append(t1 - t0)
        for j in range(M):
            r = res[j]
            g = outs[i][off[j]:off[j + 1]]
            nz = np.abs(r) > 0
            if nz.any():
                worst = max(worst, float(np.max(np.abs(g[nz] - r[nz]) / np.abs(r[nz]))))
    per_solves = MT / (sum(per_s) / len(per_s)) if per_s else None
    # a sample of the free instances against the oracle (the reference algorithm in C),
    # driven through the same get_delta_nu_update sequence
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Oracle
    O = Oracle()
    worst_oracle = 0.0
    sample = sorted(set([0, M // 4, M // 2, (3 * M) // 4, M - 1]))
    for j in sample:
        p = ps[j]
        logk, Tt = W.transfer_table(float(sum(p["MNu"])))
        ut = W.UNIT_LENGTH_MPC / 1e5
        bg = O.bg(p["MNu"], a0=0.01, h=p["h"], Omega0=p["Omega0"], UnitTime_in_s=ut)
        st_o = O.state(bg, p["nk"], 0.01, 0.01 + (p["Na"] + nsteps + 8) / 100.0, Omega0=p["Omega0"],
                       UnitTime_in_s=ut, UnitLength_in_cm=W.UNIT_LENGTH_MPC)
        O.set_transfer(st_o, logk, Tt)
        sf, dt = W.history(p["k"], p["Na"], p["a_end"])
        assert O.set_nu_state(st_o, sf, dt) == 0
        for i in range(n_cmp):
            d = base * a_list[i] / a_end
            rc, r = O.get_delta_nu_update(st_o, a_list[i], A["kph"][j], d[off[j]:off[j + 1]])
            assert rc == 0, rc
            g = outs[i][off[j]:off[j + 1]]
            nz = np.abs(r) > 0
            if nz.any():
                worst_oracle = max(worst_oracle, float(np.max(np.abs(g[nz] - r[nz]) / np.abs(r[nz]))))
    value = MT * args.steps / t_dev
    e2e = MT * args.steps / t_host
    Na = np.array([p["Na"] for p in ps])
    nks = np.array([p["nk"] for p in ps])
    res = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 integrator / c64 grids",
        "data": "synthetic (seeded per-instance cosmologies, histories and grids; no dataset)",
        "config": {"workload": "batch_m%d_g%d" % (M, G), "instances": M, "grids": G, "grid_N": A["Ns"],
                   "nbins_grid": nbg, "history_rows": [int(Na.min()), int(Na.max()), float(Na.mean())],
                   "bins": [int(nks.min()), int(nks.max()), float(nks.mean())],
                   "l2": "history tables %.1f GB (larger than L2): no flush" % (
                       sum(8.0 * 2 * p["nk"] * (p["Na"] + 2) for p in ps) / 1e9)},
        "per_instance_calls": {"solves_per_s": per_solves, "steps_timed": len(per_s),
                               "speedup_batched_device": (value / per_solves) if per_solves else None,
                               "speedup_batched_e2e": (e2e / per_solves) if per_solves else None},
        "agreement_vs_per_instance": {"max_rel": worst, "steps_compared": n_cmp, "bar": 1e-10},
        "agreement_vs_oracle": {"max_rel": worst_oracle, "instances": sample, "steps_compared": n_cmp, "bar": 1e-10},
        "autotune": {"warps_per_block_blocks_per_sm": tune[0], "ms": tune[1]} if tune else None,
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": 8 * nbins_total,
                "d2h_bytes_per_step": 8 * nbins_total},
        "gpu_launches": args.steps * (8 + 3 * G),
        "setup_s": t_setup,
        "clocks": clk.summary(),
    }
    B.close()
    for s_ in sets:
        for k in s_["insts"]:
            k.close()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="cfg2_n1024", choices=sorted(W.CONFIGS) + ["batch"])
    ap.add_argument("--batch-m", type=int, default=W.BATCH["M"])
    ap.add_argument("--autotune", type=int, default=1)
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the fwd+adjoint and error measurements")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.config == "batch":
        res = run_batch(args, dict(W.BATCH)) if args.impl == "gb300" else None
        if res is not None:
            print(json.dumps(res))
        return
    cfg = dict(W.CONFIGS[args.config])
    cfg["name"] = args.config
    if args.impl == "reference":
        res = run_reference(args, cfg)
    else:
        res = run_gb300(args, cfg)
    if res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
