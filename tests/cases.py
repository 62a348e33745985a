"""Shared set-up of a synthetic PM step for the checker (oracle) and the GPU library."""
import math

import numpy as np

import workloads as W

UL = W.UNIT_LENGTH_MPC
UT = W.UNIT_TIME


def make_case(N, nbins, Na, a_end, MNu, L=512.0, Omega0=0.3, h=0.7, seed=0, extra_rows=12, grid=True):
    count, keff_grid = W.geometry(N, nbins)
    m = count > 0
    kphys = keff_grid[m] * 2 * math.pi / L
    sf, dt = W.history(kphys, Na, a_end)
    logk, T = W.transfer_table(float(sum(MNu)))
    TimeMax = 0.01 + (Na + extra_rows) / 100.0
    c = dict(N=N, nbins=nbins, Na=Na, a_end=a_end, MNu=tuple(MNu), L=L, Omega0=Omega0, h=h, count=count[m],
             keff_grid=keff_grid[m], kphys=kphys, scalefact=sf, delta_tot=dt, logk=logk, T=T, TimeMax=TimeMax,
             nk=int(m.sum()))
    if grid:
        c["grid"] = W.make_grid(N, L, seed)
    return c


def oracle_state(O, c, fs_mode=0, exact=0):
    bg = O.bg(c["MNu"], a0=0.01, h=c["h"], Omega0=c["Omega0"], UnitTime_in_s=UT)
    s = O.state(bg, c["nbins"], 0.01, c["TimeMax"], Omega0=c["Omega0"], UnitTime_in_s=UT, UnitLength_in_cm=UL)
    O.set_transfer(s, c["logk"], c["T"])
    O.set_nu_state(s, c["scalefact"], c["delta_tot"])
    O.L.ko_state_options(s, fs_mode, exact)
    return bg, s


def gpu_instance(kg, c, device=0):
    k = kg.make_instance(c["MNu"], 0.01, c["h"], c["Omega0"], c["nbins"], c["TimeMax"], c["logk"], c["T"],
                         UnitLength_in_cm=UL, device=device)
    k.set_nu_state(c["scalefact"], c["delta_tot"])
    return k


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.abs(a - b)
    s = np.maximum(np.abs(b), 1e-300)
    return float(np.max(d / s)) if d.size else 0.0
