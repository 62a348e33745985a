"""FP64 reference of the differentiable step and of its adjoint (test infrastructure).

The step (see kspace-neutrinos_gb300/autograd.py): bin the grid, integrate delta_nu with
the provisional history row (state fixed), correct every mode.  Everything here is in
float64 except the per-mode CIC window factor, which is part of the function's
definition (the reference forms it in float, powerspectrum.c:16-24).  The integrator
and its adjoint come from the C oracle (ko_dnu_diff).  Finite differences are evaluated
as structured differences (only the terms that change), so a relative step of 1e-6 in
FP64 is not swamped by the round-off of an 8-million-term sum.
"""
import ctypes as C
import math

import numpy as np

import workloads as W

P = C.POINTER(C.c_double)


def _p(a):
    return a.ctypes.data_as(P)


def bind(O):
    L = O.L
    L.ko_state_set_vectors.argtypes = [C.c_void_p, P, P, P, C.c_int]
    L.ko_state_set_vectors.restype = C.c_int
    L.ko_state_set_jmass.argtypes = [C.c_void_p, P]
    L.ko_state_set_jmass.restype = None
    L.ko_dnu_diff.argtypes = [C.c_void_p, C.c_double, P, P, P, P, P, P]
    L.ko_dnu_diff.restype = C.c_int


class StepRef:
    def __init__(self, O, bg, s, N, nbins, L, a, count, kphys, scalefact):
        bind(O)
        self.O, self.bg, self.s = O, bg, s
        self.N, self.L, self.a = N, L, a
        self.count = np.asarray(count, dtype=np.float64)
        self.kphys = np.ascontiguousarray(kphys)
        self.logk = np.log(self.kphys)
        self.sf = np.ascontiguousarray(scalefact)
        nz = N // 2 + 1
        kx = W.kval(np.arange(N), N).astype(np.int64)
        kz = np.arange(nz, dtype=np.int64)
        k2 = (kx[:, None, None] ** 2 + kx[None, :, None] ** 2 + kz[None, None, :] ** 2)
        self.k2 = k2.ravel()
        self.wt = np.where((kz == 0) | (kz == N // 2), 1.0, 2.0)[None, None, :] * np.ones((N, N, 1))
        self.wt = self.wt.ravel()
        # window factor as the reference forms it (float products)
        w1 = np.array([1.0 if k == 0 else math.pi * k / (N * math.sin(math.pi * k / np.float32(N))) for k in range(nz)],
                      dtype=np.float32)
        ax = np.abs(kx)
        t = (w1[ax][:, None, None] * w1[ax][None, :, None]).astype(np.float32) * w1[kz][None, None, :]
        t = t.astype(np.float32)
        inv = (t * t).astype(np.float32)
        self.W4 = (inv.astype(np.float64) ** 2).ravel()
        # reference bins of every k^2, and the compact index of non-empty bins
        bpu = (nbins - 1) / math.log(math.sqrt(3) * N / 2.0)
        kk = np.sqrt(np.maximum(self.k2, 1).astype(np.float64))
        b = np.floor(bpu * np.log(kk)).astype(np.int64)
        b[self.k2 == 0] = -1
        full = np.zeros(nbins, dtype=np.int64)
        np.add.at(full, b[b >= 0], 1)
        nonempty = np.nonzero(np.bincount(b[b >= 0], minlength=nbins))[0]
        cmap = -np.ones(nbins, dtype=np.int64)
        cmap[nonempty] = np.arange(len(nonempty))
        self.cb = np.where(b >= 0, cmap[np.maximum(b, 0)], -1)
        self.nk = len(nonempty)
        # unique k^2 with interpolation weights (double) of the correction
        self.uk2, self.uinv = np.unique(self.k2, return_inverse=True)
        xq = np.log(np.sqrt(self.uk2.astype(np.float64)) * 2 * math.pi / L, where=self.uk2 > 0,
                    out=np.zeros(len(self.uk2)))
        lk = self.logk
        xc = np.clip(xq, lk[0], lk[-1])
        j0 = np.clip(np.searchsorted(lk, xc, side="right") - 1, 0, len(lk) - 2)
        tt = (xc - lk[j0]) / (lk[j0 + 1] - lk[j0])
        self.j0, self.w0, self.w1 = j0, 1 - tt, tt
        self.udc = self.uk2 == 0
        bg_om = O.L.ko_omega_nu_nopart(bg, a)
        om = O.L.ko_omega_nu(bg, a)
        self.norm = bg_om / (O.scalars(s)["Omeganonu"] / a ** 3 + (om - bg_om))

    # ---- pieces
    def power(self, x, f32=False):
        if f32:  # |F|^2 formed in float, as the reference does (powerspectrum.c:66,74,82)
            xr = x.real.astype(np.float32)
            xi = x.imag.astype(np.float32)
            a2 = (xr * xr + xi * xi).astype(np.float64).ravel()
        else:
            a2 = (x.real ** 2 + x.imag ** 2).ravel()
        m = self.cb >= 0
        S = np.bincount(self.cb[m], weights=(self.wt * a2 * self.W4)[m], minlength=self.nk)
        F0 = float(a2[0])
        return S / (F0 * self.count), F0

    def dnu(self, dcdm, D, mJ, dnu_bar=None):
        O, s = self.O, self.s
        O.set_nu_state(s, self.sf, D)
        O.L.ko_state_set_jmass(s, _p(np.ascontiguousarray(mJ, dtype=np.float64)))
        out = np.zeros(self.nk)
        if dnu_bar is None:
            st = O.L.ko_dnu_diff(s, self.a, _p(self.kphys), _p(np.ascontiguousarray(dcdm)), _p(out), None, None, None)
            assert st == 0, st
            return out
        Na = len(self.sf) + 1
        Db = np.zeros(self.nk * Na)
        mb = np.zeros(3)
        st = O.L.ko_dnu_diff(s, self.a, _p(self.kphys), _p(np.ascontiguousarray(dcdm)), _p(out),
                             _p(np.ascontiguousarray(dnu_bar)), _p(Db), _p(mb))
        assert st == 0, st
        return out, Db.reshape(self.nk, Na), mb

    def smooth_u(self, r):
        """1 + norm*interp(r) per unique k^2 (1 at k=0)."""
        s = 1 + self.norm * (self.w0 * r[self.j0] + self.w1 * r[self.j0 + 1])
        s[self.udc] = 1.0
        return s

    # ---- forward
    def forward(self, x, D, mJ, wb, f32=False):
        P, F0 = self.power(x, f32)
        dc = np.sqrt(P * self.L ** 3)
        dnu = self.dnu(dc, D, mJ)
        out = np.maximum(dnu, 0)
        r = out / dc
        su = self.smooth_u(r)
        s = su[self.uinv]
        a2 = (x.real ** 2 + x.imag ** 2).ravel()
        loss = float(np.sum(wb * out ** 2) + 0.5 * np.sum(a2 * s * s))
        return dict(P=P, F0=F0, dc=dc, dnu=dnu, out=out, r=r, su=su, s=s, loss=loss)

    # ---- adjoint of L = sum w P_nu + 0.5 |y|^2
    def adjoint(self, x, D, mJ, wb, f=None):
        if f is None:
            f = self.forward(x, D, mJ, wb)
        xf = x.ravel()
        a2 = xf.real ** 2 + xf.imag ** 2
        # dL/ds_m = y_m . x_m = |x|^2 s ; rbar_j = norm sum dL/ds dinterp/dr_j
        g = a2 * f["s"]
        gu = np.bincount(self.uinv, weights=g, minlength=len(self.uk2))
        gu[self.udc] = 0.0
        rbar = self.norm * (np.bincount(self.j0, weights=gu * self.w0, minlength=self.nk) +
                            np.bincount(self.j0 + 1, weights=gu * self.w1, minlength=self.nk))
        out, dc, dnu = f["out"], f["dc"], f["dnu"]
        dnu_bar = np.where(dnu > 0, 2 * out * wb + rbar / dc, 0.0)
        _, Db, mb = self.dnu(dc, D, mJ, dnu_bar)
        Omeganonu = self.O.scalars(self.s)["Omeganonu"]
        bg = self.bg
        OmegaNua3 = self.O.L.ko_omega_nu_nopart(bg, self.a) * self.a ** 3
        OmegaNu1 = self.O.L.ko_omega_nu(bg, 1.0)
        fcdm = 1 - OmegaNua3 / (Omeganonu + OmegaNu1)
        dcbar = -rbar * out / dc ** 2 + Db[:, -1] * fcdm
        Pbar = dcbar * self.L ** 3 / (2 * dc)
        Q = 2 * Pbar / (f["F0"] * self.count)
        xbar = xf * f["s"] * f["s"]  # gbar = y = x s  ->  gbar * s
        m = self.cb >= 0
        xbar = xbar + np.where(m, Q[np.maximum(self.cb, 0)] * self.wt * self.W4, 0.0) * xf
        xbar[0] = xf[0] - 2 * np.sum(Pbar * f["P"]) / f["F0"] * xf[0]
        return dict(xbar=xbar.reshape(x.shape), Dbar=Db[:, :-1], mbar=mb, f=f)

    # ---- structured finite differences
    def _dE(self, x_a2_u, su0, dr):
        """Change of 0.5 sum |x|^2 s^2 when r changes by dr (the correction is linear in
        r, so ds is formed from dr directly, without differencing two numbers near 1)."""
        d = self.norm * (self.w0 * dr[self.j0] + self.w1 * dr[self.j0 + 1])
        d[self.udc] = 0.0
        return float(np.sum(x_a2_u * d * (2 * su0 + d))), su0 + d

    def _a2u(self, x):
        return 0.5 * np.bincount(self.uinv, weights=(x.real ** 2 + x.imag ** 2).ravel(), minlength=len(self.uk2))

    def fd_history(self, x, D, mJ, wb, f, b, j, rel=1e-6):
        a2u = self._a2u(x)
        h = rel * abs(D[b, j])
        res = []
        for sgn in (1, -1):
            Dp = D.copy()
            Dp[b, j] += sgn * h
            out = np.maximum(self.dnu(f["dc"], Dp, mJ), 0)
            dE, _ = self._dE(a2u, f["su"], (out - f["out"]) / f["dc"])
            res.append(float(np.sum(wb * (out - f["out"]) * (out + f["out"]))) + dE)
        return (res[0] - res[1]) / (2 * h)

    def fd_mass(self, x, D, mJ, wb, f, rel=1e-6, i=0):
        """d L / d (mass of mass state i inside J)."""
        a2u = self._a2u(x)
        m0 = np.asarray(mJ, dtype=np.float64)
        h = rel * m0[i]
        res = []
        for sgn in (1, -1):
            mm = m0.copy()
            mm[i] += sgn * h
            out = np.maximum(self.dnu(f["dc"], D, mm), 0)
            dE, _ = self._dE(a2u, f["su"], (out - f["out"]) / f["dc"])
            res.append(float(np.sum(wb * (out - f["out"]) * (out + f["out"]))) + dE)
        return (res[0] - res[1]) / (2 * h)

    def fd_mode(self, x, D, mJ, wb, f, idx, part, rel=1e-6):
        """d L / d (Re or Im of the mode at flat index idx) (idx != 0)."""
        xf = x.ravel()
        a2u = self._a2u(x)
        v0 = xf[idx].real if part == 0 else xf[idx].imag
        h = rel * abs(v0)
        b = self.cb[idx]
        res = []
        for sgn in (1, -1):
            dv = sgn * h
            da2 = dv * (2 * v0 + dv)  # |x'|^2 - |x|^2
            dP = np.zeros(self.nk)
            dP[b] = self.wt[idx] * self.W4[idx] * da2 / (f["F0"] * self.count[b])
            dc_new = np.sqrt((f["P"] + dP) * self.L ** 3)
            ddc = dP * self.L ** 3 / (dc_new + f["dc"])
            out = np.maximum(self.dnu(dc_new, D, mJ), 0)
            dr = (out - f["out"]) / dc_new - f["out"] * ddc / (f["dc"] * dc_new)
            dE, su1 = self._dE(a2u, f["su"], dr)
            direct = 0.5 * da2 * su1[self.uinv[idx]] ** 2
            res.append(float(np.sum(wb * (out - f["out"]) * (out + f["out"]))) + dE + direct)
        return (res[0] - res[1]) / (2 * h)
