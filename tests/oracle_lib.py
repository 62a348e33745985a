"""ctypes bindings to the CPU checkers (test infrastructure).

* ``Oracle``  -- oracle/liboracle.so, the project's C restatement of the reference path.
* ``RefLib``  -- oracle/_ref/libkspace_ref.so, the UNMODIFIED reference C sources built
  here against the project's GSL-subset shims (only exists where the reference
  sources were available at build time; tests that need it skip otherwise).
"""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "liboracle.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "libkspace_ref.so")
# the same sources built with -DKSPACE_NEUTRINOS_2 (the Gadget-2 neutrino-run switch)
REF_NU2_SO = os.path.join(ORACLE_DIR, "_ref", "libkspace_ref_nu2.so")

d = C.c_double
i32 = C.c_int
vp = C.c_void_p
PD = C.POINTER(C.c_double)
PI = C.POINTER(C.c_int)
PLL = C.POINTER(C.c_longlong)


def _p(a, ct=C.c_double):
    return a.ctypes.data_as(C.POINTER(ct))


def build_oracle():
    """Build liboracle.so (and the reference build when its sources are present)."""
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    if not os.path.exists(REF_SO):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "ref-if-present"], check=True)


def _sig(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


class Oracle:
    _lib = None

    def __init__(self):
        if Oracle._lib is None:
            if not os.path.exists(ORACLE_SO):
                build_oracle()
            L = C.CDLL(ORACLE_SO)
            _sig(L, "ko_bg_new", vp, [PD, d, d, d, d, d, d, i32])
            _sig(L, "ko_bg_free", None, [vp])
            _sig(L, "ko_bg_hybrid", i32, [vp, d, d, d])
            for n in ("ko_hubble", "ko_omega_nu", "ko_omega_nu_nopart", "ko_omegag"):
                _sig(L, n, d, [vp, d])
            _sig(L, "ko_omega_nu_single", d, [vp, d, i32])
            _sig(L, "ko_particle_nu_fraction", d, [vp, d, i32])
            _sig(L, "ko_nufrac_low", d, [d])
            _sig(L, "ko_bg_info", None, [vp, PD, PD, PI, PD])
            _sig(L, "ko_bg_table", i32, [vp, i32, PD, PD])
            _sig(L, "ko_specialJ", d, [d, d, d])
            _sig(L, "ko_fslength", d, [vp, d, d, d, PI])
            _sig(L, "ko_state_new", vp, [vp, i32, d, d, d, d, d])
            _sig(L, "ko_state_free", None, [vp])
            _sig(L, "ko_state_set_transfer", i32, [vp, PD, PD, i32])
            _sig(L, "ko_state_set_nu_state", i32, [vp, PD, PD, i32, i32])
            _sig(L, "ko_state_get", None, [vp, PI, PD, PD, PD])
            _sig(L, "ko_state_scalars", None, [vp, PD])
            _sig(L, "ko_state_set_ia", None, [vp, i32])
            _sig(L, "ko_state_options", None, [vp, i32, i32])
            _sig(L, "ko_delta_tot_init", i32, [vp, i32, PD, PD, d])
            _sig(L, "ko_get_delta_nu_update", i32, [vp, d, i32, PD, PD, PD])
            _sig(L, "ko_get_delta_nu_combined", i32, [vp, d, PD, PD])
            _sig(L, "ko_get_delta_nu", i32, [vp, d, PD, PD, d])
            _sig(L, "ko_get_delta_tot", d, [d, d, d, d, d, d])
            _sig(L, "ko_last_qag_stats", None, [vp, PI, PLL])
            _sig(L, "ko_last_fs_table", i32, [vp, PD, PD])
            _sig(L, "ko_total_powerspectrum", i32, [i32, vp, i32, i32, i32, PD, PLL, PD, i32, i32, PD, i32])
            _sig(L, "ko_dnudcdm", d, [PD, PD, i32, d, d, PI])
            _sig(L, "ko_apply_correction", i32, [vp, i32, i32, i32, d, PD, PD, i32, d, i32, i32])
            _sig(L, "ko_neutrino_power_internal", i32, [vp, d, PD, PD, PD, i32, PD])
            _sig(L, "ko_add_nu_power_to_rhogrid", i32,
                 [vp, d, d, vp, i32, i32, i32, i32, PI, PD, PD, PD, PD, PD, PD, PD])
            Oracle._lib = L
        self.L = Oracle._lib

    # ---- background
    def bg(self, MNu, a0=0.01, h=0.7, tcmb0=2.7255, Omega0=0.3, OmegaLambda=None, UnitTime_in_s=None,
           radiation=1):
        if OmegaLambda is None:
            OmegaLambda = 1 - Omega0
        if UnitTime_in_s is None:
            UnitTime_in_s = 3.085678e24 / 1e5
        m = np.ascontiguousarray(MNu, dtype=np.float64)
        return self.L.ko_bg_new(_p(m), a0, h, tcmb0, Omega0, OmegaLambda, UnitTime_in_s, radiation)

    def bg_info(self, bg):
        rc, kb = d(), d()
        deg = (C.c_int * 3)()
        mnu = (C.c_double * 3)()
        self.L.ko_bg_info(bg, C.byref(rc), C.byref(kb), deg, mnu)
        return rc.value, kb.value, list(deg), list(mnu)

    def bg_table(self, bg, i):
        la = np.zeros(200)
        rn = np.zeros(200)
        n = self.L.ko_bg_table(bg, i, _p(la), _p(rn))
        return (la, rn) if n else (None, None)

    # ---- state
    def state(self, bg, nk_alloc, TimeTransfer, TimeMax, Omega0=0.3, UnitTime_in_s=None,
              UnitLength_in_cm=3.085678e24):
        if UnitTime_in_s is None:
            UnitTime_in_s = UnitLength_in_cm / 1e5
        return self.L.ko_state_new(bg, nk_alloc, TimeTransfer, TimeMax, Omega0, UnitTime_in_s, UnitLength_in_cm)

    def set_transfer(self, s, logk, Tnu):
        logk = np.ascontiguousarray(logk, np.float64)
        Tnu = np.ascontiguousarray(Tnu, np.float64)
        return self.L.ko_state_set_transfer(s, _p(logk), _p(Tnu), len(logk))

    def set_nu_state(self, s, scalefact, delta_tot):
        sf = np.ascontiguousarray(scalefact, np.float64)
        dt = np.ascontiguousarray(delta_tot, np.float64)
        nk, ia = dt.shape
        return self.L.ko_state_set_nu_state(s, _p(sf), _p(dt), nk, ia)

    def get_state(self, s):
        ints = (C.c_int * 5)()
        self.L.ko_state_get(s, ints, None, None, None)
        nk, nk_alloc, namax, ia, done = list(ints)
        sf = np.zeros(namax)
        dt = np.zeros((nk_alloc, namax))
        v3 = np.zeros(3 * nk_alloc)
        self.L.ko_state_get(s, ints, _p(sf), _p(dt), _p(v3))
        return dict(nk=nk, nk_alloc=nk_alloc, namax=namax, ia=ia, init_done=done, scalefact=sf,
                    delta_tot=dt, nu_init=v3[:nk_alloc], nu_last=v3[nk_alloc:2 * nk_alloc],
                    wavenum=v3[2 * nk_alloc:])

    def scalars(self, s):
        out = np.zeros(4)
        self.L.ko_state_scalars(s, _p(out))
        return dict(prefac=out[0], Omeganonu=out[1], light=out[2], TimeTransfer=out[3])

    def get_delta_nu_update(self, s, a, keff, dcdm):
        keff = np.ascontiguousarray(keff, np.float64)
        dcdm = np.ascontiguousarray(dcdm, np.float64)
        out = np.zeros(len(keff))
        st = self.L.ko_get_delta_nu_update(s, a, len(keff), _p(keff), _p(dcdm), _p(out))
        return st, out

    def qag_stats(self, s):
        mx = C.c_int()
        tot = C.c_longlong()
        self.L.ko_last_qag_stats(s, C.byref(mx), C.byref(tot))
        return mx.value, tot.value

    def fs_table(self, s):
        n = self.L.ko_last_fs_table(s, None, None)
        sc = np.zeros(n)
        ln = np.zeros(n)
        self.L.ko_last_fs_table(s, _p(sc), _p(ln))
        return sc, ln

    # ---- binning / multiply
    def total_powerspectrum(self, grid, dims, nrbins, startslab=0, nslab=None, mode=0, partial=False, nthreads=1):
        g = np.ascontiguousarray(grid)
        assert g.dtype == np.complex64
        if nslab is None:
            nslab = dims
        power = np.zeros(nrbins)
        keff = np.zeros(nrbins)
        count = np.zeros(nrbins, dtype=np.int64)
        f0 = d()
        nk = self.L.ko_total_powerspectrum(dims, g.ctypes.data, nrbins, startslab, nslab, _p(power),
                                           _p(count, C.c_longlong), _p(keff), mode, int(partial), C.byref(f0),
                                           nthreads)
        if partial:
            return power, count, keff, f0.value
        return nk, power[:nk], count[:nk], keff[:nk]

    def apply_correction(self, grid, pmgrid, slab0, nslab, BoxSize, logk, ratio, norm, mode=0, nthreads=1):
        logk = np.ascontiguousarray(logk, np.float64)
        ratio = np.ascontiguousarray(ratio, np.float64)
        assert grid.flags.c_contiguous
        return self.L.ko_apply_correction(grid.ctypes.data, pmgrid, slab0, nslab, BoxSize, _p(logk), _p(ratio),
                                          len(logk), norm, mode, nthreads)

    def add_nu_power_to_rhogrid(self, s, Time, BoxSize, grid, pmgrid, slab0=0, nslab=None, nthreads=1, nk_alloc=None):
        if nslab is None:
            nslab = pmgrid
        assert grid.dtype == np.complex64 and grid.flags.c_contiguous
        nb = nk_alloc or self.get_state(s)["nk_alloc"]
        keff, dcdm, dnu, logk, ratio = (np.zeros(nb) for _ in range(5))
        norm = d()
        nk = C.c_int()
        t = np.zeros(3)
        st = self.L.ko_add_nu_power_to_rhogrid(s, Time, BoxSize, grid.ctypes.data, pmgrid, slab0, nslab, nthreads,
                                               C.byref(nk), _p(keff), _p(dcdm), _p(dnu), _p(logk), _p(ratio),
                                               C.byref(norm), _p(t))
        n = nk.value
        return st, dict(nk=n, keff=keff[:n], dcdm=dcdm[:n], dnu=dnu[:n], logk=logk[:n], ratio=ratio[:n],
                        norm=norm.value, t_stages=t)


    def add_nu_power_to_rhogrid_fp64(self, s, Time, BoxSize, grid, pmgrid, nthreads=1, nk_alloc=None):
        """The step in FP64 throughout; returns (status, outputs, corrected complex128 grid)."""
        assert grid.dtype == np.complex64 and grid.flags.c_contiguous
        nb = nk_alloc or self.get_state(s)["nk_alloc"]
        keff, dcdm, dnu, ratio = (np.zeros(nb) for _ in range(4))
        norm = d()
        nk = C.c_int()
        out = np.zeros(grid.shape, dtype=np.complex128)
        L = self.L
        L.ko_add_nu_power_to_rhogrid_fp64.argtypes = [vp, d, d, vp, vp, i32, i32, C.POINTER(C.c_int), PD, PD, PD, PD,
                                                       C.POINTER(d)]
        L.ko_add_nu_power_to_rhogrid_fp64.restype = i32
        st = L.ko_add_nu_power_to_rhogrid_fp64(s, Time, BoxSize, grid.ctypes.data, out.ctypes.data, pmgrid, nthreads,
                                                C.byref(nk), _p(keff), _p(dcdm), _p(dnu), _p(ratio), C.byref(norm))
        n = nk.value
        return st, dict(nk=n, keff=keff[:n], dcdm=dcdm[:n], dnu=dnu[:n], ratio=ratio[:n], norm=norm.value), out


class RefLib:
    """The unmodified reference C (oracle/_ref/libkspace_ref.so, or another build of the
    same sources given by path)."""
    _libs = {}

    @staticmethod
    def available(path=REF_SO):
        return os.path.exists(path)

    def __init__(self, path=REF_SO):
        if path not in RefLib._libs:
            L = C.CDLL(path)
            _sig(L, "ref_omnu_new", vp, [])
            _sig(L, "ref_omnu_free", None, [vp])
            _sig(L, "ref_init_omega_nu", i32, [vp, PD, d, d, d])
            _sig(L, "ref_init_hybrid_nu", i32, [vp, PD, d, d, d])
            for n in ("ref_get_omega_nu", "ref_get_omega_nu_nopart", "ref_get_omegag"):
                _sig(L, n, d, [vp, d])
            _sig(L, "ref_omega_nu_single", d, [vp, d, i32])
            _sig(L, "ref_particle_nu_fraction", d, [vp, d, i32])
            _sig(L, "ref_nufrac_low", i32, [d, PD])
            _sig(L, "ref_omnu_info", None, [vp, PD, PD, PI])
            _sig(L, "ref_omnu_table", i32, [vp, i32, PD, PD])
            _sig(L, "ref_rho_nu", d, [vp, i32, d])
            _sig(L, "ref_set_hubble", None, [vp, d, d, d, i32])
            _sig(L, "ref_hubble", d, [d])
            _sig(L, "ref_transfer_new", vp, [])
            _sig(L, "ref_transfer_read", i32, [vp, d, d, d, C.c_char_p])
            _sig(L, "ref_transfer_set", None, [vp, PD, PD, i32])
            _sig(L, "ref_transfer_get", i32, [vp, PD, PD])
            _sig(L, "ref_transfer_free", None, [vp])
            _sig(L, "ref_dtot_new", vp, [])
            _sig(L, "ref_allocate_delta_tot_table", i32, [vp, i32, d, d, d, vp, d, d])
            _sig(L, "ref_dtot_free", None, [vp])
            _sig(L, "ref_delta_tot_init", i32, [vp, i32, PD, PD, vp, d])
            _sig(L, "ref_get_delta_nu_update", i32, [vp, d, i32, PD, PD, PD, vp])
            _sig(L, "ref_get_delta_nu_combined", i32, [vp, d, PD, PD])
            _sig(L, "ref_get_delta_nu", i32, [vp, d, PD, PD, d])
            _sig(L, "ref_update_delta_tot", i32, [vp, d, PD, PD, i32])
            _sig(L, "ref_read_all_nu_state", i32, [vp, C.c_char_p])
            _sig(L, "ref_save_all_nu_state", i32, [vp, C.c_char_p])
            _sig(L, "ref_save_nu_power", i32, [vp, d, i32, C.c_char_p, PI])
            _sig(L, "ref_specialJ", d, [d, d, d])
            _sig(L, "ref_fslength", i32, [d, d, d, PD])
            _sig(L, "ref_get_delta_tot", d, [d, d, d, d, d, d])
            _sig(L, "ref_dtot_ints", None, [vp, PI])
            _sig(L, "ref_dtot_scalars", None, [vp, PD])
            _sig(L, "ref_dtot_set_ia", None, [vp, i32])
            _sig(L, "ref_dtot_get", None, [vp, PD, PD, PD])
            _sig(L, "ref_dtot_set", None, [vp, PD, PD, i32, i32])
            _sig(L, "ref_total_powerspectrum", i32, [i32, vp, i32, i32, i32, PD, PLL, PD, PI])
            _sig(L, "ref_dpow_new", vp, [])
            _sig(L, "ref_init_delta_pow", i32, [vp, PD, PD, i32, d])
            _sig(L, "ref_get_dnudcdm_powerspec", i32, [vp, d, PD])
            _sig(L, "ref_dpow_free", None, [vp])
            _sig(L, "ref_set_kspace_params", None, [C.c_char_p, d, d, PD, i32, d, d])
            _sig(L, "ref_InitOmegaNu", i32, [d, d])
            _sig(L, "ref_OmegaNu", d, [d])
            _sig(L, "ref_OmegaNu_nopart", d, [d])
            _sig(L, "ref_allocate_kspace_memory", i32, [i32, d, d, d, d, C.c_char_p, d])
            _sig(L, "ref_add_nu_power_to_rhogrid", i32, [d, d, vp, i32, i32, i32])
            _sig(L, "ref_compute_total_power_spectrum", i32, [d, d, vp, i32, i32, i32])
            _sig(L, "ref_compute_neutrino_power_from_cdm", i32,
                 [d, PD, PD, C.POINTER(C.c_long), i32, PD, PD, PD, PI])
            _sig(L, "ref_save_nu_state", i32, [C.c_char_p])
            _sig(L, "ref_save_neutrino_power", i32, [d, i32, C.c_char_p, PI])
            _sig(L, "ref_save_total_power", i32, [d, i32, C.c_char_p, PI])
            _sig(L, "ref_particle_nu_active", i32, [d])
            _sig(L, "ref_get_nu_state", i32, [PD, PD, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), C.c_size_t])
            _sig(L, "ref_set_nu_state", i32, [PD, PD, C.c_size_t, C.c_size_t])
            _sig(L, "ref_global_dtot", vp, [])
            _sig(L, "ref_set_hubble_global", None, [d, d, d, i32, d, d])
            _sig(L, "ref_set_verbose", None, [i32])
            _sig(L, "ref_last_terminate_message", C.c_char_p, [])
            RefLib._libs[path] = L
        self.L = RefLib._libs[path]

    def omnu(self, MNu, a0=0.01, h=0.7, tcmb0=2.7255):
        o = self.L.ref_omnu_new()
        m = np.ascontiguousarray(MNu, np.float64)
        st = self.L.ref_init_omega_nu(o, _p(m), a0, h, tcmb0)
        assert st == 0, st
        return o

    def dtot_state(self, dt):
        ints = (C.c_int * 5)()
        self.L.ref_dtot_ints(dt, ints)
        nk, nk_alloc, namax, ia, done = list(ints)
        sf = np.zeros(namax)
        tab = np.zeros((nk_alloc, namax))
        v3 = np.zeros(3 * nk_alloc)
        self.L.ref_dtot_get(dt, _p(sf), _p(tab), _p(v3))
        return dict(nk=nk, nk_alloc=nk_alloc, namax=namax, ia=ia, init_done=done, scalefact=sf, delta_tot=tab,
                    nu_init=v3[:nk_alloc], nu_last=v3[nk_alloc:2 * nk_alloc], wavenum=v3[2 * nk_alloc:])

    def total_powerspectrum(self, grid, dims, nrbins, startslab=0, nslab=None):
        g = np.ascontiguousarray(grid)
        assert g.dtype == np.complex64
        if nslab is None:
            nslab = dims
        power = np.zeros(nrbins)
        keff = np.zeros(nrbins)
        count = np.zeros(nrbins, dtype=np.int64)
        nk = C.c_int()
        st = self.L.ref_total_powerspectrum(dims, g.ctypes.data, nrbins, startslab, nslab, _p(power),
                                            _p(count, C.c_longlong), _p(keff), C.byref(nk))
        assert st == 0
        n = nk.value
        return n, power[:n], count[:n], keff[:n]
