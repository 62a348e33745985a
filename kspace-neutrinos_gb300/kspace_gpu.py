"""Python mirror of the kspace-neutrinos interface on top of libkspace_gb300.so.

``KspaceNeutrinos`` follows the reference's public API (interface_common.h,
interface_gadget.h, delta_tot_table.h): the same operations, argument meanings and
error codes.  Where the reference calls terminate(code, ...), this raises
``KspaceError`` carrying that code.  Grids may be CUDA tensors (used in place) or
numpy/pinned host arrays (copied to the device and back inside the call).

There is no CPU path: if the CUDA library cannot be loaded, every call raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libkspace_gb300.so")

_d = C.c_double
_i = C.c_int
_vp = C.c_void_p
_PD = C.POINTER(C.c_double)
_PI = C.POINTER(C.c_int)
_PLL = C.POINTER(C.c_longlong)
_PSZ = C.POINTER(C.c_size_t)

ALLREDUCE_FN = C.CFUNCTYPE(C.c_int, _PD, C.c_int, C.c_void_p)

# name: (restype, argtypes)
_SIGS = {
    "kspace_gpu_create": (_i, [C.POINTER(_vp), _i]),
    "kspace_gpu_destroy": (_i, [_vp]),
    "kspace_gpu_error_string": (C.c_char_p, [_i]),
    "kspace_gpu_set_stream": (_i, [_vp, _vp]),
    "kspace_gpu_set_allreduce": (_i, [_vp, ALLREDUCE_FN, _vp]),
    "kspace_gpu_set_tuning": (_i, [_vp, _i, _i, _i, _i]),
    "kspace_gpu_init_omega_nu": (_i, [_vp, _PD, _d, _d, _d]),
    "kspace_gpu_init_hybrid_nu": (_i, [_vp, _d, _d, _d]),
    "kspace_gpu_set_hubble": (_i, [_vp, _d, _d, _d, _i]),
    "kspace_gpu_check_hubble": (_i, [_vp, _PD, _PD, _i, _d, _PD]),
    "kspace_gpu_omega_nu": (_i, [_vp, _d, _PD, _PD]),
    "kspace_gpu_particle_nu_active": (_i, [_vp, _d, _PI]),
    "kspace_gpu_hubble": (_i, [_vp, _d, _PD]),
    "kspace_gpu_alloc_table": (_i, [_vp, _i, _d, _d, _d, _d, _d]),
    "kspace_gpu_set_transfer": (_i, [_vp, _PD, _PD, _i]),
    "kspace_gpu_read_transfer_file": (_i, [_vp, _d, _d, _d, C.c_char_p, _PI]),
    "kspace_gpu_set_nu_state": (_i, [_vp, _PD, _PD, C.c_size_t, C.c_size_t]),
    "kspace_gpu_get_nu_state": (_i, [_vp, _PD, _PD, _PSZ, _PSZ]),
    "kspace_gpu_read_nu_state": (_i, [_vp, C.c_char_p]),
    "kspace_gpu_save_nu_state": (_i, [_vp, C.c_char_p]),
    "kspace_gpu_save_nu_power": (_i, [_vp, _d, _i, C.c_char_p]),
    "kspace_gpu_table_info": (_i, [_vp, _PI]),
    "kspace_gpu_get_vectors": (_i, [_vp, _PD, _PD, _PD]),
    "kspace_gpu_total_powerspectrum": (_i, [_vp, _i, _vp, _i, _i, _i, _PD, _PLL, _PD, _PI]),
    "kspace_gpu_get_delta_nu_update": (_i, [_vp, _d, _i, _PD, _PD, _PD]),
    "kspace_gpu_compute_neutrino_power_from_cdm": (_i, [_vp, _d, _PD, _PD, C.POINTER(C.c_long), _i, _PD, _PD,
                                                        _PD, _PI]),
    "kspace_gpu_add_nu_power_to_rhogrid": (_i, [_vp, _d, _d, _vp, _i, _i, _i]),
    "kspace_gpu_apply_delta_pow": (_i, [_vp, _d, _vp, _i, _i, _i, _i, _PD, _PD, _i, _d]),
    "kspace_gpu_compute_total_power_spectrum": (_i, [_vp, _d, _d, _vp, _i, _i, _i]),
    "kspace_gpu_save_total_power": (_i, [_vp, _d, _i, C.c_char_p]),
    "kspace_gpu_last_correction": (_i, [_vp, _PI, _PD, _PD, _PD, _PD, _PD]),
    "kspace_gpu_set_profiling": (_i, [_vp, _i]),
    "kspace_gpu_stage_times": (_i, [_vp, C.POINTER(C.c_float)]),
    "kspace_gpu_qag_stats": (_i, [_vp, _PI, _PLL]),
    "kspace_gpu_launch_count": (C.c_longlong, [_vp]),
    "kspace_gpu_set_vectors": (_i, [_vp, _PD, _PD, _PD, _i]),
    "kspace_gpu_set_jmass": (_i, [_vp, _PD]),
    "kspace_gpu_diff_forward": (_i, [_vp, _d, _d, _vp, _vp, _i, _vp, _i]),
    "kspace_gpu_diff_backward": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _PD, _i, C.c_longlong]),
    "kspace_gpu_diff_generation": (_i, [_vp, _PLL]),
    "kspace_gpu_batch_create": (_i, [C.POINTER(_vp), C.POINTER(_vp), _i]),
    "kspace_gpu_batch_destroy": (_i, [_vp]),
    "kspace_gpu_batch_bind_grid": (_i, [_vp, _i, _vp, _i, _d]),
    "kspace_gpu_batch_init": (_i, [_vp, _PD, _PI, _PD, _PD]),
    "kspace_gpu_batch_layout": (_i, [_vp, _PI, _PI]),
    "kspace_gpu_batch_step": (_i, [_vp, _PD, _vp, _vp]),
    "kspace_gpu_batch_status": (_i, [_vp, _PI]),
    "kspace_gpu_batch_set_tuning": (_i, [_vp, _i, _i, _i]),
    "kspace_gpu_batch_autotune": (_i, [_vp, _PD, _vp, _i, _PI, C.POINTER(C.c_float)]),
    "kspace_gpu_batch_last_ms": (_i, [_vp, C.POINTER(C.c_float)]),
    "kspace_gpu_bin_power_noalloc": (_i, [_i, _vp, _i, _i, _i, _vp, _vp]),
    "kspace_gpu_set_hybrid": (_i, [_vp, _i, _d, _d, _PD]),
    "kspace_gpu_set_hubble_table": (_i, [_vp, _d, _d, _i, _PD]),
    "kspace_gpu_delta_tot_init": (_i, [_vp, _i, _PD, _PD, _d]),
    "kspace_gpu_get_delta_nu": (_i, [_vp, _d, _i, _PD, _PD, _d]),
    "kspace_gpu_get_delta_nu_combined": (_i, [_vp, _d, _i, _PD, _PD]),
    "kspace_gpu_update_delta_tot": (_i, [_vp, _d, _PD, _PD, _i]),
    "kspace_gpu_set_table": (_i, [_vp, _i, _i, _i, _PD, _PD, C.c_size_t, _PD, _PD, _PD]),
    "kspace_gpu_get_table": (_i, [_vp, _i, _PI, _PI, _PI, _PD, _PD, C.c_size_t, _PD, _PD, _PD]),
    "kspace_gpu_special_j": (_i, [_vp, _PD, _i, _d, _d, _PD]),
    "kspace_gpu_nufrac_low": (_i, [_vp, _PD, _i, _PD]),
    "kspace_gpu_fslength": (_i, [_vp, _PD, _PD, _i, _d, _PD]),
    "kspace_gpu_omega_nu_single": (_i, [_vp, _d, _i, _PD]),
    "kspace_gpu_omega_g": (_i, [_vp, _d, _PD]),
    "kspace_gpu_background_info": (_i, [_vp, _PD, _PD, _PI, _PD]),
}

_lib = None


def load_library(path=None):
    """Load libkspace_gb300.so (raises OSError if it is missing)."""
    global _lib
    if _lib is None:
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise OSError("libkspace_gb300.so not built: run build.py in %s" % HERE)
        lib = C.CDLL(p)
        for name, (res, args) in _SIGS.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def exported_symbols():
    return sorted(_SIGS)


class KspaceError(RuntimeError):
    """A failure the reference reports through terminate(code, ...)."""

    def __init__(self, code, where=""):
        msg = _lib.kspace_gpu_error_string(code).decode() if _lib is not None else ""
        super().__init__("%s: status %d (%s)" % (where, code, msg))
        self.code = code


def _check(code, where):
    if code != 0:
        raise KspaceError(code, where)


def _pd(a):
    return a.ctypes.data_as(_PD)


def _f64(x):
    return np.ascontiguousarray(x, dtype=np.float64)


def _grid_ptr(grid):
    """(pointer, keepalive) for a complex64 grid: torch tensor (CUDA or CPU) or numpy."""
    try:
        import torch
        if isinstance(grid, torch.Tensor):
            if grid.dtype not in (torch.complex64, torch.float32):
                raise TypeError("grid must be complex64 (or float32 re/im pairs)")
            if not grid.is_contiguous():
                raise ValueError("grid must be contiguous")
            return grid.data_ptr(), grid
    except ImportError:
        pass
    g = grid
    if not isinstance(g, np.ndarray) or g.dtype not in (np.complex64, np.float32) or not g.flags.c_contiguous:
        raise TypeError("grid must be a contiguous complex64 numpy array or torch tensor")
    return g.ctypes.data, g


class KspaceNeutrinos:
    """One integrator instance (the reference's global state, as an object)."""

    def __init__(self, device=0):
        self.L = load_library()
        h = _vp()
        _check(self.L.kspace_gpu_create(C.byref(h), device), "kspace_gpu_create")
        self.h = h
        self._ar = None

    def close(self):
        if getattr(self, "h", None):
            self.L.kspace_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- configuration
    def set_stream(self, stream):
        """Run on a torch.cuda.Stream (or raw cudaStream_t int); None = own stream."""
        ptr = None
        if stream is not None:
            ptr = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
        _check(self.L.kspace_gpu_set_stream(self.h, ptr), "set_stream")

    def set_tuning(self, tma=-1, rows=-1, stages=-1, qag_warps=-1):
        _check(self.L.kspace_gpu_set_tuning(self.h, tma, rows, stages, qag_warps), "set_tuning")

    def set_allreduce(self, fn):
        """fn(np.ndarray[float64]) -> None sums in place across ranks (None = one rank)."""
        if fn is None:
            self._ar = None
            _check(self.L.kspace_gpu_set_allreduce(self.h, ALLREDUCE_FN(), None), "set_allreduce")
            return

        def cb(buf, count, user):
            try:
                arr = np.ctypeslib.as_array(buf, shape=(count,))
                fn(arr)
                return 0
            except Exception:
                return 1

        self._ar = ALLREDUCE_FN(cb)
        _check(self.L.kspace_gpu_set_allreduce(self.h, self._ar, None), "set_allreduce")

    # ---- background (InitOmegaNu, interface_common.c:183-188)
    def init_omega_nu(self, MNu, TimeTransfer, HubbleParam, tcmb0=2.7255):
        m = _f64(MNu)
        assert m.shape == (3,)
        _check(self.L.kspace_gpu_init_omega_nu(self.h, _pd(m), TimeTransfer, HubbleParam, tcmb0), "InitOmegaNu")

    def init_hybrid_nu(self, vcrit, light, nu_crit_time):
        _check(self.L.kspace_gpu_init_hybrid_nu(self.h, vcrit, light, nu_crit_time), "init_hybrid_nu")

    def set_hubble(self, Omega0, OmegaLambda=None, UnitTime_in_s=3.085678e24 / 1e5, include_radiation=True):
        if OmegaLambda is None:
            OmegaLambda = 1.0 - Omega0
        _check(self.L.kspace_gpu_set_hubble(self.h, Omega0, OmegaLambda, UnitTime_in_s, int(include_radiation)),
               "set_hubble")

    def set_hubble_table(self, loga_lo, dloga, H):
        h = _f64(H)
        _check(self.L.kspace_gpu_set_hubble_table(self.h, loga_lo, dloga, len(h), _pd(h)), "set_hubble_table")

    def check_hubble(self, a, H, rtol=1e-12):
        a = _f64(a)
        H = _f64(H)
        mx = _d()
        st = self.L.kspace_gpu_check_hubble(self.h, _pd(a), _pd(H), len(a), rtol, C.byref(mx))
        return st, mx.value

    def OmegaNu(self, a):
        o = _d()
        _check(self.L.kspace_gpu_omega_nu(self.h, a, C.byref(o), None), "OmegaNu")
        return o.value

    def OmegaNu_nopart(self, a):
        o = _d()
        _check(self.L.kspace_gpu_omega_nu(self.h, a, None, C.byref(o)), "OmegaNu_nopart")
        return o.value

    def particle_nu_active(self, a):
        v = _i()
        _check(self.L.kspace_gpu_particle_nu_active(self.h, a, C.byref(v)), "particle_nu_active")
        return v.value

    def hubble(self, a):
        v = _d()
        _check(self.L.kspace_gpu_hubble(self.h, a, C.byref(v)), "hubble")
        return v.value

    def set_hybrid(self, enabled, vcrit_frac, nu_crit_time, nufrac_low):
        f = _f64(nufrac_low)
        _check(self.L.kspace_gpu_set_hybrid(self.h, int(enabled), vcrit_frac, nu_crit_time, _pd(f)), "set_hybrid")

    def omega_nu_single(self, a, i):
        v = _d()
        _check(self.L.kspace_gpu_omega_nu_single(self.h, a, i, C.byref(v)), "omega_nu_single")
        return v.value

    def omegag(self, a):
        v = _d()
        _check(self.L.kspace_gpu_omega_g(self.h, a, C.byref(v)), "get_omegag")
        return v.value

    def background_info(self):
        rc, kb = _d(), _d()
        deg = (C.c_int * 3)()
        nfl = np.zeros(3)
        _check(self.L.kspace_gpu_background_info(self.h, C.byref(rc), C.byref(kb), deg, _pd(nfl)),
               "background_info")
        return dict(rhocrit=rc.value, kBtnu=kb.value, deg=list(deg), nufrac_low=nfl)

    def fslength(self, logai, logaf, light):
        """fslength (delta_tot_table.c:394-407) of arrays of intervals, on the device."""
        a = np.atleast_1d(_f64(logai))
        b = np.atleast_1d(_f64(logaf))
        out = np.zeros(len(a))
        _check(self.L.kspace_gpu_fslength(self.h, _pd(a), _pd(b), len(a), light, _pd(out)), "fslength")
        return out

    # ---- table (allocate_kspace_memory, interface_common.c:77-102)
    def alloc_table(self, nk_alloc, TimeTransfer, TimeMax, Omega0, UnitTime_in_s, UnitLength_in_cm):
        _check(self.L.kspace_gpu_alloc_table(self.h, nk_alloc, TimeTransfer, TimeMax, Omega0, UnitTime_in_s,
                                             UnitLength_in_cm), "allocate_delta_tot_table")

    def set_transfer(self, logk, T_nu):
        lk = _f64(logk)
        t = _f64(T_nu)
        _check(self.L.kspace_gpu_set_transfer(self.h, _pd(lk), _pd(t), len(lk)), "set_transfer")

    def read_transfer_file(self, BoxSize, UnitLength_in_cm, InputSpectrum_UnitLength_in_cm, path):
        n = _i()
        _check(self.L.kspace_gpu_read_transfer_file(self.h, BoxSize, UnitLength_in_cm,
                                                    InputSpectrum_UnitLength_in_cm, path.encode(), C.byref(n)),
               "allocate_transfer_init_table")
        return n.value

    def set_nu_state(self, scalefact, delta_tot):
        """scalefact: host array [ia]; delta_tot: [nk][ia] float64, numpy or a torch tensor
        (host or CUDA)."""
        sf = _f64(scalefact)
        try:
            import torch
            if isinstance(delta_tot, torch.Tensor):
                t = delta_tot.detach().to(torch.float64).contiguous()
                nk, ia = t.shape
                _check(self.L.kspace_gpu_set_nu_state(self.h, _pd(sf), C.cast(t.data_ptr(), _PD), nk, ia),
                       "set_nu_state")
                return
        except ImportError:
            pass
        dt = _f64(delta_tot)
        nk, ia = dt.shape
        _check(self.L.kspace_gpu_set_nu_state(self.h, _pd(sf), _pd(dt), nk, ia), "set_nu_state")

    def get_nu_state(self):
        nk = C.c_size_t()
        ia = C.c_size_t()
        _check(self.L.kspace_gpu_get_nu_state(self.h, None, None, C.byref(nk), C.byref(ia)), "get_nu_state")
        sf = np.zeros(ia.value)
        dt = np.zeros((nk.value, ia.value))
        _check(self.L.kspace_gpu_get_nu_state(self.h, _pd(sf), _pd(dt), C.byref(nk), C.byref(ia)), "get_nu_state")
        return sf, dt

    def read_nu_state(self, path):
        _check(self.L.kspace_gpu_read_nu_state(self.h, path.encode()), "read_all_nu_state")

    def save_nu_state(self, path):
        _check(self.L.kspace_gpu_save_nu_state(self.h, path.encode()), "save_all_nu_state")

    def save_nu_power(self, Time, snapnum, OutputDir):
        return self.L.kspace_gpu_save_nu_power(self.h, Time, snapnum, OutputDir.encode())

    def table_info(self):
        a = (C.c_int * 5)()
        _check(self.L.kspace_gpu_table_info(self.h, a), "table_info")
        return dict(zip(("nk", "nk_allocated", "namax", "ia", "delta_tot_init_done"), list(a)))

    def vectors(self):
        n = self.table_info()["nk_allocated"]
        a, b, c = np.zeros(n), np.zeros(n), np.zeros(n)
        _check(self.L.kspace_gpu_get_vectors(self.h, _pd(a), _pd(b), _pd(c)), "get_vectors")
        return dict(delta_nu_init=a, delta_nu_last=b, wavenum=c)

    # ---- hot path
    def total_powerspectrum(self, dims, grid, nrbins, startslab=0, nslab=None):
        if nslab is None:
            nslab = dims
        ptr, keep = _grid_ptr(grid)
        power = np.zeros(nrbins)
        keff = np.zeros(nrbins)
        count = np.zeros(nrbins, dtype=np.int64)
        nk = _i()
        _check(self.L.kspace_gpu_total_powerspectrum(self.h, dims, ptr, nrbins, startslab, nslab, _pd(power),
                                                     count.ctypes.data_as(_PLL), _pd(keff), C.byref(nk)),
               "total_powerspectrum")
        n = nk.value
        return n, power[:n], count[:n], keff[:n]

    def get_delta_nu_update(self, a, keff, P_cdm_sqrt):
        k = _f64(keff)
        d = _f64(P_cdm_sqrt)
        out = np.zeros(len(k))
        _check(self.L.kspace_gpu_get_delta_nu_update(self.h, a, len(k), _pd(k), _pd(d), _pd(out)),
               "get_delta_nu_update")
        return out

    def delta_tot_init(self, keff, P_cdm_sqrt, Time):
        k = _f64(keff)
        d = _f64(P_cdm_sqrt)
        _check(self.L.kspace_gpu_delta_tot_init(self.h, len(k), _pd(k), _pd(d), Time), "delta_tot_init")

    def get_delta_nu(self, a, wavenum, mnu):
        k = _f64(wavenum)
        out = np.zeros(len(k))
        _check(self.L.kspace_gpu_get_delta_nu(self.h, a, len(k), _pd(k), _pd(out), mnu), "get_delta_nu")
        return out

    def get_delta_nu_combined(self, a, wavenum):
        k = _f64(wavenum)
        out = np.zeros(len(k))
        _check(self.L.kspace_gpu_get_delta_nu_combined(self.h, a, len(k), _pd(k), _pd(out)), "get_delta_nu_combined")
        return out

    def update_delta_tot(self, a, P_cdm_sqrt, delta_nu, overwrite):
        d = _f64(P_cdm_sqrt)
        n = _f64(delta_nu)
        _check(self.L.kspace_gpu_update_delta_tot(self.h, a, _pd(d), _pd(n), int(overwrite)), "update_delta_tot")

    def compute_neutrino_power_from_cdm(self, Time, keff, P_cdm, Nmodes):
        k = _f64(keff)
        p = _f64(P_cdm)
        nm = np.ascontiguousarray(Nmodes, dtype=np.int64)
        n = len(k)
        logk, ratio = np.zeros(n), np.zeros(n)
        norm = _d()
        nb = _i()
        _check(self.L.kspace_gpu_compute_neutrino_power_from_cdm(self.h, Time, _pd(k), _pd(p),
                                                                 nm.ctypes.data_as(C.POINTER(C.c_long)), n,
                                                                 _pd(logk), _pd(ratio), C.byref(norm), C.byref(nb)),
               "compute_neutrino_power_from_cdm")
        return logk[:nb.value], ratio[:nb.value], norm.value

    def add_nu_power_to_rhogrid(self, Time, BoxSize, grid, pmgrid, slabstart_y=0, nslab_y=None):
        if nslab_y is None:
            nslab_y = pmgrid
        ptr, keep = _grid_ptr(grid)
        _check(self.L.kspace_gpu_add_nu_power_to_rhogrid(self.h, Time, BoxSize, ptr, pmgrid, slabstart_y, nslab_y),
               "add_nu_power_to_rhogrid")

    def apply_delta_pow(self, BoxSize, grid, pmgrid, nrbins, logk, ratio, norm, slabstart_y=0, nslab_y=None):
        if nslab_y is None:
            nslab_y = pmgrid
        ptr, keep = _grid_ptr(grid)
        lk = _f64(logk)
        r = _f64(ratio)
        _check(self.L.kspace_gpu_apply_delta_pow(self.h, BoxSize, ptr, pmgrid, slabstart_y, nslab_y, nrbins,
                                                 _pd(lk), _pd(r), len(lk), norm), "apply_delta_pow")

    def compute_total_power_spectrum(self, Time, BoxSize, grid, pmgrid, slabstart_y=0, nslab_y=None):
        if nslab_y is None:
            nslab_y = pmgrid
        ptr, keep = _grid_ptr(grid)
        _check(self.L.kspace_gpu_compute_total_power_spectrum(self.h, Time, BoxSize, ptr, pmgrid, slabstart_y,
                                                              nslab_y), "compute_total_power_spectrum")

    def save_total_power(self, Time, snapnum, OutputDir):
        return self.L.kspace_gpu_save_total_power(self.h, Time, snapnum, OutputDir.encode())

    # ---- differentiation
    def set_vectors(self, nu_init, nu_last, wavenum):
        a, b, c = _f64(nu_init), _f64(nu_last), _f64(wavenum)
        _check(self.L.kspace_gpu_set_vectors(self.h, _pd(a), _pd(b), _pd(c), len(a)), "set_vectors")

    def set_jmass(self, MNu=None):
        if MNu is None:
            _check(self.L.kspace_gpu_set_jmass(self.h, None), "set_jmass")
        else:
            m = _f64(MNu)
            _check(self.L.kspace_gpu_set_jmass(self.h, _pd(m)), "set_jmass")

    def diff_forward(self, Time, BoxSize, grid_in, grid_out, pmgrid, pnu_out, store_intervals=True):
        """One differentiable step; returns its generation (for diff_backward)."""
        _check(self.L.kspace_gpu_diff_forward(self.h, Time, BoxSize, grid_in.data_ptr(), grid_out.data_ptr(),
                                              pmgrid, pnu_out.data_ptr(), int(store_intervals)), "diff_forward")
        g = C.c_longlong()
        _check(self.L.kspace_gpu_diff_generation(self.h, C.byref(g)), "diff_generation")
        return g.value

    def diff_backward(self, gbar_out, grid_in, pnu_bar, gbar_in, Dbar, recompute=False, generation=None):
        """Adjoint of the forward of that generation (default: the last forward)."""
        if generation is None:
            g = C.c_longlong()
            _check(self.L.kspace_gpu_diff_generation(self.h, C.byref(g)), "diff_generation")
            generation = g.value
        mbar = np.zeros(3)
        _check(self.L.kspace_gpu_diff_backward(self.h, gbar_out.data_ptr(), grid_in.data_ptr(), pnu_bar.data_ptr(),
                                               gbar_in.data_ptr(), Dbar.data_ptr() if Dbar is not None else None,
                                               _pd(mbar), int(recompute), generation), "diff_backward")
        return mbar

    # ---- diagnostics
    def last_correction(self):
        n_alloc = self.table_info()["nk_allocated"]
        nk = _i()
        lk, r, dc, ke = (np.zeros(n_alloc) for _ in range(4))
        norm = _d()
        _check(self.L.kspace_gpu_last_correction(self.h, C.byref(nk), _pd(lk), _pd(r), C.byref(norm), _pd(dc),
                                                 _pd(ke)), "last_correction")
        n = nk.value
        return dict(nk=n, logk=lk[:n], ratio=r[:n], norm=norm.value, dcdm=dc[:n], keff=ke[:n])

    def set_profiling(self, on=True):
        _check(self.L.kspace_gpu_set_profiling(self.h, int(on)), "set_profiling")

    def stage_times(self):
        a = (C.c_float * 4)()
        _check(self.L.kspace_gpu_stage_times(self.h, a), "stage_times")
        return list(a)

    def qag_stats(self):
        m = _i()
        t = C.c_longlong()
        _check(self.L.kspace_gpu_qag_stats(self.h, C.byref(m), C.byref(t)), "qag_stats")
        return m.value, t.value

    def launch_count(self):
        return int(self.L.kspace_gpu_launch_count(self.h))


def special_j(x, qc=-1.0, nufrac_low=0.0, device_ctx=None):
    """specialJ (delta_tot_table.c:457-463) of an array on the device."""
    L = load_library()
    xx = np.atleast_1d(_f64(x))
    out = np.zeros(len(xx))
    _check(L.kspace_gpu_special_j(device_ctx, _pd(xx), len(xx), qc, nufrac_low, _pd(out)), "specialJ")
    return out


def nufrac_low(qc, device_ctx=None):
    """nufrac_low (omega_nu_single.c:214-228) of an array on the device."""
    L = load_library()
    q = np.atleast_1d(_f64(qc))
    out = np.zeros(len(q))
    _check(L.kspace_gpu_nufrac_low(device_ctx, _pd(q), len(q), _pd(out)), "nufrac_low")
    return out


def _buf_ptr(x):
    """(pointer, keepalive) of a float64 array: numpy (host) or torch tensor (host or CUDA)."""
    if x is None:
        return None, None
    try:
        import torch
        if isinstance(x, torch.Tensor):
            if x.dtype != torch.float64 or not x.is_contiguous():
                raise TypeError("expected a contiguous float64 tensor")
            return x.data_ptr(), x
    except ImportError:
        pass
    if not isinstance(x, np.ndarray) or x.dtype != np.float64 or not x.flags.c_contiguous:
        raise TypeError("expected a contiguous float64 array")
    return x.ctypes.data, x


class KspaceBatch:
    """Many independent instances advanced by one captured CUDA graph (no counterpart
    in the reference, which holds one integrator per process).  Instance i's bins are
    entries offsets[i]:offsets[i+1] of the concatenated ("pool") arrays."""

    def __init__(self, instances):
        self.L = load_library()
        self.instances = list(instances)
        arr = (_vp * len(self.instances))(*[k.h for k in self.instances])
        h = _vp()
        _check(self.L.kspace_gpu_batch_create(C.byref(h), arr, len(self.instances)), "batch_create")
        self.h = h
        self.M = len(self.instances)
        self._grids = []
        self.nk = None
        self.offsets = None

    def close(self):
        if getattr(self, "h", None):
            self.L.kspace_gpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bind_grid(self, inst, grid, pmgrid, BoxSize):
        """Bin this CUDA complex64 grid into instance inst's delta_cdm every step and
        correct it in place afterwards."""
        ptr, keep = _grid_ptr(grid)
        self._grids.append(keep)
        _check(self.L.kspace_gpu_batch_bind_grid(self.h, inst, ptr, pmgrid, BoxSize), "batch_bind_grid")

    def init(self, a, nk, keff, dcdm):
        a = _f64(a)
        nk = np.ascontiguousarray(nk, dtype=np.int32)
        keff = _f64(keff)
        dcdm = _f64(dcdm)
        _check(self.L.kspace_gpu_batch_init(self.h, _pd(a), nk.ctypes.data_as(_PI), _pd(keff), _pd(dcdm)),
               "batch_init")
        self.nk = np.zeros(self.M, dtype=np.int32)
        self.offsets = np.zeros(self.M + 1, dtype=np.int32)
        _check(self.L.kspace_gpu_batch_layout(self.h, self.nk.ctypes.data_as(_PI), self.offsets.ctypes.data_as(_PI)),
               "batch_layout")

    def step(self, a, dcdm=None, dnu=None):
        """One step of every instance at a[i].  dcdm / dnu: pools (numpy or torch,
        host or CUDA); dnu=None returns a new numpy pool."""
        a = _f64(a)
        out = dnu
        if out is None:
            out = np.zeros(int(self.offsets[-1]), dtype=np.float64)
        dp, keep1 = _buf_ptr(dcdm if dcdm is None or not isinstance(dcdm, np.ndarray) else _f64(dcdm))
        op, keep2 = _buf_ptr(out)
        _check(self.L.kspace_gpu_batch_step(self.h, _pd(a), dp, op), "batch_step")
        return out

    def status(self):
        st = np.zeros(self.M, dtype=np.int32)
        _check(self.L.kspace_gpu_batch_status(self.h, st.ctypes.data_as(_PI)), "batch_status")
        return st

    def set_tuning(self, warps_per_block=4, blocks_per_sm=2, use_graph=True):
        _check(self.L.kspace_gpu_batch_set_tuning(self.h, warps_per_block, blocks_per_sm, int(use_graph)),
               "batch_set_tuning")

    def autotune(self, a, dcdm=None, reps=3):
        a = _f64(a)
        dp, keep = _buf_ptr(dcdm if dcdm is None or not isinstance(dcdm, np.ndarray) else _f64(dcdm))
        best = (C.c_int * 2)()
        ms = C.c_float()
        _check(self.L.kspace_gpu_batch_autotune(self.h, _pd(a), dp, reps, best, C.byref(ms)), "batch_autotune")
        return (best[0], best[1]), ms.value

    def last_ms(self):
        ms = C.c_float()
        _check(self.L.kspace_gpu_batch_last_ms(self.h, C.byref(ms)), "batch_last_ms")
        return ms.value


def make_instance(MNu, TimeTransfer, HubbleParam, Omega0, nk_alloc, TimeMax, logk, T_nu, UnitLength_in_cm=3.085678e24,
                  UnitTime_in_s=None, OmegaLambda=None, tcmb0=2.7255, include_radiation=True, device=0):
    """InitOmegaNu + allocate_kspace_memory with a transfer table given as arrays."""
    if UnitTime_in_s is None:
        UnitTime_in_s = UnitLength_in_cm / 1e5
    k = KspaceNeutrinos(device)
    k.init_omega_nu(MNu, TimeTransfer, HubbleParam, tcmb0)
    k.set_hubble(Omega0, OmegaLambda, UnitTime_in_s, include_radiation)
    k.alloc_table(nk_alloc, TimeTransfer, TimeMax, Omega0, UnitTime_in_s, UnitLength_in_cm)
    k.set_transfer(logk, T_nu)
    return k
