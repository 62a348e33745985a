// ksp_gridutil.cuh -- per-mode arithmetic shared by the grid passes (binning K1,
// correction K3 and their adjoints): mode coordinates, the exact log bin of integer
// k^2, the CIC window factor and the correction interpolation.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "ksp_internal.h"

namespace ksp {

// n / d for n < 2^31: m = floor(2^s/d)+1 with s = 31 + ceil(log2 d)
struct FastDiv {
    uint32_t d, m;
    int s;
};
inline FastDiv make_fastdiv(uint32_t d) {
    FastDiv f;
    f.d = d;
    int l = 0;
    while ((1u << l) < d) l++;
    f.s = 31 + l;
    f.m = (uint32_t)((((unsigned __int128)1) << f.s) / d + 1);
    return f;
}
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
    return (uint32_t)(((uint64_t)n * f.m) >> f.s);
}

struct GridArgs {
    int N, nz, half, slab0, nrbins, nk;
    long long nmodes, nrows16;
    float c1;       // binsperunit * ln2 / 2: bin ~ c1 * log2(k^2)
    float lnscale;  // log(2 pi / BoxSize) (K3)
    FastDiv fd_nz, fd_N;
};

__device__ __forceinline__ int kval(int n, int N) { return n <= N / 2 ? n : n - N; }

// reference bin of integer k^2 >= 1: max b with thresh[b] <= k2
__device__ __forceinline__ int bin_of(int k2, float c1, const int* thr, int nb) {
    int b = __float2int_rd(c1 * __log2f((float)k2));
    b = b < 0 ? 0 : (b > nb - 1 ? nb - 1 : b);
    while (b > 0 && k2 < thr[b]) b--;
    while (b < nb - 1 && k2 >= thr[b + 1]) b++;
    return b;
}

// Mode coordinates that advance through a row of the slab.
struct ModeCursor {
    int il, j, z;       // local slab, second index, z
    int kxy2;
    float iwxy;
    __device__ __forceinline__ void set_row(const GridArgs& g, const float* w1) {
        const int kx = kval(g.slab0 + il, g.N), ky = kval(j, g.N);
        kxy2 = kx * kx + ky * ky;
        iwxy = __fmul_rn(w1[kx < 0 ? -kx : kx], w1[ky < 0 ? -ky : ky]);
    }
    __device__ __forceinline__ void init(const GridArgs& g, const float* w1, long long row_base, int z_base, int add) {
        // row_base/z_base: decoded flat mode index of the tile start; add: modes from there
        const uint32_t o = (uint32_t)(z_base + add);
        const uint32_t dr = fdiv(o, g.fd_nz);
        z = (int)(o - dr * (uint32_t)g.nz);
        const uint32_t r = (uint32_t)(row_base + dr);
        const uint32_t i = fdiv(r, g.fd_N);
        il = (int)i;
        j = (int)(r - i * (uint32_t)g.N);
        set_row(g, w1);
    }
    __device__ __forceinline__ void next(const GridArgs& g, const float* w1) {
        if (++z == g.nz) {
            z = 0;
            if (++j == g.N) { j = 0; il++; }
            set_row(g, w1);
        }
    }
};

// Coordinates for K3, which needs only k^2.
struct KCursor {
    int il, j, z, kxy2;
    __device__ __forceinline__ void set_row(const GridArgs& g) {
        const int kx = kval(g.slab0 + il, g.N), ky = kval(j, g.N);
        kxy2 = kx * kx + ky * ky;
    }
    __device__ __forceinline__ void init(const GridArgs& g, long long row_base, int z_base, int add) {
        const uint32_t o = (uint32_t)(z_base + add);
        const uint32_t dr = fdiv(o, g.fd_nz);
        z = (int)(o - dr * (uint32_t)g.nz);
        const uint32_t r = (uint32_t)(row_base + dr);
        const uint32_t i = fdiv(r, g.fd_N);
        il = (int)i;
        j = (int)(r - i * (uint32_t)g.N);
        set_row(g);
    }
    __device__ __forceinline__ void next(const GridArgs& g) {
        if (++z == g.nz) {
            z = 0;
            if (++j == g.N) { j = 0; il++; }
            set_row(g);
        }
    }
};

// K1 contribution of one mode: w |F|^2 W^4 with W the product of the 1-D inverse windows.
// |F|^2 and the window product are formed in float exactly as the reference does
// (powerspectrum.c:16-24,68,76,84); the reference then multiplies the float |F|^2 by
// the exact double square of the float window factor.  That product is carried here
// as an unevaluated float pair (hi + lo, FMA error terms) accurate to ~2^-48.
struct ModeP { float hi, lo; };
__device__ __forceinline__ ModeP mode_power2(float re, float im, const ModeCursor& c, const float* w1, int half) {
    const float t = __fmul_rn(c.iwxy, w1[c.z]);
    const float inv = __fmul_rn(t, t);
    const float f_hi = __fmul_rn(inv, inv);
    const float f_lo = fmaf(inv, inv, -f_hi);            // inv^2 = f_hi + f_lo exactly
    const float F2 = __fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im));
    ModeP p;
    p.hi = __fmul_rn(F2, f_hi);
    p.lo = __fadd_rn(fmaf(F2, f_hi, -p.hi), __fmul_rn(F2, f_lo));
    if (c.z != 0 && c.z != half) { p.hi = p.hi + p.hi; p.lo = p.lo + p.lo; }
    return p;
}
// the same value in double (plain and tail paths)
__device__ __forceinline__ double mode_power_d(float re, float im, const ModeCursor& c, const float* w1, int half) {
    const float t = __fmul_rn(c.iwxy, w1[c.z]);
    const float inv = __fmul_rn(t, t);
    const float F2 = __fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im));
    double p = (double)F2 * ((double)inv * (double)inv);
    if (c.z != 0 && c.z != half) p += p;
    return p;
}

// Sum of a run of modes in one bin as a float pair (hi, lo) with error-free
// additions (Knuth's TwoSum), flushed once per run as a double.
struct RunAcc {
    int b = -1;
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(int bin, ModeP p, double* hist) {
        if (bin == b) {
            const float s = __fadd_rn(hi, p.hi);
            const float bb = __fsub_rn(s, hi);
            const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p.hi, bb));
            const float t = __fadd_rn(e, __fadd_rn(lo, p.lo));
            hi = __fadd_rn(s, t);
            lo = __fsub_rn(t, __fsub_rn(hi, s));
        } else {
            flush(hist);
            b = bin; hi = p.hi; lo = p.lo;
        }
    }
    __device__ __forceinline__ void flush(double* hist) {
        if (b >= 0) atomicAdd(hist + b, (double)hi + (double)lo);
        b = -1;
    }
};

// Per-CTA bin totals as float pairs (H, L) in shared memory, updated with FP32 atomics
// only: H[b] += v by an atomic that returns the old value; the rounding error of that
// addition is recomputed exactly (TwoSum of the old value and v; the hardware adds with
// round-to-nearest) and added, with v's own low part, to L[b].  H + L then carries the
// bin total to ~2^-48 relative, without the FP64 pipe.
__device__ __forceinline__ void pair_atomic_add(float* H, float* L, int b, float hi, float lo) {
    const float old = atomicAdd(H + b, hi);
    const float s = __fadd_rn(old, hi);
    const float bb = __fsub_rn(s, old);
    const float e = __fadd_rn(__fsub_rn(old, __fsub_rn(s, bb)), __fsub_rn(hi, bb));
    atomicAdd(L + b, __fadd_rn(e, lo));
}

// A run of modes in one bin, accumulated as a float pair with TwoSum; the bin is
// tracked by its integer k^2 range [tlo, thi), so a mode costs two compares unless it
// leaves the range.
struct RunAcc32 {
    int b = -1, tlo = 1, thi = 0;
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void flush(float* H, float* L) {
        if (b >= 0) pair_atomic_add(H, L, b, hi, lo);
        hi = 0.f;
        lo = 0.f;
    }
    __device__ __forceinline__ void enter(int k2, const GridArgs& g, const int* thr, float* H, float* L) {
        if (k2 < tlo || k2 >= thi) {
            flush(H, L);
            b = bin_of(k2, g.c1, thr, g.nrbins);
            tlo = thr[b];
            thi = b + 1 < g.nrbins ? thr[b + 1] : 0x7fffffff;
        }
    }
    __device__ __forceinline__ void add(ModeP p) {
        const float s = __fadd_rn(hi, p.hi);
        const float bb = __fsub_rn(s, hi);
        const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p.hi, bb));
        const float t = __fadd_rn(e, __fadd_rn(lo, p.lo));
        hi = __fadd_rn(s, t);
        lo = __fsub_rn(t, __fsub_rn(hi, s));
    }
};

// Two adjacent bins b, b+1 accumulated as float pairs: a mode costs two compares and a
// select unless it leaves [thr[b], thr[b+2]), where both pairs go to the CTA totals and
// the window restarts at the mode's bin.  At the end of a thread's modes the pairs are
// flushed by all threads together.
struct BinPairAcc {
    int b = -1, tlo = 1, thi2 = 0, thi = 0;
    float ha = 0.f, la = 0.f, hb = 0.f, lb = 0.f;
    __device__ __forceinline__ void flush(float* H, float* L) {
        if (ha != 0.f || la != 0.f) pair_atomic_add(H, L, b, ha, la);
        if (hb != 0.f || lb != 0.f) pair_atomic_add(H, L, b + 1, hb, lb);
        ha = la = hb = lb = 0.f;
    }
    __device__ __forceinline__ void add(int k2, ModeP p, const GridArgs& g, const int* thr, float* H, float* L) {
        if (k2 < tlo || k2 >= thi2) {
            flush(H, L);
            b = bin_of(k2, g.c1, thr, g.nrbins);
            tlo = thr[b];
            thi = thr[b + 1];
            thi2 = b + 2 <= g.nrbins ? thr[b + 2] : 0x7fffffff;
        }
        const bool up = k2 >= thi;
        float h = up ? hb : ha, l = up ? lb : la;
        const float s = __fadd_rn(h, p.hi);
        const float bb = __fsub_rn(s, h);
        const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(p.hi, bb));
        const float t = __fadd_rn(e, __fadd_rn(l, p.lo));
        h = __fadd_rn(s, t);
        l = __fsub_rn(t, __fsub_rn(h, s));
        if (up) { hb = h; lb = l; } else { ha = h; la = l; }
    }
};

// ------------------------------------------------------------------ K3 helpers
struct CorrSmem {
    const int* thr; const int* cmap; const float* xf; const float* rn; const float* sn;
};

// The correction factor of one bin's modes, resolved once per bin: modes with
// x = log k below the bin's node use segment (x0a, sa, ra), the others (x0b, sb, rb);
// the same arithmetic as corr_delta.
struct CorrRun {
    int b = -1, tlo = 1, thi = 0;
    float xc, x0a, sa, ra, x0b, sb, rb, xwarn;
    bool bad;
    __device__ __forceinline__ void enter(int k2, const GridArgs& g, const CorrSmem& t) {
        if (k2 >= tlo && k2 < thi) return;
        b = bin_of(k2, g.c1, t.thr, g.nrbins);
        tlo = t.thr[b];
        thi = b + 1 < g.nrbins ? t.thr[b + 1] : 0x7fffffff;
        const int c = t.cmap[b];
        bad = c < 0;
        xwarn = -3.0e38f;
        if (bad) { xc = 0.f; x0a = x0b = 0.f; sa = sb = 0.f; ra = rb = 0.f; return; }
        const int nk = g.nk;
        xc = t.xf[c];
        if (c == 0) {  // below the first node: constant (delta_pow.c:26-29)
            x0a = 0.f; sa = 0.f; ra = t.rn[0];
            xwarn = t.xf[0] - 0.69314718f;
        } else {
            x0a = t.xf[c - 1]; sa = t.sn[c - 1]; ra = t.rn[c - 1];
        }
        if (c >= nk - 1) { x0b = 0.f; sb = 0.f; rb = t.rn[nk - 1]; }
        else { x0b = t.xf[c]; sb = t.sn[c]; rb = t.rn[c]; }
    }
    // correction minus one for a mode of this bin with integer k^2
    __device__ __forceinline__ float delta(int k2, float lnscale, unsigned& flags) const {
        const float x = fmaf(0.5f, __logf((float)k2), lnscale);
        if (bad) { flags |= kStGsl; return 0.f; }
        if (x < xwarn) flags |= kStKWarn;
        const bool below = x < xc;
        const float x0 = below ? x0a : x0b, sl = below ? sa : sb, r0 = below ? ra : rb;
        return fmaf(x - x0, sl, r0);  // the constant ends have sl = 0: exactly r0
    }
};

// The correction as a function of x = log k (delta_pow.c:19-37): linear on the
// segments [xf[j], xf[j+1]) of the table, constant below xf[0] and from xf[nk-1] on.
// A thread keeps its current segment and moves it only when x leaves [xlo, xhi).
struct SegTrack {
    float xlo = 3.0e38f, xhi = -3.0e38f, x0 = 0.f, sl = 0.f, r0 = 0.f, xwarn = -3.0e38f;
    __device__ __forceinline__ void locate(float x, const CorrSmem& t, int nk) {
        // largest j with xf[j] <= x (j = -1 below the table)
        int lo = -1, hi = nk;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (t.xf[mid] <= x) lo = mid; else hi = mid;
        }
        xwarn = -3.0e38f;
        if (lo < 0) {  // below the first node: constant
            xlo = -3.0e38f; xhi = t.xf[0]; x0 = 0.f; sl = 0.f; r0 = t.rn[0];
            xwarn = t.xf[0] - 0.69314718f;
        } else if (lo >= nk - 1) {  // from the last node on: constant
            xlo = t.xf[nk - 1]; xhi = 3.0e38f; x0 = 0.f; sl = 0.f; r0 = t.rn[nk - 1];
        } else {
            xlo = t.xf[lo]; xhi = t.xf[lo + 1]; x0 = t.xf[lo]; sl = t.sn[lo]; r0 = t.rn[lo];
        }
    }
    __device__ __forceinline__ float delta(int k2, float lnscale, const CorrSmem& t, int nk, unsigned& flags) {
        const float x = fmaf(0.5f, __logf((float)k2), lnscale);
        if (x < xlo || x >= xhi) locate(x, t, nk);
        if (x < xwarn) flags |= kStKWarn;
        return fmaf(x - x0, sl, r0);
    }
};

// 1 + norm*interp(log k) - 1 for a mode with integer k^2 (delta_pow.c:19-37 clamping)
__device__ __forceinline__ float corr_delta(int k2, const GridArgs& g, const CorrSmem& t, unsigned& flags) {
    const int b = bin_of(k2, g.c1, t.thr, g.nrbins);
    const int c = t.cmap[b];
    if (c < 0) { flags |= kStGsl; return 0.f; }
    const float x = fmaf(0.5f, __logf((float)k2), g.lnscale);
    const int nk = g.nk;
    if (x < t.xf[c]) {
        if (c == 0) {
            if (x < t.xf[0] - 0.69314718f) flags |= kStKWarn;
            return t.rn[0];
        }
        return fmaf(x - t.xf[c - 1], t.sn[c - 1], t.rn[c - 1]);
    }
    if (c >= nk - 1) return t.rn[nk - 1];
    return fmaf(x - t.xf[c], t.sn[c], t.rn[c]);
}


inline GridArgs make_grid_args(const GridGeom& g, int nk, float lnscale) {
    GridArgs a;
    a.N = g.N;
    a.nz = g.N / 2 + 1;
    a.half = g.N / 2;
    a.slab0 = g.slab0;
    a.nrbins = g.nrbins;
    a.nk = nk;
    a.nmodes = g.nmodes;
    a.nrows16 = g.nmodes / 16;
    a.c1 = g.bin_c1;
    a.lnscale = lnscale;
    a.fd_nz = make_fastdiv((uint32_t)a.nz);
    a.fd_N = make_fastdiv((uint32_t)g.N);
    return a;
}

}  // namespace ksp
