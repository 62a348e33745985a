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

// ------------------------------------------------------------------ K3 helpers
struct CorrSmem {
    const int* thr; const int* cmap; const float* xf; const float* rn; const float* sn;
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
