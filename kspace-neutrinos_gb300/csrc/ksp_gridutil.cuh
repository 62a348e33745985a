// ksp_gridutil.cuh -- per-mode arithmetic shared by the grid passes (binning K1,
// correction K3 and their adjoints): mode coordinates, the exact log bin of integer
// k^2, the CIC window factor and the correction interpolation.
#pragma once
#include <stdlib.h>
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include "ksp_internal.h"

namespace ksp {

// 2-D tensor map of a slab viewed as [nrows16][16 modes] complex64 (128-byte rows,
// 128-byte swizzle), box of `rows` rows; false if the driver entry point is missing or
// the grid pointer is not 16-byte aligned (ksp_grid.cu)
bool make_grid_tmap(CUtensorMap* map, const void* grid, long long nrows16, int rows);

struct GridArgs;
// warp-pipelined K1 / K3 (ksp_stream.cu): 0 launched, -1 not applicable, -2 launch error
int launch_bin_stream(const struct GridGeom& g, const GridArgs& a, const float* grid, double* bin_sum, double* F0sq,
                      unsigned* status, int warps, int stages, bool exact, cudaStream_t st);
int launch_correct_stream(const GridArgs& a, float* grid, struct CorrTable corr, unsigned* status, int warps,
                          int stages, cudaStream_t st);
// K1 over row-aligned runs of 17 modes (ksp_stream.cu): same return codes
int launch_bin_rows(const struct GridGeom& g, const GridArgs& a, const float* grid, double* bin_sum, double* F0sq,
                    unsigned* status, int warps, int stages, bool exact, cudaStream_t st);

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
    int first_wait;  // poll limit of the binning pass's first bounded wait (2^22; a test may shorten it)
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
// mode_power2 with the k_z weight taken from a table (1 on the z = 0 and N/2 planes, 2
// elsewhere): multiplying |F|^2 by it is exact, so the pair equals mode_power2's.
__device__ __forceinline__ ModeP mode_power2w(float re, float im, const ModeCursor& c, const float* w1,
                                              const float* wt) {
    const float t = __fmul_rn(c.iwxy, w1[c.z]);
    const float inv = __fmul_rn(t, t);
    const float f_hi = __fmul_rn(inv, inv);
    const float f_lo = fmaf(inv, inv, -f_hi);
    const float F2 = __fmul_rn(__fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im)), wt[c.z]);
    ModeP p;
    p.hi = __fmul_rn(F2, f_hi);
    p.lo = __fadd_rn(fmaf(F2, f_hi, -p.hi), __fmul_rn(F2, f_lo));
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

// (h, l) += (oh, ol) for float pairs: TwoSum of the high parts, the low parts and the
// error carried in the low part, then renormalised.
__device__ __forceinline__ void pair_add(float& h, float& l, float oh, float ol) {
    const float s = __fadd_rn(h, oh);
    const float bb = __fsub_rn(s, h);
    const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(oh, bb));
    const float t = __fadd_rn(e, __fadd_rn(l, ol));
    h = __fadd_rn(s, t);
    l = __fsub_rn(t, __fsub_rn(h, s));
}

// Warp-wide flush of one float pair per lane into the CTA totals: lanes are consecutive
// stretches of the grid, so equal bins sit in runs of neighbouring lanes; a segmented
// scan (TwoSum pairs) leaves each run's total on its last lane, which alone touches the
// shared totals.  key < 0: nothing to add.  Called by all 32 lanes together.
__device__ __forceinline__ void warp_flush_pairs(int key, float h, float l, float* H, float* L) {
    const int lane = threadIdx.x & 31;
    const int up = __shfl_up_sync(0xffffffffu, key, 1);
    const bool head = lane == 0 || up != key;
    const unsigned heads = __ballot_sync(0xffffffffu, head);
    const int my_head = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const float oh = __shfl_up_sync(0xffffffffu, h, d);
        const float ol = __shfl_up_sync(0xffffffffu, l, d);
        if (lane - d >= my_head) pair_add(h, l, oh, ol);
    }
    const bool tail = lane == 31 || ((heads >> (lane + 1)) & 1u);
    if (tail && key >= 0 && (h != 0.f || l != 0.f)) pair_atomic_add(H, L, key, h, l);
}

// Two adjacent bins b, b+1 as float pairs (h: the exact float sum of the high parts,
// l: the sum of their TwoSum errors and of the low parts).  A mode outside
// [thr[b], thr[b+2]) -- in practice a thread's first mode of a row -- sends the pairs to
// the warp's own bin totals and restarts the window at the mode's bin.
struct BinPairAcc2 {
    int b = -1, tlo = 1, t1 = 0, t2 = 0;
    float h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f;
    __device__ __forceinline__ void flush(float* H, float* L) {
        if (h0 != 0.f || l0 != 0.f) pair_atomic_add(H, L, b, h0, l0);
        if (h1 != 0.f || l1 != 0.f) pair_atomic_add(H, L, b + 1, h1, l1);
        h0 = l0 = h1 = l1 = 0.f;
    }
    __device__ __forceinline__ void add(int k2, ModeP p, const GridArgs& g, const int* thr, float* H, float* L) {
        if (k2 < tlo || k2 >= t2) {
            flush(H, L);
            b = bin_of(k2, g.c1, thr, g.nrbins);
            tlo = thr[b];
            t1 = thr[b + 1];
            t2 = b + 2 <= g.nrbins ? thr[b + 2] : 0x7fffffff;
        }
        const bool up = k2 >= t1;
        const float h = up ? h1 : h0;
        const float s = __fadd_rn(h, p.hi);
        const float bb = __fsub_rn(s, h);
        const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(p.hi, bb));
        const float l = __fadd_rn(up ? l1 : l0, __fadd_rn(e, p.lo));
        if (up) { h1 = s; l1 = l; } else { h0 = s; l0 = l; }
    }
};

// Three adjacent bins b, b+1, b+2 accumulated as float pairs: a mode costs three
// compares and a few selects unless it leaves [thr[b], thr[b+3]) -- in practice only at
// a thread's first mode of a row, where the window restarts at the mode's bin (a row
// of 8 modes spans more than three bins rarely: k^2 grows slowly along z).  The pairs
// go to the CTA totals at the end of the row, by all lanes together (flush_warp).
struct BinWinAcc {
    int b = -1, tlo = 1, t1 = 0, t2 = 0, t3 = 0;
    float h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f, h2 = 0.f, l2 = 0.f;
    // single-thread flush (the rare window restarts inside a row)
    __device__ __forceinline__ void flush(float* H, float* L) {
        if (h0 != 0.f || l0 != 0.f) pair_atomic_add(H, L, b, h0, l0);
        if (h1 != 0.f || l1 != 0.f) pair_atomic_add(H, L, b + 1, h1, l1);
        if (h2 != 0.f || l2 != 0.f) pair_atomic_add(H, L, b + 2, h2, l2);
        h0 = l0 = h1 = l1 = h2 = l2 = 0.f;
    }
    // end of a row: all lanes of the warp
    __device__ __forceinline__ void flush_warp(float* H, float* L) {
        warp_flush_pairs(b >= 0 ? b : -1, h0, l0, H, L);
        warp_flush_pairs(b >= 0 ? b + 1 : -1, h1, l1, H, L);
        warp_flush_pairs(b >= 0 ? b + 2 : -1, h2, l2, H, L);
        h0 = l0 = h1 = l1 = h2 = l2 = 0.f;
    }
    __device__ __forceinline__ void add(int k2, ModeP p, const GridArgs& g, const int* thr, float* H, float* L) {
        if (k2 < tlo || k2 >= t3) {
            flush(H, L);
            b = bin_of(k2, g.c1, thr, g.nrbins);
            tlo = thr[b];
            t1 = thr[b + 1];
            t2 = b + 2 <= g.nrbins ? thr[b + 2] : 0x7fffffff;
            t3 = b + 3 <= g.nrbins ? thr[b + 3] : 0x7fffffff;
        }
        const bool u1 = k2 >= t1, u2 = k2 >= t2;
        float h = u2 ? h2 : (u1 ? h1 : h0);
        float l = u2 ? l2 : (u1 ? l1 : l0);
        pair_add(h, l, p.hi, p.lo);
        if (u2) { h2 = h; l2 = l; } else if (u1) { h1 = h; l1 = l; } else { h0 = h; l0 = l; }
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
    int j = -2;  // segment index: -1 below the table, nk-1 from the last node on
    float xlo = 3.0e38f, xhi = -3.0e38f, x0 = 0.f, sl = 0.f, r0 = 0.f, xwarn = -3.0e38f;
    __device__ __forceinline__ void set(int jj, const CorrSmem& t, int nk) {
        j = jj;
        xwarn = -3.0e38f;
        if (jj < 0) {  // below the first node: constant
            xlo = -3.0e38f; xhi = t.xf[0]; x0 = 0.f; sl = 0.f; r0 = t.rn[0];
            xwarn = t.xf[0] - 0.69314718f;
        } else if (jj >= nk - 1) {  // from the last node on: constant
            xlo = t.xf[nk - 1]; xhi = 3.0e38f; x0 = 0.f; sl = 0.f; r0 = t.rn[nk - 1];
        } else {
            xlo = t.xf[jj]; xhi = t.xf[jj + 1]; x0 = xlo; sl = t.sn[jj]; r0 = t.rn[jj];
        }
    }
    __device__ __forceinline__ void locate(float x, const CorrSmem& t, int nk) {
        int lo = -1, hi = nk;  // largest j with xf[j] <= x
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (t.xf[mid] <= x) lo = mid; else hi = mid;
        }
        set(lo, t, nk);
    }
    __device__ __forceinline__ float delta(int k2, float lnscale, const CorrSmem& t, int nk, unsigned& flags) {
        const float x = fmaf(0.5f, __logf((float)k2), lnscale);
        if (x >= xhi && j > -2) {  // along a column x grows: usually the next segment
            set(j + 1, t, nk);
            if (x >= xhi) locate(x, t, nk);
        } else if (x < xlo) {
            locate(x, t, nk);
        }
        if (x < xwarn) flags |= kStKWarn;
        return fmaf(x - x0, sl, r0);  // the constant ends have sl = 0: exactly r0
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


// The poll limit of the first bounded wait of the default binning pass: 2^22, or, for
// the test of the expiry path (a wait that runs out ends the pass with
// KSPACE_ERR_TIMEOUT after draining its copies, with no fault), the value of
// KSPACE_GPU_TEST_FIRST_WAIT read once per process.
inline int first_wait_limit() {
    static int v = -1;
    if (v < 0) {
        const char* e = getenv("KSPACE_GPU_TEST_FIRST_WAIT");
        v = e ? atoi(e) : (1 << 22);
        if (v < 0) v = 0;
    }
    return v;
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
    a.first_wait = first_wait_limit();
    return a;
}

}  // namespace ksp
