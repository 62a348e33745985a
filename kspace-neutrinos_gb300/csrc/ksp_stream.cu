// ksp_stream.cu -- warp-pipelined streaming passes over the half-complex grid: the
// binning pass (K1, powerspectrum.c:56-89) and the correction multiply (K3,
// interface_gadget.c:163-188).
//
// Each warp is a pipeline of its own: it owns a ring of STAGES shared-memory tiles of
// 32 rows x 16 modes (4 KB, 128-byte swizzle), its lane 0 keeps the ring full with 2-D
// TMA loads (and, for K3, writes each corrected tile back with a TMA store), and no
// barrier spans more than the warp.  A lane handles the 16 consecutive modes of one
// row.  Along such a run k^2 grows with z, so the bin (K1) or the interpolation
// segment (K3) can only step forward: each mode compares its integer k^2 with the next
// threshold, and a crossing is a few predicated moves, not a divergent branch.  A run
// starting below ksafe -- the k^2 under which some threshold gap is narrower than one
// k^2 step (2z + 1 <= 2 sqrt(k^2) + 1), so that a step could cross two thresholds --
// and a run that crosses the end of a grid row go to a warp-cooperative path instead,
// one mode per lane (low k and row ends: a few percent of the runs).
//
// K1 per mode: |F|^2 and the window factor inv = (w1x w1y w1z)^2 rounded in float as
// the reference forms them; the reference then multiplies |F|^2 inv^2 in double.  The
// exact variant carries that product and the run sums as float pairs (TwoSum), so
// the bin sums agree with the reference's double sums to ~1e-14; the lean variant
// rounds the product to float and sums a run (at most 16 modes) in plain FP32.  Both
// hand each closed run to the CTA's float-pair totals (compensated atomics) and the
// CTA totals to the global FP64 sums once.
//
// The default binning kernel is k_bin_mirror (further down): 17-mode runs of a grid row
// and of its mirror row (ky and -ky fall in the same bins), moved by 1-D bulk copies
// with their run-table rows, the two modes of a pair summed exactly before they are
// binned.  k_bin_rows, over tiles of whole grid rows and runs of one row, bins grids of
// more than 32 runs per row (N > 1086) and works without a run table.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>
#include "ksp_internal.h"
#include "ksp_gridutil.cuh"
#include "ksp_ptx.cuh"

namespace ksp {
namespace {

constexpr int kRowsPerWarp = 32;                // 16-mode rows per warp tile
constexpr int kTileBytes = kRowsPerWarp * 128;  // 4 KB
constexpr int kSpillSlots = 16;                 // bins a lane can close within one run
constexpr unsigned kFull = 0xffffffffu;
constexpr float kHalfLn2 = 0.34657359027997264f;

struct StreamPlan {
    size_t stage_off, bar_off, spill_off, hist_off, thr_off, tab_off, total;
};

// K1 shared memory (from a 1024-byte aligned base): stage rings | mbarriers | per-warp
// spill slots | float-pair bin totals | bin thresholds | {w1[z], multiplicity(z)}
__host__ __device__ inline StreamPlan plan_bin_stream(int warps, int stages, int nrbins, int nz, bool exact) {
    StreamPlan p{};
    size_t o = 0;
    p.stage_off = o;
    o += (size_t)warps * stages * kTileBytes;
    p.bar_off = o;
    o += sizeof(uint64_t) * (size_t)warps * stages;
    o = (o + 15) & ~size_t(15);
    p.spill_off = o;
    o += (size_t)warps * kSpillSlots * 32 * (exact ? 8 : 4);
    p.hist_off = o;
    o += sizeof(float) * 2 * (size_t)nrbins;
    p.thr_off = o;
    o += sizeof(int) * (size_t)(nrbins + 1);
    o = (o + 15) & ~size_t(15);
    p.tab_off = o;
    o += sizeof(float2) * (size_t)(nz + (nz >> 4) + 1);
    p.total = o + 1024;  // alignment slack
    return p;
}

// The z-window table is read at z, z+1, ..., z+15 by every lane at once, lanes 16 z
// apart: one padding entry after every 16 (entry z at z + z/16) spreads a warp's reads
// over all banks.
__device__ __forceinline__ int wpad(int z) { return z + (z >> 4); }

// K3 shared memory: stage rings | mbarriers | segments {x0, slope, value, next k^2} | k^2 thresholds
__host__ __device__ inline StreamPlan plan_corr_stream(int warps, int stages, int nk) {
    StreamPlan p{};
    size_t o = 0;
    p.stage_off = o;
    o += (size_t)warps * stages * kTileBytes;
    p.bar_off = o;
    o += sizeof(uint64_t) * (size_t)warps * stages;
    o = (o + 15) & ~size_t(15);
    p.tab_off = o;
    o += sizeof(float4) * (size_t)(nk + 1);
    p.thr_off = o;
    o += sizeof(int) * (size_t)(nk + 1);
    p.total = o + 1024;
    return p;
}

template <bool EXACT> struct SpillOf { typedef float type; };
template <> struct SpillOf<true> { typedef float2 type; };

// w |F|^2 inv^2 of one mode; w = {w1[z], multiplicity}, iwxy = w1x * w1y (float)
template <bool EXACT>
__device__ __forceinline__ void mode_value(float re, float im, float iwxy, float2 w, float& hi, float& lo) {
    const float t = __fmul_rn(iwxy, w.x);
    const float inv = __fmul_rn(t, t);
    const float F2 = __fmul_rn(__fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im)), w.y);
    const float f_hi = __fmul_rn(inv, inv);
    hi = __fmul_rn(F2, f_hi);
    if (EXACT) {
        const float f_lo = fmaf(inv, inv, -f_hi);
        lo = fmaf(F2, f_lo, fmaf(F2, f_hi, -hi));
    } else {
        lo = 0.f;
    }
}

// one mode of a fast run: close the current bin if k^2 reached the next threshold,
// then add the mode to the (new) current bin
template <bool EXACT>
__device__ __forceinline__ void bin_step(float re, float im, float iwxy, float2 w, int& k2, int& d, int& tnext,
                                         const int*& tq, typename SpillOf<EXACT>::type*& sp, float& h, float& l) {
    float phi, plo;
    mode_value<EXACT>(re, im, iwxy, w, phi, plo);
    const bool c = k2 >= tnext;
    if (c) {
        if constexpr (EXACT) *sp = make_float2(h, l);
        else *sp = h;
        sp += 32;
        ++tq;
        tnext = *tq;
    }
    const float h0 = c ? 0.f : h;
    if constexpr (EXACT) {
        const float l0 = c ? 0.f : l;
        const float s = __fadd_rn(h0, phi);
        const float bb = __fsub_rn(s, h0);
        const float e = __fadd_rn(__fsub_rn(h0, __fsub_rn(s, bb)), __fsub_rn(phi, bb));
        h = s;
        l = __fadd_rn(l0, __fadd_rn(e, plo));
    } else {
        h = __fadd_rn(h0, phi);
    }
    k2 += d;
    d += 2;
}

// The same step without a branch: the running sum of the current bin is stored to the
// lane's current slot every mode, and a crossing just moves on to the next slot and the
// next threshold.  After a run, slots 0..n hold the sums of bins b..b+n.
template <bool EXACT>
__device__ __forceinline__ void bin_step_slots(float re, float im, float iwxy, float2 w, int& k2, int& d,
                                               int& tnext, const int*& tq, typename SpillOf<EXACT>::type*& sp,
                                               float& h, float& l) {
    float phi, plo;
    mode_value<EXACT>(re, im, iwxy, w, phi, plo);
    const bool c = k2 >= tnext;
    sp += c ? 32 : 0;
    tq += c ? 1 : 0;
    tnext = *tq;
    const float h0 = c ? 0.f : h;
    if constexpr (EXACT) {
        const float l0 = c ? 0.f : l;
        const float s = __fadd_rn(h0, phi);
        const float bb = __fsub_rn(s, h0);
        const float e = __fadd_rn(__fsub_rn(h0, __fsub_rn(s, bb)), __fsub_rn(phi, bb));
        h = s;
        l = __fadd_rn(l0, __fadd_rn(e, plo));
        *sp = make_float2(h, l);
    } else {
        h = __fadd_rn(h0, phi);
        *sp = h;
    }
    k2 += d;
    d += 2;
}

// The same step with the crossing read from the run's bit mask (the run table): no k^2,
// no threshold load.
template <bool EXACT>
__device__ __forceinline__ void bin_step_bit(float re, float im, float iwxy, float2 w, bool c,
                                             typename SpillOf<EXACT>::type*& sp, float& h, float& l) {
    float phi, plo;
    mode_value<EXACT>(re, im, iwxy, w, phi, plo);
    sp += c ? 32 : 0;
    const float h0 = c ? 0.f : h;
    if constexpr (EXACT) {
        const float l0 = c ? 0.f : l;
        const float s = __fadd_rn(h0, phi);
        const float bb = __fsub_rn(s, h0);
        const float e = __fadd_rn(__fsub_rn(h0, __fsub_rn(s, bb)), __fsub_rn(phi, bb));
        h = s;
        l = __fadd_rn(l0, __fadd_rn(e, plo));
        *sp = make_float2(h, l);
    } else {
        h = __fadd_rn(h0, phi);
        *sp = h;
    }
}

__device__ __forceinline__ void add_pair(float* H, float* L, int b, float hi, float lo) {
    if (hi != 0.f || lo != 0.f) pair_atomic_add(H, L, b, hi, lo);
}

// Segmented sums of float pairs over the lanes of a warp: each run of equal key (in
// lane order) is summed, with error-free additions, onto its last lane (tail).
__device__ __forceinline__ void warp_seg_pair(int key, float& h, float& l, bool& tail) {
    const int lane = threadIdx.x & 31;
    const int up = __shfl_up_sync(kFull, key, 1);
    const unsigned heads = __ballot_sync(kFull, lane == 0 || up != key);
    const int my_head = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
#pragma unroll
    for (int dd = 1; dd < 32; dd <<= 1) {
        const float oh = __shfl_up_sync(kFull, h, dd), ol = __shfl_up_sync(kFull, l, dd);
        if (lane - dd >= my_head) pair_add(h, l, oh, ol);
    }
    tail = lane == 31 || ((heads >> (lane + 1)) & 1u);
}

template <int WARPS, int STAGES, bool EXACT>
__global__ void __launch_bounds__(WARPS * 32)
    k_bin_stream(const __grid_constant__ CUtensorMap tmap, GridArgs g, const int* __restrict__ thresh,
                 const float* __restrict__ w1g, const float* __restrict__ grid, double* bin_sum, double* F0sq,
                 unsigned* status, long long ntiles, int adv_r, int adv_z) {
    typedef typename SpillOf<EXACT>::type Spill;
    extern __shared__ unsigned char sm_raw[];
    __shared__ int s_gap;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const StreamPlan P = plan_bin_stream(WARPS, STAGES, g.nrbins, g.nz, EXACT);
    unsigned char* base = sm_raw + ((1024 - (ptx::smem_u32(sm_raw) & 1023)) & 1023);
    unsigned char* my_stage = base + P.stage_off + (size_t)warp * STAGES * kTileBytes;
    uint64_t* my_bar = reinterpret_cast<uint64_t*>(base + P.bar_off) + warp * STAGES;
    Spill* my_spill = reinterpret_cast<Spill*>(base + P.spill_off) + (size_t)warp * kSpillSlots * 32 + lane;
    float* s_H = reinterpret_cast<float*>(base + P.hist_off);
    float* s_L = s_H + g.nrbins;
    int* s_thr = reinterpret_cast<int*>(base + P.thr_off);
    float2* s_wt = reinterpret_cast<float2*>(base + P.tab_off);
    for (int i = tid; i < 2 * g.nrbins; i += blockDim.x) s_H[i] = 0.f;
    for (int i = tid; i <= g.nrbins; i += blockDim.x) s_thr[i] = thresh[i];
    for (int i = tid; i < g.nz; i += blockDim.x)
        s_wt[wpad(i)] = make_float2(w1g[i], (i == 0 || i == g.half) ? 1.f : 2.f);
    if (tid == 0) s_gap = -1;
    if (lane == 0) {
        for (int s = 0; s < STAGES; s++) ptx::mbar_init(&my_bar[s], 1);
        ptx::mbar_init_fence();
    }
    __syncthreads();
    // ksafe: the lower threshold of the highest reachable gap narrower than a k^2 step
    const int k2max = 3 * g.half * g.half;
    for (int b = tid; b < g.nrbins - 1; b += blockDim.x) {
        const int t0 = s_thr[b], t1 = s_thr[b + 1];
        if (t1 <= k2max && (float)(t1 - t0) < 2.f * sqrtf((float)t0) + 3.f) atomicMax(&s_gap, b);
    }
    __syncthreads();
    const int ksafe = s_gap >= 0 ? s_thr[s_gap] : 1;

    const int gw = blockIdx.x * WARPS + warp;
    const long long TW = (long long)gridDim.x * WARPS;
    const long long my_n = gw < ntiles ? (ntiles - 1 - gw) / TW + 1 : 0;
    if (lane == 0)
        for (int s = 0; s < STAGES && s < my_n; s++) {
            ptx::mbar_expect_tx(&my_bar[s], kTileBytes);
            ptx::tma_load_2d(my_stage + s * kTileBytes, &tmap, &my_bar[s], 0, (int)((gw + s * TW) * kRowsPerWarp));
        }
    // first mode of the warp's current tile: grid row rb of the slab, z zb
    const uint32_t mb = (uint32_t)gw * (kRowsPerWarp * 16);
    int rb = (int)fdiv(mb, g.fd_nz);
    int zb = (int)(mb - (uint32_t)rb * (uint32_t)g.nz);
    bool ok = true;
    long long k = 0;
    int s = 0;
    unsigned phase = 0;
    for (; k < my_n; k++) {
        const bool got = ptx::mbar_wait_bounded(&my_bar[s], phase);
        if (!__all_sync(kFull, got)) {
            ok = false;
            break;
        }
        const unsigned char* tb = my_stage + s * kTileBytes;
        const bool valid = (gw + k * TW) * kRowsPerWarp + lane < g.nrows16;
        // this lane's run: 16 modes from z of grid row pr
        const uint32_t o = (uint32_t)(zb + 16 * lane);
        const uint32_t dr = fdiv(o, g.fd_nz);
        const int z = (int)(o - dr * (uint32_t)g.nz);
        const int pr = rb + (int)dr;
        const int il = (int)fdiv((uint32_t)pr, g.fd_N);
        const int kx = kval(g.slab0 + il, g.N), ky = kval(pr - il * g.N, g.N);
        int k2 = kx * kx + ky * ky + z * z;
        const bool fast = valid && z + 15 < g.nz && k2 >= ksafe;
        if (fast) {
            const float iwxy = __fmul_rn(s_wt[wpad(kx < 0 ? -kx : kx)].x, s_wt[wpad(ky < 0 ? -ky : ky)].x);
            const float2* wz = s_wt + wpad(z);
            const int cut = 16 - (z & 15);  // modes from z + cut on sit past one more padding entry
            const int b = bin_of(k2, g.c1, s_thr, g.nrbins);
            const int* tq = s_thr + b + 1;
            int tnext = *tq;
            Spill* sp = my_spill;
            float h = 0.f, l = 0.f;
            int d = 2 * z + 1;
            const unsigned char* rp = tb + lane * 128;
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const float4 v = *reinterpret_cast<const float4*>(rp + ((u ^ (lane & 7)) << 4));
                bin_step<EXACT>(v.x, v.y, iwxy, wz[2 * u + (2 * u >= cut)], k2, d, tnext, tq, sp, h, l);
                bin_step<EXACT>(v.z, v.w, iwxy, wz[2 * u + 1 + (2 * u + 1 >= cut)], k2, d, tnext, tq, sp, h, l);
            }
            const int nsp = (int)(sp - my_spill) >> 5;
            for (int q = 0; q < nsp; q++) {
                const Spill v = my_spill[32 * q];
                if constexpr (EXACT) add_pair(s_H, s_L, b + q, v.x, v.y);
                else add_pair(s_H, s_L, b + q, v, 0.f);
            }
            add_pair(s_H, s_L, b + nsp, h, l);
        }
        // runs off the fast path: two at a time, one mode per lane
        unsigned slow = __ballot_sync(kFull, valid && !fast);
        while (slow) {
            const int L0 = __ffs(slow) - 1;
            slow &= slow - 1;
            int L1 = -1;
            if (slow) {
                L1 = __ffs(slow) - 1;
                slow &= slow - 1;
            }
            const int L = lane < 16 ? L0 : L1;
            const int zL = __shfl_sync(kFull, z, L < 0 ? 0 : L);
            const int pL = __shfl_sync(kFull, pr, L < 0 ? 0 : L);
            int key = -1;
            float phi = 0.f, plo = 0.f;
            if (L >= 0) {
                const int i = lane & 15;
                int zz = zL + i, pp = pL;
                while (zz >= g.nz) {
                    zz -= g.nz;
                    pp++;
                }
                const int il2 = (int)fdiv((uint32_t)pp, g.fd_N);
                const int kx2 = kval(g.slab0 + il2, g.N), ky2 = kval(pp - il2 * g.N, g.N);
                const int k2m = kx2 * kx2 + ky2 * ky2 + zz * zz;
                if (k2m != 0) {
                    const float2 v = *reinterpret_cast<const float2*>(tb + L * 128 + (((i >> 1) ^ (L & 7)) << 4) +
                                                                      (i & 1) * 8);
                    const float iw =
                        __fmul_rn(s_wt[wpad(kx2 < 0 ? -kx2 : kx2)].x, s_wt[wpad(ky2 < 0 ? -ky2 : ky2)].x);
                    mode_value<EXACT>(v.x, v.y, iw, s_wt[wpad(zz)], phi, plo);
                    key = bin_of(k2m, g.c1, s_thr, g.nrbins);
                }
            }
            // consecutive modes mostly share a bin: one shared-memory update per run
            bool tail;
            warp_seg_pair(key, phi, plo, tail);
            if (tail && key >= 0) add_pair(s_H, s_L, key, phi, plo);
        }
        __syncwarp();
        if (lane == 0 && k + STAGES < my_n) {
            ptx::mbar_expect_tx(&my_bar[s], kTileBytes);
            ptx::tma_load_2d(my_stage + s * kTileBytes, &tmap, &my_bar[s], 0,
                             (int)((gw + (k + STAGES) * TW) * kRowsPerWarp));
        }
        if (++s == STAGES) {
            s = 0;
            phase ^= 1;
        }
        zb += adv_z;
        rb += adv_r;
        if (zb >= g.nz) {
            zb -= g.nz;
            rb++;
        }
    }
    if (!ok && lane == 0) {
        // wait (bounded) for this warp's loads still in flight, then leave the tiles
        atomicOr(status, kStTimeout);
        for (long long kk = k; kk < my_n && kk < k + STAGES; kk++) {
            ptx::mbar_wait_bounded(&my_bar[s], phase);
            if (++s == STAGES) {
                s = 0;
                phase ^= 1;
            }
        }
    }
    __syncthreads();
    if (blockIdx.x == 0 && tid == 0) {
        // the modes after the last full 16-mode row
        for (long long m = g.nrows16 * 16; m < g.nmodes; m++) {
            const long long rr = m / g.nz;
            const int zz = (int)(m - rr * g.nz);
            const int il2 = (int)(rr / g.N);
            const int kx2 = kval(g.slab0 + il2, g.N), ky2 = kval((int)(rr - (long long)il2 * g.N), g.N);
            const int k2m = kx2 * kx2 + ky2 * ky2 + zz * zz;
            if (k2m == 0) continue;
            const float iw = __fmul_rn(s_wt[wpad(kx2 < 0 ? -kx2 : kx2)].x, s_wt[wpad(ky2 < 0 ? -ky2 : ky2)].x);
            float phi, plo;
            mode_value<EXACT>(grid[2 * m], grid[2 * m + 1], iw, s_wt[wpad(zz)], phi, plo);
            add_pair(s_H, s_L, bin_of(k2m, g.c1, s_thr, g.nrbins), phi, plo);
        }
        if (g.slab0 == 0 && g.nmodes > 0) {
            const float re = grid[0], im = grid[1];
            *F0sq = (double)__fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im));
        }
    }
    __syncthreads();
    for (int b = tid; b < g.nrbins; b += blockDim.x) {
        const double v = (double)s_H[b] + (double)s_L[b];
        if (v != 0.0) atomicAdd(bin_sum + b, v);
    }
}

// ------------------------------------------------------------------ K3
// one mode of a fast run: step to the next segment if k^2 reached its start, then
// multiply by 1 + (value + slope (log k - x0))
__device__ __forceinline__ void corr_step(float& re, float& im, int& k2, int& d, int& tnext, const float4*& sq,
                                          float4& cs, float lnscale) {
    if (k2 >= tnext) {
        ++sq;
        cs = *sq;
        tnext = __float_as_int(cs.w);
    }
    const float x = fmaf(__log2f((float)k2), kHalfLn2, lnscale);
    const float f = fmaf(x - cs.x, cs.y, cs.z);
    re = fmaf(re, f, re);
    im = fmaf(im, f, im);
    k2 += d;
    d += 2;
}

// segment of k^2: the number of node thresholds at or below it
__device__ __forceinline__ int seg_of(int k2, const int* k2t, int nk) {
    int lo = 0, hi = nk;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (k2t[mid] <= k2) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

template <int WARPS, int STAGES>
__global__ void __launch_bounds__(WARPS * 32)
    k_correct_stream(const __grid_constant__ CUtensorMap tmap, GridArgs g, CorrTable corr, float* grid,
                     unsigned* status, long long ntiles, int adv_r, int adv_z) {
    extern __shared__ unsigned char sm_raw[];
    __shared__ int s_gap, s_abort;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nk = g.nk;
    const StreamPlan P = plan_corr_stream(WARPS, STAGES, nk);
    unsigned char* base = sm_raw + ((1024 - (ptx::smem_u32(sm_raw) & 1023)) & 1023);
    unsigned char* my_stage = base + P.stage_off + (size_t)warp * STAGES * kTileBytes;
    uint64_t* my_bar = reinterpret_cast<uint64_t*>(base + P.bar_off) + warp * STAGES;
    float4* s_seg = reinterpret_cast<float4*>(base + P.tab_off);
    int* s_k2t = reinterpret_cast<int*>(base + P.thr_off);
    // the first tiles' loads go out first, and land while the tables are built; the grid
    // is read and written once, so its lines leave L2 first
    const uint64_t pol = ptx::policy_evict_first();
    const int gw = blockIdx.x * WARPS + warp;
    const long long TW = (long long)gridDim.x * WARPS;
    const long long my_n = gw < ntiles ? (ntiles - 1 - gw) / TW + 1 : 0;
    if (lane == 0) {
        for (int s = 0; s < STAGES; s++) ptx::mbar_init(&my_bar[s], 1);
        ptx::mbar_init_fence();
        for (int s = 0; s < STAGES - 1 && s < my_n; s++) {
            ptx::mbar_expect_tx(&my_bar[s], kTileBytes);
            ptx::tma_load_2d_hint(my_stage + s * kTileBytes, &tmap, &my_bar[s], 0, (int)((gw + s * TW) * kRowsPerWarp), pol);
        }
    }
    // an error of the step so far (the reference terminates before the multiply): the
    // grid stays as it is
    if (tid == 0) s_abort = (*reinterpret_cast<volatile unsigned*>(status) & kStAbort) != 0u;
    // segment s covers k^2 in [k2t[s-1], k2t[s]): s = 0 below the first node (value of
    // node 0), 1..nk-1 the linear pieces between nodes, nk from the last node on (its
    // value) -- the clamped interpolation of delta_pow.c:19-37 in log k.  k2t[j]: the
    // first integer k^2 whose log k reaches node j.
    for (int j = tid; j < nk; j += blockDim.x) {
        const float e = expf(2.f * (corr.xf[j] - g.lnscale));
        int t = e >= 1.0e9f ? 1000000000 : (int)ceilf(e);
        s_k2t[j] = t < 1 ? 1 : t;
    }
    if (tid == 0) {
        s_k2t[nk] = 0x7fffffff;
        s_gap = -1;
    }
    __syncthreads();
    if (s_abort) {
        if (lane == 0)
            for (int s = 0; s < STAGES - 1 && s < my_n; s++) ptx::mbar_wait_bounded(&my_bar[s], 0);
        return;
    }
    for (int s = tid; s <= nk; s += blockDim.x) {
        float4 v;
        if (s == 0) v = make_float4(0.f, 0.f, corr.rn[0], 0.f);
        else if (s == nk) v = make_float4(0.f, 0.f, corr.rn[nk - 1], 0.f);
        else v = make_float4(corr.xf[s - 1], corr.sn[s - 1], corr.rn[s - 1], 0.f);
        v.w = __int_as_float(s_k2t[s]);
        s_seg[s] = v;
    }
    const int k2max = 3 * g.half * g.half;
    for (int j = tid; j < nk - 1; j += blockDim.x) {
        const int t0 = s_k2t[j], t1 = s_k2t[j + 1];
        if (t1 <= k2max && (float)(t1 - t0) < 2.f * sqrtf((float)t0) + 3.f) atomicMax(&s_gap, j);
    }
    __syncthreads();
    const int ksafe = s_gap >= 0 ? s_k2t[s_gap] : 1;
    const float xwarn = corr.xf[0] - 0.69314718f;

    const uint32_t mb = (uint32_t)gw * (kRowsPerWarp * 16);
    int rb = (int)fdiv(mb, g.fd_nz);
    int zb = (int)(mb - (uint32_t)rb * (uint32_t)g.nz);
    unsigned flags = 0;
    bool ok = true;
    long long k = 0;
    int s = 0, s2 = STAGES - 1;  // stage of tile k, and of tile k + STAGES - 1
    unsigned phase = 0;
    for (; k < my_n; k++) {
        const long long tile = gw + k * TW;
        const bool got = ptx::mbar_wait_bounded(&my_bar[s], phase);
        if (!__all_sync(kFull, got)) {
            ok = false;
            break;
        }
        unsigned char* tb = my_stage + s * kTileBytes;
        const bool valid = tile * kRowsPerWarp + lane < g.nrows16;
        const uint32_t o = (uint32_t)(zb + 16 * lane);
        const uint32_t dr = fdiv(o, g.fd_nz);
        const int z = (int)(o - dr * (uint32_t)g.nz);
        const int pr = rb + (int)dr;
        const int il = (int)fdiv((uint32_t)pr, g.fd_N);
        const int kx = kval(g.slab0 + il, g.N), ky = kval(pr - il * g.N, g.N);
        int k2 = kx * kx + ky * ky + z * z;
        const bool fast = valid && z + 15 < g.nz && k2 >= ksafe;
        if (fast) {
            const float4* sq = s_seg + seg_of(k2, s_k2t, nk);
            // log k grows along the run: only its first mode can be far below node 0
            if (sq == s_seg && fmaf(__log2f((float)k2), kHalfLn2, g.lnscale) < xwarn) flags |= kStKWarn;
            float4 cs = *sq;
            int tnext = __float_as_int(cs.w);
            int d = 2 * z + 1;
            unsigned char* rp = tb + lane * 128;
#pragma unroll
            for (int u = 0; u < 8; u++) {
                float4* vp = reinterpret_cast<float4*>(rp + ((u ^ (lane & 7)) << 4));
                float4 v = *vp;
                corr_step(v.x, v.y, k2, d, tnext, sq, cs, g.lnscale);
                corr_step(v.z, v.w, k2, d, tnext, sq, cs, g.lnscale);
                *vp = v;
            }
        }
        unsigned slow = __ballot_sync(kFull, valid && !fast);
        while (slow) {
            const int L0 = __ffs(slow) - 1;
            slow &= slow - 1;
            int L1 = -1;
            if (slow) {
                L1 = __ffs(slow) - 1;
                slow &= slow - 1;
            }
            const int L = lane < 16 ? L0 : L1;
            const int zL = __shfl_sync(kFull, z, L < 0 ? 0 : L);
            const int pL = __shfl_sync(kFull, pr, L < 0 ? 0 : L);
            if (L >= 0) {
                const int i = lane & 15;
                int zz = zL + i, pp = pL;
                while (zz >= g.nz) {
                    zz -= g.nz;
                    pp++;
                }
                const int il2 = (int)fdiv((uint32_t)pp, g.fd_N);
                const int kx2 = kval(g.slab0 + il2, g.N), ky2 = kval(pp - il2 * g.N, g.N);
                const int k2m = kx2 * kx2 + ky2 * ky2 + zz * zz;
                if (k2m != 0) {
                    float2* vp = reinterpret_cast<float2*>(tb + L * 128 + (((i >> 1) ^ (L & 7)) << 4) + (i & 1) * 8);
                    const float x = fmaf(__log2f((float)k2m), kHalfLn2, g.lnscale);
                    const int sg = seg_of(k2m, s_k2t, nk);
                    const float4 cs = s_seg[sg];
                    if (x < xwarn) flags |= kStKWarn;
                    const float f = fmaf(x - cs.x, cs.y, cs.z);
                    float2 v = *vp;
                    v.x = fmaf(v.x, f, v.x);
                    v.y = fmaf(v.y, f, v.y);
                    *vp = v;
                }
            }
        }
        ptx::fence_async_smem();
        __syncwarp();
        if (lane == 0) {
            ptx::tma_store_2d_hint(&tmap, tb, 0, (int)(tile * kRowsPerWarp), pol);
            ptx::bulk_commit();
            if (k + STAGES - 1 < my_n) {
                ptx::bulk_wait_read_le1();  // the store from stage s2 (one tile ago) has read it
                ptx::mbar_expect_tx(&my_bar[s2], kTileBytes);
                ptx::tma_load_2d_hint(my_stage + s2 * kTileBytes, &tmap, &my_bar[s2], 0,
                                 (int)((gw + (k + STAGES - 1) * TW) * kRowsPerWarp), pol);
            }
        }
        if (++s == STAGES) {
            s = 0;
            phase ^= 1;
        }
        if (++s2 == STAGES) s2 = 0;
        zb += adv_z;
        rb += adv_r;
        if (zb >= g.nz) {
            zb -= g.nz;
            rb++;
        }
    }
    if (lane == 0) {
        if (!ok) {
            atomicOr(status, kStTimeout);
            for (long long kk = k; kk < my_n && kk < k + STAGES - 1; kk++) {
                ptx::mbar_wait_bounded(&my_bar[s], phase);
                if (++s == STAGES) {
                    s = 0;
                    phase ^= 1;
                }
            }
        }
        ptx::bulk_wait_all();
    }
    if (blockIdx.x == 0 && tid == 0) {
        // the modes after the last full 16-mode row
        for (long long m = g.nrows16 * 16; m < g.nmodes; m++) {
            const long long rr = m / g.nz;
            const int zz = (int)(m - rr * g.nz);
            const int il2 = (int)(rr / g.N);
            const int kx2 = kval(g.slab0 + il2, g.N), ky2 = kval((int)(rr - (long long)il2 * g.N), g.N);
            const int k2m = kx2 * kx2 + ky2 * ky2 + zz * zz;
            if (k2m == 0) continue;
            const float x = fmaf(__log2f((float)k2m), kHalfLn2, g.lnscale);
            const float4 cs = s_seg[seg_of(k2m, s_k2t, nk)];
            if (x < xwarn) flags |= kStKWarn;
            const float f = fmaf(x - cs.x, cs.y, cs.z);
            grid[2 * m] = fmaf(grid[2 * m], f, grid[2 * m]);
            grid[2 * m + 1] = fmaf(grid[2 * m + 1], f, grid[2 * m + 1]);
        }
    }
    if (flags) atomicOr(status, flags);
}

// ------------------------------------------------------------------ K1, row-aligned runs
// A tile is an even number of whole grid rows (one 1-D bulk copy: 16-byte aligned
// because rows come in pairs), split into runs of 17 modes that never cross a row end;
// the 136-byte stride between lanes' runs makes the 8-byte shared reads of data and
// window table conflict-free.  Rows shorter than a multiple of 17 leave a short last
// run, masked per mode.  Tiles of few rows (small N) hold several row pairs; long rows
// (N >= 1024) give a tile to a group of warps that share its stage ring.
constexpr int kRun = 17;

struct RowTiling {
    int R;            // runs per grid row: ceil(nz / 17)
    int trows;        // grid rows per tile (even)
    int wg;           // warps per tile group
    int tile_bytes;   // trows * nz * 8
    int stage_bytes;  // tile + read-past slack, 128-byte multiple
    int copies;       // copies of the CTA's bin totals: tile row r adds to copy r % copies
    int Rp;           // run-table row length (R rounded up to 4), 0 without the run table
    int tab_bytes;    // run-table rows at the start of a stage: trows * Rp * 4
};

// floats from one copy of the bin totals ({H[nrbins]}, {L[nrbins]}) to the next: 2 nrbins
// padded to 16 modulo 32, so that a bin sits in opposite half-banks of neighbouring copies
__host__ __device__ inline int totals_stride(int nrbins) { return 2 * nrbins + ((48 - (2 * nrbins) % 32) % 32); }

inline RowTiling make_row_tiling(int nz, bool table) {
    RowTiling t;
    t.R = (nz + kRun - 1) / kRun;
    int pairs = 32 / (2 * t.R);
    if (pairs < 1) pairs = 1;
    t.trows = 2 * pairs;
    t.wg = (t.trows * t.R + 31) / 32;
    t.tile_bytes = t.trows * nz * 8;
    t.Rp = table ? (t.R + 3) & ~3 : 0;
    t.tab_bytes = t.trows * t.Rp * 4;
    t.stage_bytes = (t.tab_bytes + t.tile_bytes + kRun * 8 + 127) & ~127;
    t.copies = 1;
    return t;
}

// stage rings (per group) | mbarriers | per-warp spill slots | float-pair bin totals
// (T.copies copies) | thresholds | {w1[z], multiplicity} for z < nz + 17 (zero past nz)
__host__ __device__ inline StreamPlan plan_bin_rows(int warps, int stages, int nrbins, int nz, bool exact,
                                                   const RowTiling& T) {
    StreamPlan p{};
    const int groups = warps / T.wg;
    size_t o = 0;
    p.stage_off = o;
    o += (size_t)groups * stages * T.stage_bytes;
    p.bar_off = o;
    o += sizeof(uint64_t) * (size_t)groups * stages;
    o = (o + 15) & ~size_t(15);
    p.spill_off = o;
    o += (size_t)warps * kRun * 32 * (exact ? 8 : 4);  // a slot per bin of a run: at most kRun
    p.hist_off = o;
    o += sizeof(float) * (size_t)totals_stride(nrbins) * T.copies;
    p.thr_off = o;
    o += sizeof(int) * (size_t)(nrbins + 1);
    o = (o + 15) & ~size_t(15);
    p.tab_off = o;
    o += sizeof(float2) * (size_t)(nz + kRun);
    p.total = o + 128;  // alignment slack
    return p;
}

__device__ __forceinline__ void named_sync(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
__device__ __forceinline__ bool named_and(int id, int nthreads, bool v) {
    uint32_t out;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, %2, %3, p;\n selp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(out)
        : "r"((uint32_t)v), "r"(id), "r"(nthreads)
        : "memory");
    return out != 0;
}

// One tile into a stage: its rows and, with the run table, the table rows of each of its
// row pairs (|kx|, min |ky|, then min |ky| + 1: one 16-byte aligned copy per pair), all on
// one mbarrier.
__device__ __forceinline__ void issue_row_tile(const GridArgs& g, const RowTiling& T, const unsigned* runtab,
                                               const unsigned char* gsrc, unsigned char* dst, uint64_t* bar,
                                               long long r0, long long nrows) {
    const long long nr = nrows - r0 < T.trows ? nrows - r0 : T.trows;
    const unsigned bytes = (unsigned)(nr * g.nz * 8);
    const unsigned tbytes = (unsigned)((nr / 2) * 2 * T.Rp * 4);
    ptx::mbar_expect_tx(bar, bytes + tbytes);
    ptx::bulk_g2s(dst + T.tab_bytes, gsrc + r0 * g.nz * 8, bytes, bar);
    for (int p = 0; 2 * p < nr && T.Rp; p++) {
        const uint32_t row0 = (uint32_t)(r0 + 2 * p);
        const uint32_t il = fdiv(row0, g.fd_N);
        const int j0 = (int)(row0 - il * (uint32_t)g.N);
        const int kx = kval(g.slab0 + (int)il, g.N), ky0 = kval(j0, g.N), ky1 = kval(j0 + 1, g.N);
        const int ax = kx < 0 ? -kx : kx, ay0 = ky0 < 0 ? -ky0 : ky0, ay1 = ky1 < 0 ? -ky1 : ky1;
        const int aymin = ay0 < ay1 ? ay0 : ay1;
        ptx::bulk_g2s(dst + (size_t)p * 2 * T.Rp * 4, runtab + ((size_t)ax * (g.half + 1) + aymin) * T.Rp,
                      (unsigned)(2 * T.Rp * 4), bar);
    }
}

template <int WARPS, int STAGES, bool EXACT, bool TAB>
__global__ void __launch_bounds__(WARPS * 32)
    k_bin_rows(GridArgs g, RowTiling T, const int* __restrict__ thresh, const float* __restrict__ w1g,
               const float* __restrict__ grid, double* bin_sum, double* F0sq, unsigned* status, long long ntiles,
               long long nrows, const unsigned* __restrict__ runtab) {
    typedef typename SpillOf<EXACT>::type Spill;
    extern __shared__ unsigned char sm_raw[];
    __shared__ int s_gap;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const StreamPlan P = plan_bin_rows(WARPS, STAGES, g.nrbins, g.nz, EXACT, T);
    unsigned char* base = sm_raw + ((128 - (ptx::smem_u32(sm_raw) & 127)) & 127);
    const int groups = WARPS / T.wg;
    const int grp = warp / T.wg, wig = warp - grp * T.wg;
    unsigned char* gstage = base + P.stage_off + (size_t)grp * STAGES * T.stage_bytes;
    uint64_t* gbar = reinterpret_cast<uint64_t*>(base + P.bar_off) + grp * STAGES;
    Spill* my_spill = reinterpret_cast<Spill*>(base + P.spill_off) + (size_t)warp * kRun * 32 + lane;
    float* s_H0 = reinterpret_cast<float*>(base + P.hist_off);
    int* s_thr = reinterpret_cast<int*>(base + P.thr_off);
    float2* s_wt = reinterpret_cast<float2*>(base + P.tab_off);
    const int hstride = totals_stride(g.nrbins);
    for (int i = tid; i < hstride * T.copies; i += blockDim.x) s_H0[i] = 0.f;
    for (int i = tid; i < g.nrbins; i += blockDim.x) s_thr[i] = thresh[i];
    for (int i = tid; i < g.nz + kRun; i += blockDim.x)
        s_wt[i] = i < g.nz ? make_float2(w1g[i], (i == 0 || i == g.half) ? 1.f : 2.f) : make_float2(0.f, 0.f);
    const bool leader = wig == 0 && lane == 0;
    // Modes past a row end (the short last run of a row) are read from the next row or
    // from the slack after the tile and weighted by the zero table entries past nz; the
    // slack starts zeroed, so nothing read there is ever uninitialised.
    {
        uint4* st4 = reinterpret_cast<uint4*>(base + P.stage_off);
        for (int i = tid; i < groups * STAGES * T.stage_bytes / 16; i += blockDim.x) st4[i] = make_uint4(0, 0, 0, 0);
        ptx::fence_async_smem();
    }
    if (tid == 0) {
        s_thr[g.nrbins] = 0x7fffffff;  // never crossed, also by the zero-weight modes past a row end
        s_gap = -1;
    }
    if (leader) {
        for (int s = 0; s < STAGES; s++) ptx::mbar_init(&gbar[s], 1);
        ptx::mbar_init_fence();
    }
    __syncthreads();
    const int k2max = 3 * g.half * g.half;
    for (int b = tid; b < g.nrbins - 1; b += blockDim.x) {
        const int t0 = s_thr[b], t1 = s_thr[b + 1];
        if (t1 <= k2max && (float)(t1 - t0) < 2.f * sqrtf((float)t0) + 3.f) atomicMax(&s_gap, b);
    }
    __syncthreads();
    const int ksafe = s_gap >= 0 ? s_thr[s_gap] : 1;

    // this lane's run within every tile
    const int run = wig * 32 + lane;
    const bool lane_ok = run < T.trows * T.R;
    const int row_t = lane_ok ? run / T.R : 0;
    const int z0 = (run - row_t * T.R) * kRun;
    const int len = g.nz - z0 < kRun ? g.nz - z0 : kRun;
    const unsigned lane_off = (unsigned)(row_t * g.nz + z0) * 8u;
    const float2* wz = s_wt + z0;
    const int gsz = T.wg * 32;
    // Lanes of one warp on different tile rows cover nearly the same bins at the same
    // time (neighbouring rows have nearly the same kx^2 + ky^2); separate copies of the
    // totals keep their shared atomics off each other's addresses.
    float* s_H = s_H0 + (size_t)(row_t % T.copies) * hstride;
    float* s_L = s_H + g.nrbins;

    const long long gg = (long long)blockIdx.x * groups + grp, TG = (long long)gridDim.x * groups;
    const long long my_n = gg < ntiles ? (ntiles - 1 - gg) / TG + 1 : 0;
    const unsigned char* gsrc = reinterpret_cast<const unsigned char*>(grid);
    if (leader)
        for (int s = 0; s < STAGES && s < my_n; s++)
            issue_row_tile(g, T, runtab, gsrc, gstage + s * T.stage_bytes, &gbar[s], (gg + s * TG) * T.trows, nrows);
    bool ok = true;
    long long k = 0;
    int s = 0;
    unsigned phase = 0;
    for (; k < my_n; k++) {
        const bool got = ptx::mbar_wait_bounded_n(&gbar[s], phase, k == 0 ? g.first_wait : (1 << 22));
        const bool all = T.wg == 1 ? __all_sync(kFull, got) : named_and(1 + grp, gsz, got);
        if (!all) {
            ok = false;
            break;
        }
        const unsigned char* tb = gstage + s * T.stage_bytes + T.tab_bytes;
        const long long pr64 = (gg + k * TG) * T.trows + row_t;
        const bool valid = lane_ok && pr64 < nrows;
        const int pr = (int)(valid ? pr64 : 0);
        const int il = (int)fdiv((uint32_t)pr, g.fd_N);
        const int jy = pr - il * g.N;
        const int kx = kval(g.slab0 + il, g.N), ky = kval(jy, g.N);
        const int kxy2 = kx * kx + ky * ky;
        int k2 = kxy2 + z0 * z0;
        const float iwxy = __fmul_rn(s_wt[kx < 0 ? -kx : kx].x, s_wt[ky < 0 ? -ky : ky].x);
        unsigned e = 1u;
        if (TAB && valid) {
            // the run's table entry: b_start << 17 | crossing bits | slow bit (the pair's
            // rows are |ky| ascending in the stage)
            const int kyp = kval(row_t & 1 ? jy - 1 : jy + 1, g.N);
            const int ay = ky < 0 ? -ky : ky, ayp = kyp < 0 ? -kyp : kyp;
            const unsigned* et = reinterpret_cast<const unsigned*>(gstage + s * T.stage_bytes) +
                                 (row_t >> 1) * 2 * T.Rp;
            e = et[(ay < ayp ? 0 : T.Rp) + (run - row_t * T.R)];
        }
        const bool fast = TAB ? valid && (e & 1u) == 0 : valid && k2 >= ksafe;
        if constexpr (TAB) {
            const int b = (int)(e >> 17);
            const int nsp = fast ? __popc(e & 0x1fffeu) : 0;  // the run's closed bins
            if (fast) {
                Spill* sp = my_spill;
                float h = 0.f, l = 0.f;
                const float2* vp = reinterpret_cast<const float2*>(tb + lane_off);
#pragma unroll
                for (int i = 0; i < kRun; i++) {
                    const float2 v = vp[i];  // past the row end: weight 0 (table entries past nz)
                    bin_step_bit<EXACT>(v.x, v.y, iwxy, wz[i], i > 0 && ((e >> i) & 1u), sp, h, l);
                }
            }
            // The next lane's run continues this one along the row: where it starts in
            // the bin this run ends in and has a later bin of its own, its first sum is
            // added to this run's last one here, and that bin goes to the totals once.
            const float2 first = fast ? my_spill[0] : make_float2(0.f, 0.f);
            const int info = fast ? (row_t << 8) | (nsp + 1) : 0;  // row, items; 0: no run
            const int nb_info = __shfl_down_sync(kFull, info, 1);
            const int nb_b = __shfl_down_sync(kFull, b, 1);
            const float nfx = __shfl_down_sync(kFull, first.x, 1), nfy = __shfl_down_sync(kFull, first.y, 1);
            const bool take = fast && lane < 31 && (nb_info >> 8) == row_t && (nb_info & 255) >= 2 &&
                              nb_b == b + nsp;
            const bool given = __shfl_up_sync(kFull, take ? 1 : 0, 1) != 0 && lane > 0;
            if (fast) {
                for (int q = given ? 1 : 0; q <= nsp; q++) {
                    Spill v = my_spill[32 * q];
                    if (q == nsp && take) pair_add(v.x, v.y, nfx, nfy);
                    add_pair(s_H, s_L, b + q, v.x, v.y);
                }
            }
        } else if (fast) {
            const int b = bin_of(k2, g.c1, s_thr, g.nrbins);
            const int* tq = s_thr + b + 1;
            int tnext = *tq;
            Spill* sp = my_spill;
            float h = 0.f, l = 0.f;
            int d = 2 * z0 + 1;
            const float2* vp = reinterpret_cast<const float2*>(tb + lane_off);
#pragma unroll
            for (int i = 0; i < kRun; i++) {
                const float2 v = vp[i];  // past the row end: weight 0 (table entries past nz)
                bin_step_slots<EXACT>(v.x, v.y, iwxy, wz[i], k2, d, tnext, tq, sp, h, l);
            }
            const int nsp = (int)(sp - my_spill) >> 5;
            for (int q = 0; q <= nsp; q++) {
                const Spill v = my_spill[32 * q];
                if constexpr (EXACT) add_pair(s_H, s_L, b + q, v.x, v.y);
                else add_pair(s_H, s_L, b + q, v, 0.f);
            }
        }
        // runs below ksafe (and the k = 0 mode): one run at a time, a mode per lane
        unsigned slow = __ballot_sync(kFull, valid && !fast);
        while (slow) {
            const int L = __ffs(slow) - 1;
            slow &= slow - 1;
            const int zL = __shfl_sync(kFull, z0, L), lenL = __shfl_sync(kFull, len, L);
            const int kxyL = __shfl_sync(kFull, kxy2, L);
            const float iwL = __shfl_sync(kFull, iwxy, L);
            const unsigned offL = __shfl_sync(kFull, lane_off, L);
            int key = -1;
            float phi = 0.f, plo = 0.f;
            const int zz = zL + lane;
            const int k2m = kxyL + zz * zz;
            if (lane < lenL && k2m != 0) {
                const float2 v = *reinterpret_cast<const float2*>(tb + offL + 8 * lane);
                mode_value<EXACT>(v.x, v.y, iwL, s_wt[zz], phi, plo);
                key = bin_of(k2m, g.c1, s_thr, g.nrbins);
            }
            bool tail;
            warp_seg_pair(key, phi, plo, tail);
            if (tail && key >= 0) add_pair(s_H, s_L, key, phi, plo);
        }
        if (T.wg == 1) __syncwarp();
        else named_sync(1 + grp, gsz);
        if (leader && k + STAGES < my_n)
            issue_row_tile(g, T, runtab, gsrc, gstage + s * T.stage_bytes, &gbar[s], (gg + (k + STAGES) * TG) * T.trows,
                           nrows);
        if (++s == STAGES) {
            s = 0;
            phase ^= 1;
        }
    }
    if (!ok && leader) {
        atomicOr(status, kStTimeout);
        for (long long kk = k; kk < my_n && kk < k + STAGES; kk++) {
            ptx::mbar_wait_bounded(&gbar[s], phase);
            if (++s == STAGES) {
                s = 0;
                phase ^= 1;
            }
        }
    }
    __syncthreads();
    if (blockIdx.x == 0 && tid == 0 && g.slab0 == 0 && g.nmodes > 0) {
        const float re = grid[0], im = grid[1];
        *F0sq = (double)__fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im));
    }
    for (int b = tid; b < g.nrbins; b += blockDim.x) {
        double v = 0.0;
        for (int c = 0; c < T.copies; c++)
            v += (double)s_H0[c * hstride + b] + (double)s_H0[c * hstride + g.nrbins + b];
        if (v != 0.0) atomicAdd(bin_sum + b, v);
    }
}

// ------------------------------------------------------------------ K1 over mirrored rows
// The rows ky and -ky of a plane (grid rows j and N - j) hold, at every z, modes of the
// same |k|, the same window factor and the same multiplicity: they fall in the same bins
// at the same z.  So a lane takes one 17-mode run of both rows at once.  The two |F|^2
// (each rounded in float as the reference forms it) are added exactly (Fast2Sum of the
// larger and the smaller), and the pair goes through the window product, the crossing and
// the compensated run sum once: the sum of the two double products the reference adds,
// to float-pair precision.  Crossings come from the run table, as in k_bin_rows; a run
// and its closed bins now cover 34 modes.
// A tile is P consecutive |ky| = q of one plane (P = 32 / runs per row): rows q0..q0+P-1
// (one copy) and their mirrors N-q (one copy, q descending).  q = 0 and q = N/2 are
// their own mirrors: their lanes pair the row with zeros (the stage's zeroed tail).  A
// copy starts at the 16-byte boundary at or below its first row and ends at the one at
// or above its last row end (a row is 8 (N/2+1) bytes, so odd rows start 8 bytes past a
// boundary).  Each warp owns a ring of two stages.
// zeroed bytes after a stage's rows: reads past the last row end, and the zero partner
// (17 modes) of a row that is its own mirror
constexpr int kMirrorTail = 144;
constexpr int kMirrorMaxWarps = 12;
// Spill slots per lane: a run closing more than kMirrorSlots - 1 bins (low k only) takes
// the warp-cooperative path; the shared memory saved holds one more warp per SM.
constexpr int kMirrorSlots = 9;

struct MirrorTiling {
    int R;            // 17-mode runs per row
    int P;            // |ky| values (row pairs) per tile
    int Rp;           // run-table row length
    int tpp;          // tiles per plane: ceil((N/2 + 1) / P)
    FastDiv fd_tpp;
    int tab_bytes;    // run-table rows of a tile, rounded to 16
    int blk;          // bytes of the region one copy lands in: P rows + 16, rounded to 16
    int stage_bytes;  // table rows | rows q | mirror rows | tail
    int copies;       // copies of the CTA's bin totals: pair p adds to copy p % copies
};

inline MirrorTiling make_mirror_tiling(int nz) {
    MirrorTiling t{};
    t.R = (nz + kRun - 1) / kRun;
    t.P = t.R <= 32 ? 32 / t.R : 0;
    if (t.P > nz) t.P = nz;
    t.Rp = (t.R + 3) & ~3;
    t.tpp = t.P > 0 ? (nz + t.P - 1) / t.P : 0;
    t.fd_tpp = make_fastdiv((uint32_t)(t.tpp > 0 ? t.tpp : 1));
    t.tab_bytes = (t.P * t.Rp * 4 + 15) & ~15;
    t.blk = (t.P * nz * 8 + 16 + 15) & ~15;
    t.stage_bytes = (t.tab_bytes + 2 * t.blk + kMirrorTail + 127) & ~127;
    t.copies = 1;
    return t;
}

// stage rings (two stages per warp) | mbarriers | per-warp spill slots | float-pair bin
// totals (T.copies copies) | thresholds | {w1[z], multiplicity} for z < nz + 17 (zero past nz)
__host__ __device__ inline StreamPlan plan_bin_mirror(int warps, int nrbins, int nz, bool exact,
                                                      const MirrorTiling& T) {
    StreamPlan p{};
    size_t o = 0;
    p.stage_off = o;
    o += (size_t)warps * 2 * T.stage_bytes;
    p.bar_off = o;
    o += sizeof(uint64_t) * (size_t)warps * 2;
    o = (o + 15) & ~size_t(15);
    p.spill_off = o;
    o += (size_t)warps * kMirrorSlots * 32 * (exact ? 8 : 4);
    p.hist_off = o;
    o += sizeof(float) * (size_t)totals_stride(nrbins) * T.copies;
    p.thr_off = o;
    o += sizeof(int) * (size_t)(nrbins + 1);
    o = (o + 15) & ~size_t(15);
    p.tab_off = o;
    o += sizeof(float2) * (size_t)(nz + kRun);
    p.total = o + 128;  // alignment slack
    return p;
}

__device__ __forceinline__ float spill_hi(float2 v) { return v.x; }
__device__ __forceinline__ float spill_lo(float2 v) { return v.y; }
__device__ __forceinline__ float spill_hi(float v) { return v; }
__device__ __forceinline__ float spill_lo(float) { return 0.f; }

// One mode pair of a fast run (z of row q and of its mirror): close the current bin if
// the run table marks a crossing, then add m (|F_a|^2 + |F_b|^2) inv^2 to the (new)
// current bin.  m (0, 1 or 2) multiplies exactly inside the fused multiply-adds.
template <bool EXACT>
__device__ __forceinline__ void mirror_step(float2 a, float2 b, float iwxy, float wz, float m, bool c,
                                            typename SpillOf<EXACT>::type*& sp, float& h, float& l) {
    const float Fa = __fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y));
    const float Fb = __fadd_rn(__fmul_rn(b.x, b.x), __fmul_rn(b.y, b.y));
    const float t = __fmul_rn(iwxy, wz);
    const float inv = __fmul_rn(t, t);
    const float fh = __fmul_rn(inv, inv);
    sp += c ? 32 : 0;
    const float h0 = c ? 0.f : h;
    if constexpr (EXACT) {
        const float mx = ptx::fmax_nan(Fa, Fb), mn = ptx::fmin_nan(Fa, Fb);
        const float sh = __fadd_rn(mx, mn);
        const float sl = __fsub_rn(mn, __fsub_rn(sh, mx));
        const float fl = fmaf(inv, inv, -fh);
        const float hi = __fmul_rn(sh, fh);
        const float lo = fmaf(sh, fl, fmaf(sl, fh, fmaf(sh, fh, -hi)));
        const float l0 = c ? 0.f : l;
        const float s = fmaf(hi, m, h0);
        const float bb = __fsub_rn(s, h0);
        const float e = __fadd_rn(__fsub_rn(h0, __fsub_rn(s, bb)), fmaf(hi, m, -bb));
        h = s;
        l = __fadd_rn(l0, fmaf(lo, m, e));
        *sp = make_float2(h, l);
    } else {
        h = fmaf(__fmul_rn(__fadd_rn(Fa, Fb), fh), m, h0);
        *sp = h;
    }
}

// Tile t into a stage: its run-table rows, rows q0.. and their mirrors, on one mbarrier.
__device__ __forceinline__ void issue_mirror_tile(const GridArgs& g, const MirrorTiling& T, const unsigned* runtab,
                                                  const unsigned char* gsrc, unsigned char* dst, uint64_t* bar,
                                                  long long t) {
    const int plane = (int)fdiv((uint32_t)t, T.fd_tpp);
    const int q0 = ((int)t - plane * T.tpp) * T.P;
    const int nA = min(T.P, g.nz - q0);
    const int qlo = max(q0, 1), qhi = min(q0 + nA - 1, g.half - 1);
    const size_t rb = (size_t)g.nz * 8;
    const size_t a0 = ((size_t)plane * g.N + q0) * rb;
    const size_t as = a0 & ~size_t(15), ae = (a0 + (size_t)nA * rb + 15) & ~size_t(15);
    size_t bs = 0, be = 0;
    if (qhi >= qlo) {
        const size_t b0 = ((size_t)plane * g.N + g.N - qhi) * rb;
        bs = b0 & ~size_t(15);
        be = (b0 + (size_t)(qhi - qlo + 1) * rb + 15) & ~size_t(15);
    }
    const int kx = kval(g.slab0 + plane, g.N), ax = kx < 0 ? -kx : kx;
    const unsigned tb = (unsigned)(nA * T.Rp * 4);
    ptx::fence_async_smem();
    ptx::mbar_expect_tx(bar, (unsigned)(ae - as + be - bs) + tb);
    ptx::bulk_g2s(dst, runtab + ((size_t)ax * (g.half + 1) + q0) * T.Rp, tb, bar);
    // grid rows are read once: their lines leave L2 first (the run table's stay)
    const uint64_t pol = ptx::policy_evict_first();
    ptx::bulk_g2s_hint(dst + T.tab_bytes, gsrc + as, (unsigned)(ae - as), bar, pol);
    if (be > bs) ptx::bulk_g2s_hint(dst + T.tab_bytes + T.blk, gsrc + bs, (unsigned)(be - bs), bar, pol);
}

template <bool EXACT>
__global__ void __launch_bounds__(kMirrorMaxWarps * 32)
    k_bin_mirror(GridArgs g, MirrorTiling T, const int* __restrict__ thresh, const float* __restrict__ w1g,
                 const float* __restrict__ grid, double* bin_sum, double* F0sq, unsigned* status, long long ntiles,
                 const unsigned* __restrict__ runtab) {
    typedef typename SpillOf<EXACT>::type Spill;
    extern __shared__ unsigned char sm_raw[];
    const int W = blockDim.x >> 5;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const StreamPlan Pl = plan_bin_mirror(W, g.nrbins, g.nz, EXACT, T);
    unsigned char* base = sm_raw + ((128 - (ptx::smem_u32(sm_raw) & 127)) & 127);
    unsigned char* wst = base + Pl.stage_off + (size_t)warp * 2 * T.stage_bytes;
    uint64_t* wbar = reinterpret_cast<uint64_t*>(base + Pl.bar_off) + warp * 2;
    Spill* my_spill = reinterpret_cast<Spill*>(base + Pl.spill_off) + (size_t)warp * kMirrorSlots * 32 + lane;
    float* s_H0 = reinterpret_cast<float*>(base + Pl.hist_off);
    int* s_thr = reinterpret_cast<int*>(base + Pl.thr_off);
    float2* s_wt = reinterpret_cast<float2*>(base + Pl.tab_off);
    const int hstride = totals_stride(g.nrbins);
    for (int i = tid; i < hstride * T.copies; i += blockDim.x) s_H0[i] = 0.f;
    for (int i = tid; i < g.nrbins; i += blockDim.x) s_thr[i] = thresh[i];
    for (int i = tid; i < g.nz + kRun; i += blockDim.x)
        s_wt[i] = i < g.nz ? make_float2(w1g[i], (i == 0 || i == g.half) ? 1.f : 2.f) : make_float2(0.f, 0.f);
    // the stages start zeroed: bytes a lane reads past a row end that no copy wrote are 0
    {
        uint4* st4 = reinterpret_cast<uint4*>(base + Pl.stage_off);
        for (int i = tid; i < W * 2 * T.stage_bytes / 16; i += blockDim.x) st4[i] = make_uint4(0, 0, 0, 0);
        ptx::fence_async_smem();
    }
    if (tid == 0) s_thr[g.nrbins] = 0x7fffffff;
    if (lane == 0) {
        ptx::mbar_init(&wbar[0], 1);
        ptx::mbar_init(&wbar[1], 1);
        ptx::mbar_init_fence();
    }
    __syncthreads();

    // this lane's pair and run within every tile; its window factors and multiplicities
    const int p = lane / T.R, r = lane - p * T.R;
    const bool lane_ok = p < T.P;
    const int z0 = r * kRun;
    float wz[kRun], mz[kRun];
#pragma unroll
    for (int i = 0; i < kRun; i++) {
        const float2 w = s_wt[z0 + i];
        wz[i] = w.x;
        mz[i] = w.y;
    }
    float* s_H = s_H0 + (size_t)(p % T.copies) * hstride;
    float* s_L = s_H + g.nrbins;
    const size_t rb = (size_t)g.nz * 8;

    const long long gw = (long long)blockIdx.x * W + warp, TW = (long long)gridDim.x * W;
    const long long my_n = gw < ntiles ? (ntiles - 1 - gw) / TW + 1 : 0;
    const unsigned char* gsrc = reinterpret_cast<const unsigned char*>(grid);
    if (lane == 0)
        for (int s = 0; s < 2 && s < my_n; s++)
            issue_mirror_tile(g, T, runtab, gsrc, wst + s * T.stage_bytes, &wbar[s], gw + s * TW);
    bool ok = true;
    long long k = 0;
    int s = 0;
    unsigned phase = 0;
    for (; k < my_n; k++) {
        const bool got = ptx::mbar_wait_bounded_n(&wbar[s], phase, k == 0 ? g.first_wait : (1 << 22));
        if (!__all_sync(kFull, got)) {
            ok = false;
            break;
        }
        const unsigned char* st = wst + s * T.stage_bytes;
        const uint32_t t = (uint32_t)(gw + k * TW);
        const int plane = (int)fdiv(t, T.fd_tpp);
        const int q0 = ((int)t - plane * T.tpp) * T.P;
        const int nA = min(T.P, g.nz - q0);
        const bool valid = lane_ok && p < nA;
        const int q = valid ? q0 + p : 0;
        const int kx = kval(g.slab0 + plane, g.N), ax = kx < 0 ? -kx : kx;
        const float iwxy = __fmul_rn(s_wt[ax].x, s_wt[q].x);
        const bool single = q == 0 || q == g.half;
        const int qhi = min(q0 + nA - 1, g.half - 1);
        const size_t a0 = ((size_t)plane * g.N + q0) * rb, b0 = ((size_t)plane * g.N + g.N - qhi) * rb;
        const unsigned offA = (unsigned)T.tab_bytes + (unsigned)(a0 & 15) + (unsigned)(p * g.nz + z0) * 8u;
        // a row that is its own mirror pairs with the stage's zeroed tail
        const unsigned offB = !valid ? offA
                              : single ? (unsigned)(T.tab_bytes + 2 * T.blk)
                                       : (unsigned)(T.tab_bytes + T.blk) + (unsigned)(b0 & 15) +
                                             (unsigned)((qhi - q) * g.nz + z0) * 8u;
        unsigned e = 1u;
        if (valid) e = reinterpret_cast<const unsigned*>(st)[p * T.Rp + r];
        const bool fast = valid && (e & 1u) == 0 && __popc(e & 0x1fffeu) < kMirrorSlots;
        const int b = (int)(e >> 17);
        const int nsp = fast ? __popc(e & 0x1fffeu) : 0;  // the run's closed bins
        if (fast) {
            Spill* sp = my_spill;
            float h = 0.f, l = 0.f;
            const float2* va = reinterpret_cast<const float2*>(st + offA);
            const float2* vb = reinterpret_cast<const float2*>(st + offB);
#pragma unroll
            for (int i = 0; i < kRun; i++)
                mirror_step<EXACT>(va[i], vb[i], iwxy, wz[i], mz[i], i > 0 && ((e >> i) & 1u), sp, h, l);
        }
        // The next lane's run continues this one: where it starts in the bin this run ends
        // in and has a later bin of its own, its first sum joins this run's last one here.
        float fx = 0.f, fy = 0.f;
        if (fast) {
            const Spill f0 = my_spill[0];
            fx = spill_hi(f0);
            fy = spill_lo(f0);
        }
        const int info = fast ? (p << 8) | (nsp + 1) : 0;  // pair, items; 0: no run
        const int nb_info = __shfl_down_sync(kFull, info, 1);
        const int nb_b = __shfl_down_sync(kFull, b, 1);
        const float nfx = __shfl_down_sync(kFull, fx, 1), nfy = __shfl_down_sync(kFull, fy, 1);
        const bool take = fast && lane < 31 && (nb_info >> 8) == p && (nb_info & 255) >= 2 && nb_b == b + nsp;
        const bool given = __shfl_up_sync(kFull, take ? 1 : 0, 1) != 0 && lane > 0;
        if (take) {
            const Spill v = my_spill[32 * nsp];
            float vh = spill_hi(v), vl = spill_lo(v);
            pair_add(vh, vl, nfx, nfy);
            if constexpr (EXACT) my_spill[32 * nsp] = make_float2(vh, vl);
            else my_spill[32 * nsp] = vh;
        }
        // slow runs (the k = 0 mode; a bin skipped between two modes; more closed bins than
        // spill slots): one run at a time, a mode of both rows per lane
        unsigned slow = __ballot_sync(kFull, valid && !fast);
        while (slow) {
            const int L = __ffs(slow) - 1;
            slow &= slow - 1;
            const int zL = __shfl_sync(kFull, z0, L);
            const int kxyL = __shfl_sync(kFull, ax * ax + q * q, L);
            const float iwL = __shfl_sync(kFull, iwxy, L);
            const unsigned oaL = __shfl_sync(kFull, offA, L), obL = __shfl_sync(kFull, offB, L);
            const bool sgL = __shfl_sync(kFull, single ? 1 : 0, L) != 0;
            int key = -1;
            float phi = 0.f, plo = 0.f;
            const int zz = zL + lane;
            const int k2m = kxyL + zz * zz;
            if (lane < kRun && zz < g.nz && k2m != 0) {
                const float2 va = *reinterpret_cast<const float2*>(st + oaL + 8 * lane);
                mode_value<EXACT>(va.x, va.y, iwL, s_wt[zz], phi, plo);
                if (!sgL) {
                    const float2 vb = *reinterpret_cast<const float2*>(st + obL + 8 * lane);
                    float qh, ql;
                    mode_value<EXACT>(vb.x, vb.y, iwL, s_wt[zz], qh, ql);
                    pair_add(phi, plo, qh, ql);
                }
                key = bin_of(k2m, g.c1, s_thr, g.nrbins);
            }
            bool tail;
            warp_seg_pair(key, phi, plo, tail);
            if (tail && key >= 0) add_pair(s_H, s_L, key, phi, plo);
        }
        __syncwarp();
        if (lane == 0 && k + 2 < my_n)
            issue_mirror_tile(g, T, runtab, gsrc, wst + s * T.stage_bytes, &wbar[s], gw + (k + 2) * TW);
        // the closed bins of the fast runs go to the totals from the spill slots, after the
        // stage is on its way again
        if (fast) {
            for (int qq = given ? 1 : 0; qq <= nsp; qq++) {
                const Spill v = my_spill[32 * qq];
                add_pair(s_H, s_L, b + qq, spill_hi(v), spill_lo(v));
            }
        }
        if (++s == 2) {
            s = 0;
            phase ^= 1;
        }
    }
    if (!ok && lane == 0) {
        atomicOr(status, kStTimeout);
        for (long long kk = k; kk < my_n && kk < k + 2; kk++) {
            ptx::mbar_wait_bounded(&wbar[s], phase);
            if (++s == 2) {
                s = 0;
                phase ^= 1;
            }
        }
    }
    __syncthreads();
    if (blockIdx.x == 0 && tid == 0 && g.slab0 == 0 && g.nmodes > 0) {
        const float re = grid[0], im = grid[1];
        *F0sq = (double)__fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im));
    }
    for (int bb = tid; bb < g.nrbins; bb += blockDim.x) {
        double v = 0.0;
        for (int c = 0; c < T.copies; c++)
            v += (double)s_H0[c * hstride + bb] + (double)s_H0[c * hstride + g.nrbins + bb];
        if (v != 0.0) atomicAdd(bin_sum + bb, v);
    }
}

int sm_count_s() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// Blocks of `kern` resident per SM with `threads` threads and `smem` bytes of dynamic
// shared memory on the current device, memoised: the occupancy query and the attribute
// call cost host microseconds, and at every step the device waits for the first launch.
// The kernel's dynamic shared-memory limit is raised once per device to the largest any
// of these passes asks for (226 KB: the 227 KB a block may use, less room for static shared
// memory); each launch still asks for its own size.  The memo
// is a fixed table (no host allocation: the allocation-free entry point runs through
// here): 64 (kernel, device, threads, smem) results, replaced round-robin, and the
// kernels whose shared-memory limit was raised.
constexpr int kMaxSmemPass = 226 * 1024;
struct OccEntry {
    const void* kern;
    int dev, threads, n;
    size_t smem;
};
template <typename K>
int resident_blocks(K kern, int threads, size_t smem) {
    static std::mutex m;
    static OccEntry memo[64];
    static int memo_n = 0, memo_next = 0;
    static std::pair<const void*, int> raised[64];
    static int raised_n = 0;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    const void* kp = reinterpret_cast<const void*>(kern);
    std::lock_guard<std::mutex> lock(m);
    for (int i = 0; i < memo_n; i++)
        if (memo[i].kern == kp && memo[i].dev == dev && memo[i].threads == threads && memo[i].smem == smem)
            return memo[i].n;
    bool done = false;
    for (int i = 0; i < raised_n && !done; i++) done = raised[i].first == kp && raised[i].second == dev;
    if (!done) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmemPass);
        if (raised_n < 64) raised[raised_n++] = std::make_pair(kp, dev);
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, threads, smem) != cudaSuccess) n = 0;
    memo[memo_next] = OccEntry{kp, dev, threads, n, smem};
    memo_next = (memo_next + 1) % 64;
    if (memo_n < 64) memo_n++;
    return n;
}

// The 2-D tensor map of a grid pointer, memoised per device (a handful of grids and slab
// chunks recur at every step) in a fixed table of 64, replaced round-robin.
struct TmapEntry {
    int dev, rows;
    const void* grid;
    long long nrows16;
    CUtensorMap map;
};
bool grid_tmap_cached(CUtensorMap* map, const void* grid, long long nrows16, int rows) {
    static std::mutex m;
    static TmapEntry memo[64];
    static int memo_n = 0, memo_next = 0;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    std::lock_guard<std::mutex> lock(m);
    for (int i = 0; i < memo_n; i++)
        if (memo[i].dev == dev && memo[i].grid == grid && memo[i].nrows16 == nrows16 && memo[i].rows == rows) {
            *map = memo[i].map;
            return true;
        }
    if (!make_grid_tmap(map, grid, nrows16, rows)) return false;
    memo[memo_next].dev = dev;
    memo[memo_next].rows = rows;
    memo[memo_next].grid = grid;
    memo[memo_next].nrows16 = nrows16;
    memo[memo_next].map = *map;
    memo_next = (memo_next + 1) % 64;
    if (memo_n < 64) memo_n++;
    return true;
}

// grid size and the per-iteration advance of a warp's tile start (TW tiles)
template <typename K>
bool stream_grid(K kern, int warps, size_t smem, long long ntiles, int nz, int& grid_n, int& adv_r, int& adv_z) {
    if (smem > (size_t)kMaxSmemPass) return false;
    const int per_sm = resident_blocks(kern, warps * 32, smem);
    if (per_sm < 1) return false;
    long long n = (long long)sm_count_s() * per_sm;
    const long long need = (ntiles + warps - 1) / warps;
    if (n > need) n = need > 0 ? need : 1;
    grid_n = (int)n;
    const long long adv = n * warps * kRowsPerWarp * 16;
    adv_r = (int)(adv / nz);
    adv_z = (int)(adv % nz);
    return true;
}

template <int WARPS, int STAGES, bool EXACT>
int run_bin_stream(const GridGeom& g, const GridArgs& a, const float* grid, double* bin_sum, double* F0sq,
                   unsigned* status, cudaStream_t st) {
    CUtensorMap map;
    if (!make_grid_tmap(&map, grid, a.nrows16, kRowsPerWarp)) return -1;
    const StreamPlan P = plan_bin_stream(WARPS, STAGES, g.nrbins, a.nz, EXACT);
    if (P.total > 220 * 1024) return -1;
    auto kern = k_bin_stream<WARPS, STAGES, EXACT>;
    const long long ntiles = (a.nrows16 + kRowsPerWarp - 1) / kRowsPerWarp;
    int grid_n = 1, adv_r = 0, adv_z = 0;
    if (!stream_grid(kern, WARPS, P.total, ntiles, a.nz, grid_n, adv_r, adv_z)) return -1;
    kern<<<grid_n, WARPS * 32, P.total, st>>>(map, a, g.thresh, g.w1, grid, bin_sum, F0sq, status, ntiles, adv_r,
                                              adv_z);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -2;
}

template <int WARPS, int STAGES, bool EXACT, bool TAB>
int run_bin_rows(const GridGeom& g, const GridArgs& a, const float* grid, double* bin_sum, double* F0sq,
                 unsigned* status, cudaStream_t st) {
    if ((reinterpret_cast<uintptr_t>(grid) & 15) != 0) return -1;
    RowTiling T = make_row_tiling(a.nz, TAB);
    if (WARPS % T.wg != 0) return -1;
    const long long nrows = (long long)g.nslab * g.N;
    if (nrows <= 0) return -1;
    auto kern = k_bin_rows<WARPS, STAGES, EXACT, TAB>;
    auto blocks_per_sm = [&](const RowTiling& t) -> int {
        const StreamPlan p = plan_bin_rows(WARPS, STAGES, g.nrbins, a.nz, EXACT, t);
        return p.total > (size_t)kMaxSmemPass ? 0 : resident_blocks(kern, WARPS * 32, p.total);
    };
    const int per_sm = blocks_per_sm(T);
    if (per_sm < 1) return -1;
    // a copy of the totals per tile row of a warp (at most 4), while that costs no
    // resident blocks
    for (int c = T.wg == 1 ? (T.trows < 4 ? T.trows : 4) : 1; c > 1; c /= 2) {
        RowTiling t2 = T;
        t2.copies = c;
        if (blocks_per_sm(t2) == per_sm) {
            T = t2;
            break;
        }
    }
    const StreamPlan P = plan_bin_rows(WARPS, STAGES, g.nrbins, a.nz, EXACT, T);
    const long long ntiles = (nrows + T.trows - 1) / T.trows;
    const int groups = WARPS / T.wg;
    long long n = (long long)sm_count_s() * per_sm;
    const long long need = (ntiles + groups - 1) / groups;
    if (n > need) n = need > 0 ? need : 1;
    kern<<<(int)n, WARPS * 32, P.total, st>>>(a, T, g.thresh, g.w1, grid, bin_sum, F0sq, status, ntiles, nrows,
                                              g.runtab);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -2;
}

// the exact variant reads bin crossings from the geometry's run table when it has one
template <int WARPS, int STAGES, bool EXACT>
int run_bin_rows_any(const GridGeom& g, const GridArgs& a, const float* grid, double* bin_sum, double* F0sq,
                     unsigned* status, cudaStream_t st) {
    if (EXACT && g.runtab && g.run_Rp == ((a.nz + kRun - 1) / kRun + 3) / 4 * 4)
        return run_bin_rows<WARPS, STAGES, EXACT, EXACT>(g, a, grid, bin_sum, F0sq, status, st);
    return run_bin_rows<WARPS, STAGES, EXACT, false>(g, a, grid, bin_sum, F0sq, status, st);
}

// The mirrored-row pass needs the geometry's run table and rows of at most 32 runs
// (N <= 1086).  Warps per CTA: the most resident warps per SM, then the largest CTA
// (KSPACE_GPU_MIRROR_WARPS fixes it).
template <bool EXACT>
int run_bin_mirror(const GridGeom& g, const GridArgs& a, const float* grid, double* bin_sum, double* F0sq,
                   unsigned* status, cudaStream_t st) {
    static const int force_w = [] {
        const char* e = getenv("KSPACE_GPU_MIRROR_WARPS");
        return e ? atoi(e) : 0;
    }();
    if ((reinterpret_cast<uintptr_t>(grid) & 15) != 0) return -1;
    // rows q = 0 and N/2 are their own mirrors only for even N (the geometry requires it)
    if (a.N & 1) return -1;
    MirrorTiling T = make_mirror_tiling(a.nz);
    if (T.P < 1 || !g.runtab || g.run_Rp != T.Rp || g.nslab <= 0) return -1;
    const long long ntiles = (long long)g.nslab * T.tpp;
    if (ntiles >= (1LL << 31)) return -1;
    auto kern = k_bin_mirror<EXACT>;
    int best_w = 0, best_occ = 0;
    for (int w = kMirrorMaxWarps; w >= 2; w--) {
        if (force_w > 0 && w != force_w) continue;
        const StreamPlan p = plan_bin_mirror(w, g.nrbins, a.nz, EXACT, T);
        if (p.total > (size_t)kMaxSmemPass) continue;
        const int occ = resident_blocks(kern, w * 32, p.total);
        if (occ * w > best_occ * best_w) {
            best_w = w;
            best_occ = occ;
        }
    }
    if (best_w == 0) return -1;
    // a copy of the totals per pair of a warp (at most 4), while that costs no resident blocks
    for (int c = T.P < 4 ? T.P : 4; c > 1; c /= 2) {
        MirrorTiling t2 = T;
        t2.copies = c;
        const StreamPlan p = plan_bin_mirror(best_w, g.nrbins, a.nz, EXACT, t2);
        if (p.total <= (size_t)kMaxSmemPass && resident_blocks(kern, best_w * 32, p.total) == best_occ) {
            T = t2;
            break;
        }
    }
    const StreamPlan P = plan_bin_mirror(best_w, g.nrbins, a.nz, EXACT, T);
    long long n = (long long)sm_count_s() * best_occ;
    const long long need = (ntiles + best_w - 1) / best_w;
    if (n > need) n = need > 0 ? need : 1;
    kern<<<(int)n, best_w * 32, P.total, st>>>(a, T, g.thresh, g.w1, grid, bin_sum, F0sq, status, ntiles, g.runtab);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -2;
}

template <int WARPS, int STAGES>
int run_corr_stream(const GridArgs& a, float* grid, CorrTable corr, unsigned* status, cudaStream_t st) {
    CUtensorMap map;
    if (!grid_tmap_cached(&map, grid, a.nrows16, kRowsPerWarp)) return -1;
    const StreamPlan P = plan_corr_stream(WARPS, STAGES, a.nk);
    if (P.total > 220 * 1024) return -1;
    auto kern = k_correct_stream<WARPS, STAGES>;
    const long long ntiles = (a.nrows16 + kRowsPerWarp - 1) / kRowsPerWarp;
    int grid_n = 1, adv_r = 0, adv_z = 0;
    if (!stream_grid(kern, WARPS, P.total, ntiles, a.nz, grid_n, adv_r, adv_z)) return -1;
    kern<<<grid_n, WARPS * 32, P.total, st>>>(map, a, corr, grid, status, ntiles, adv_r, adv_z);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -2;
}

// Run table of a geometry: for |kx|, |ky| in [0, N/2] and run r (modes z = 17r .. 17r+16
// of a grid row), entry = b_start << 17 | bit i (i = 1..16) set where mode i opens the next
// bin | bit 0 "slow".  Slow: the run holds the k = 0 mode (excluded, powerspectrum.c:65)
// or skips a bin between two consecutive modes (low k, a bin narrower than one k^2 step).
// Rows of Rp = R rounded up to 4 entries (16-byte rows); entries past R are slow.
__global__ void k_run_table(const int* __restrict__ thr, int nrbins, float c1, int half, int nz, int R, int Rp,
                            unsigned* __restrict__ tab) {
    const long long n = (long long)(half + 1) * (half + 1) * Rp;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e % Rp);
        const long long q = e / Rp;
        if (r >= R) {
            tab[e] = 1u;
            continue;
        }
        const int ay = (int)(q % (half + 1)), ax = (int)(q / (half + 1));
        const int kxy2 = ax * ax + ay * ay;
        unsigned mask = 0;
        int bprev = -1, bstart = 0;
        bool slow = false;
        for (int i = 0; i < kRun; i++) {
            const int z = kRun * r + i;
            if (z >= nz) break;
            const int k2 = kxy2 + z * z;
            if (k2 == 0) {
                slow = true;
                continue;
            }
            const int b = bin_of(k2, c1, thr, nrbins);
            if (bprev < 0) {
                bstart = b;
            } else if (b != bprev) {
                if (b - bprev > 1) slow = true;
                mask |= 1u << i;
            }
            bprev = b;
        }
        tab[e] = ((unsigned)bstart << 17) | mask | (slow ? 1u : 0u);
    }
}

}  // namespace

int build_run_table(GridGeom& g, cudaStream_t st) {
    g.runtab = nullptr;
    g.run_Rp = 0;
    const int half = g.N / 2, nz = half + 1;
    const int R = (nz + kRun - 1) / kRun, Rp = (R + 3) & ~3;
    const size_t n = (size_t)(half + 1) * (half + 1) * Rp;
    if (g.nrbins >= (1 << 15) || n * sizeof(unsigned) > (size_t(1) << 30)) return 1;
    unsigned* tab = nullptr;
    if (cudaMalloc(&tab, n * sizeof(unsigned)) != cudaSuccess) return -1;
    long long blocks = ((long long)n + 255) / 256;
    if (blocks > 8LL * sm_count_s()) blocks = 8LL * sm_count_s();
    k_run_table<<<(int)blocks, 256, 0, st>>>(g.thresh, g.nrbins, g.bin_c1, half, nz, R, Rp, tab);
    if (cudaPeekAtLastError() != cudaSuccess) {
        cudaFree(tab);
        return -1;
    }
    g.runtab = tab;
    g.run_Rp = Rp;
    return 0;
}

int launch_bin_stream(const GridGeom& g, const GridArgs& a, const float* grid, double* bin_sum, double* F0sq,
                      unsigned* status, int warps, int stages, bool exact, cudaStream_t st) {
    if (a.nrows16 <= 0 || a.N >= 32768) return -1;
#define KSP_BS(W, S)                                                                              \
    if (warps == W && stages == S)                                                                \
        return exact ? run_bin_stream<W, S, true>(g, a, grid, bin_sum, F0sq, status, st)          \
                     : run_bin_stream<W, S, false>(g, a, grid, bin_sum, F0sq, status, st);
    KSP_BS(4, 2) KSP_BS(4, 3) KSP_BS(4, 4) KSP_BS(8, 2) KSP_BS(8, 3) KSP_BS(8, 4)
#undef KSP_BS
    return exact ? run_bin_stream<8, 2, true>(g, a, grid, bin_sum, F0sq, status, st)
                 : run_bin_stream<8, 2, false>(g, a, grid, bin_sum, F0sq, status, st);
}

int launch_bin_rows(const GridGeom& g, const GridArgs& a, const float* grid, double* bin_sum, double* F0sq,
                    unsigned* status, int warps, int stages, bool exact, cudaStream_t st) {
    if (a.N >= 32768) return -1;
    // the mirrored-row pass where it applies (KSPACE_GPU_MIRROR=0: the row pass only)
    static const int mirror = [] {
        const char* e = getenv("KSPACE_GPU_MIRROR");
        return e ? atoi(e) : 1;
    }();
    if (mirror) {
        const int r = exact ? run_bin_mirror<true>(g, a, grid, bin_sum, F0sq, status, st)
                            : run_bin_mirror<false>(g, a, grid, bin_sum, F0sq, status, st);
        if (r != -1) return r;
    }
#define KSP_BR(W, S)                                                                            \
    if (warps == W && stages == S)                                                              \
        return exact ? run_bin_rows_any<W, S, true>(g, a, grid, bin_sum, F0sq, status, st)      \
                     : run_bin_rows_any<W, S, false>(g, a, grid, bin_sum, F0sq, status, st);
    KSP_BR(4, 2) KSP_BR(4, 3) KSP_BR(8, 2) KSP_BR(8, 3)
#undef KSP_BR
    return exact ? run_bin_rows_any<8, 2, true>(g, a, grid, bin_sum, F0sq, status, st)
                 : run_bin_rows_any<8, 2, false>(g, a, grid, bin_sum, F0sq, status, st);
}

int launch_correct_stream(const GridArgs& a, float* grid, CorrTable corr, unsigned* status, int warps, int stages,
                          cudaStream_t st) {
    if (a.nrows16 <= 0 || a.nk < 2 || a.N >= 32768) return -1;
#define KSP_CS(W, S) \
    if (warps == W && stages == S) return run_corr_stream<W, S>(a, grid, corr, status, st);
    KSP_CS(4, 2) KSP_CS(4, 3) KSP_CS(4, 4) KSP_CS(8, 2) KSP_CS(8, 3) KSP_CS(8, 4)
#undef KSP_CS
    return run_corr_stream<8, 2>(a, grid, corr, status, st);
}

}  // namespace ksp
