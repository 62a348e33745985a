// ksp_grid.cu -- the two streaming passes over the half-complex k-space grid.
//
// K1 (bin power, powerspectrum.c:56-89) and K3 (correction multiply,
// interface_gadget.c:163-188) stream the slab [nslab][N][N/2+1] complex64 once each.
// The slab is viewed as rows of 16 modes (128 bytes); a persistent CTA pulls tiles of
// ROWS such rows into a ring of shared-memory stages with 2-D TMA loads (128-byte
// swizzle, so that each thread reading "its" row is bank-conflict free) and, for K3,
// writes the corrected tile back with TMA stores.  Every thread handles the 16
// consecutive modes of one row: the mode coordinates advance incrementally, the log
// bin comes from an approximate log2 settled exactly against integer k^2 thresholds
// (so counts match the reference's floor(bpu log|k|) bit for bit), and K1 sums runs of
// equal bins in registers (Kahan, FP32) before one shared-memory FP64 add per run.
// Mode counts and sum|k| per bin depend only on the geometry and are computed once.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include "ksp_internal.h"
#include "ksp_gridutil.cuh"
#include "ksp_ptx.cuh"

namespace ksp {

// ------------------------------------------------------------------ shared-memory layout
struct SmemPlan {
    size_t stages_off, hist_off, thr_off, tab_off, bar_off, total;
};
__host__ __device__ inline SmemPlan plan_smem(int rows, int stages, int nrbins, int ntab_floats, int hist_copies = 1) {
    SmemPlan p;
    p.stages_off = 0;  // aligned to 1024 at run time (slack included)
    size_t o = (size_t)stages * rows * 128 + 1024;
    p.hist_off = o;
    o += sizeof(double) * (size_t)nrbins * hist_copies;
    p.thr_off = o;
    o += sizeof(int) * (size_t)(nrbins + 1);
    o = (o + 15) & ~size_t(15);
    p.tab_off = o;
    o += sizeof(float) * (size_t)ntab_floats;
    o = (o + 15) & ~size_t(15);
    p.bar_off = o;
    o += sizeof(uint64_t) * (size_t)stages;
    p.total = o;
    return p;
}

// ------------------------------------------------------------------ K1 (TMA)
// Persistent CTAs stream 128-byte rows (16 modes) through a STAGES-deep TMA ring;
// 16/MPT threads per row, MPT consecutive modes each.  A thread sums its modes into two
// adjacent bins as float pairs (BinPairAcc2) and hands them, at the end of its modes, to
// its warp's own float-pair bin totals by FP32 atomics (no other warp writes them); each
// CTA adds its warps' totals to the global FP64 sums once.
template <int ROWS, int STAGES, int MPT>
__global__ void __launch_bounds__(ROWS * (16 / MPT), 1024 / (ROWS * (16 / MPT)))
k_bin_power_tma(const __grid_constant__ CUtensorMap tmap, GridArgs g, const int* __restrict__ thresh,
                const float* __restrict__ w1g, const float* __restrict__ grid, double* bin_sum, double* F0sq,
                unsigned* status, int ntiles) {
    constexpr int TPR = 16 / MPT, NT = ROWS * TPR, NW = NT / 32;
    extern __shared__ unsigned char sm_raw[];
    __shared__ int s_abort;
    __shared__ long long s_rowbase;
    __shared__ int s_zbase;
    const SmemPlan P = plan_smem(ROWS, STAGES, g.nrbins, 2 * g.nz, NW);
    const uint32_t base_u = ptx::smem_u32(sm_raw);
    unsigned char* stage0 = sm_raw + ((1024 - (base_u & 1023)) & 1023);
    float* s_hist = reinterpret_cast<float*>(sm_raw + P.hist_off);  // per warp: nrbins high, nrbins low parts
    int* s_thr = reinterpret_cast<int*>(sm_raw + P.thr_off);
    float* s_w1 = reinterpret_cast<float*>(sm_raw + P.tab_off);
    float* s_wt = s_w1 + g.nz;  // k_z weights
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm_raw + P.bar_off);
    const int tid = threadIdx.x;
    const int r = tid / TPR, q = tid - r * TPR;
    float* s_H = s_hist + (size_t)(tid >> 5) * 2 * g.nrbins;  // this warp's totals
    float* s_L = s_H + g.nrbins;
    for (int i = tid; i < 2 * NW * g.nrbins; i += NT) s_hist[i] = 0.f;
    for (int i = tid; i <= g.nrbins; i += NT) s_thr[i] = thresh[i];
    for (int i = tid; i < g.nz; i += NT) {
        s_w1[i] = w1g[i];
        s_wt[i] = (i == 0 || i == g.half) ? 1.f : 2.f;
    }
    if (tid == 0) {
        s_abort = 0;
        for (int st = 0; st < STAGES; st++) ptx::mbar_init(&bars[st], 1);
        ptx::mbar_init_fence();
    }
    __syncthreads();
    const int my_n = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    if (tid == 0) {
        for (int k = 0; k < STAGES && k < my_n; k++) {
            const int tile = blockIdx.x + k * gridDim.x;
            ptx::mbar_expect_tx(&bars[k], ROWS * 128);
            ptx::tma_load_2d(stage0 + (size_t)k * ROWS * 128, &tmap, &bars[k], 0, tile * ROWS);
        }
    }
    BinPairAcc2 acc;
    int k = 0;
    for (; k < my_n; k++) {
        const int st = k % STAGES;
        const int tile = blockIdx.x + k * gridDim.x;
        if (tid == 0) {
            if (!ptx::mbar_wait_bounded(&bars[st], (k / STAGES) & 1)) s_abort = 1;
            const long long m = (long long)tile * ROWS * 16;
            s_rowbase = m / g.nz;
            s_zbase = (int)(m - s_rowbase * g.nz);
        }
        __syncthreads();
        if (s_abort) break;
        const long long row = (long long)tile * ROWS + r;
        if (row < g.nrows16) {
            const unsigned char* rp = stage0 + (size_t)st * ROWS * 128 + (size_t)r * 128;
            ModeCursor c;
            c.init(g, s_w1, s_rowbase, s_zbase, r * 16 + q * MPT);
            if (c.z + MPT <= g.nz && c.kxy2 != 0) {
                // the common case: all MPT modes in one column, none of them k = 0; k^2 and
                // z follow from the first mode
                const int z0 = c.z;
                int k2 = c.kxy2 + z0 * z0;
#pragma unroll
                for (int u = 0; u < MPT / 2; u++) {
                    const float4 v = *reinterpret_cast<const float4*>(rp + (((q * (MPT / 2) + u) ^ (r & 7)) << 4));
                    c.z = z0 + 2 * u;
                    acc.add(k2, mode_power2w(v.x, v.y, c, s_w1, s_wt), g, s_thr, s_H, s_L);
                    k2 += 2 * c.z + 1;
                    c.z++;
                    acc.add(k2, mode_power2w(v.z, v.w, c, s_w1, s_wt), g, s_thr, s_H, s_L);
                    k2 += 2 * c.z + 1;
                }
            } else {
#pragma unroll
                for (int u = q * (MPT / 2); u < (q + 1) * (MPT / 2); u++) {
                    const float4 v = *reinterpret_cast<const float4*>(rp + ((u ^ (r & 7)) << 4));
                    {
                        const int k2 = c.kxy2 + c.z * c.z;
                        if (k2 != 0) acc.add(k2, mode_power2w(v.x, v.y, c, s_w1, s_wt), g, s_thr, s_H, s_L);
                        c.next(g, s_w1);
                    }
                    {
                        const int k2 = c.kxy2 + c.z * c.z;
                        if (k2 != 0) acc.add(k2, mode_power2w(v.z, v.w, c, s_w1, s_wt), g, s_thr, s_H, s_L);
                        c.next(g, s_w1);
                    }
                }
            }
            acc.flush(s_H, s_L);
        }
        __syncthreads();
        if (tid == 0 && k + STAGES < my_n) {
            const int nt = blockIdx.x + (k + STAGES) * gridDim.x;
            ptx::mbar_expect_tx(&bars[st], ROWS * 128);
            ptx::tma_load_2d(stage0 + (size_t)st * ROWS * 128, &tmap, &bars[st], 0, nt * ROWS);
        }
    }
    if (s_abort) {
        // wait (bounded) for the loads still in flight, then leave
        if (tid == 0) {
            atomicOr(status, kStTimeout);
            for (int kk = k; kk < my_n && kk < k + STAGES; kk++)
                ptx::mbar_wait_bounded(&bars[kk % STAGES], (kk / STAGES) & 1);
        }
        return;
    }
    // the modes after the last full 16-mode row (fewer than 16), by CTA 0
    if (blockIdx.x == 0 && tid == 0) {
        for (long long m = g.nrows16 * 16; m < g.nmodes; m++) {
            const long long rr = m / g.nz;
            ModeCursor c;
            c.z = (int)(m - rr * g.nz);
            c.il = (int)(rr / g.N);
            c.j = (int)(rr - (long long)c.il * g.N);
            c.set_row(g, s_w1);
            const int k2 = c.kxy2 + c.z * c.z;
            if (k2 != 0) {
                const ModeP p = mode_power2(grid[2 * m], grid[2 * m + 1], c, s_w1, g.half);
                pair_atomic_add(s_H, s_L, bin_of(k2, g.c1, s_thr, g.nrbins), p.hi, p.lo);
            }
        }
    }
    if (blockIdx.x == 0 && tid == 0 && g.slab0 == 0 && g.nmodes > 0) {
        const float re = grid[0], im = grid[1];
        *F0sq = (double)__fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im));
    }
    __syncthreads();
    for (int i = tid; i < g.nrbins; i += NT) {
        double v = 0.0;
        for (int w = 0; w < NW; w++)
            v += (double)s_hist[(size_t)w * 2 * g.nrbins + i] + (double)s_hist[(size_t)w * 2 * g.nrbins + g.nrbins + i];
        if (v != 0.0) atomicAdd(bin_sum + i, v);
    }
}

// ------------------------------------------------------------------ K1 (plain loads)
__global__ void k_bin_power_plain(GridArgs g, const int* __restrict__ thresh, const float* __restrict__ w1g,
                                  const float* __restrict__ grid, double* bin_sum, double* F0sq) {
    extern __shared__ unsigned char sm_raw[];
    double* s_hist = reinterpret_cast<double*>(sm_raw);
    int* s_thr = reinterpret_cast<int*>(s_hist + g.nrbins);
    float* s_w1 = reinterpret_cast<float*>(s_thr + g.nrbins + 1);
    for (int i = threadIdx.x; i < g.nrbins; i += blockDim.x) s_hist[i] = 0.0;
    for (int i = threadIdx.x; i <= g.nrbins; i += blockDim.x) s_thr[i] = thresh[i];
    for (int i = threadIdx.x; i < g.nz; i += blockDim.x) s_w1[i] = w1g[i];
    __syncthreads();
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < g.nmodes;
         m += (long long)gridDim.x * blockDim.x) {
        const long long r = m / g.nz;
        ModeCursor c;
        c.z = (int)(m - r * g.nz);
        c.il = (int)(r / g.N);
        c.j = (int)(r - (long long)c.il * g.N);
        c.set_row(g, s_w1);
        const int k2 = c.kxy2 + c.z * c.z;
        if (k2 == 0) continue;
        const float2 v = reinterpret_cast<const float2*>(grid)[m];
        atomicAdd(&s_hist[bin_of(k2, g.c1, s_thr, g.nrbins)], mode_power_d(v.x, v.y, c, s_w1, g.half));
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && g.slab0 == 0 && g.nmodes > 0) {
        const float re = grid[0], im = grid[1];
        *F0sq = (double)__fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < g.nrbins; i += blockDim.x)
        if (s_hist[i] != 0.0) atomicAdd(bin_sum + i, s_hist[i]);
}

// ------------------------------------------------------------------ K3 (TMA in/out)
// The same tile engine; each thread multiplies its MPT modes in shared memory by
// 1 + norm interp(log k), following the table segment of its modes (SegTrack); the tile
// goes back by a TMA store.
template <int ROWS, int STAGES, int MPT>
__global__ void __launch_bounds__(ROWS * (16 / MPT), 1024 / (ROWS * (16 / MPT)))
k_correct_tma(const __grid_constant__ CUtensorMap tmap, GridArgs g, const int* __restrict__ thresh,
              const int* __restrict__ cmapg, CorrTable corr, float* grid, unsigned* status, int ntiles) {
    constexpr int TPR = 16 / MPT, NT = ROWS * TPR;
    extern __shared__ unsigned char sm_raw[];
    // an error of the step so far: the grid stays as it is (as in k_correct_stream)
    if (*reinterpret_cast<volatile unsigned*>(status) & kStAbort) return;
    __shared__ int s_abort;
    __shared__ long long s_rowbase;
    __shared__ int s_zbase;
    const SmemPlan P = plan_smem(ROWS, STAGES, g.nrbins, 3 * g.nk + g.nrbins);
    const uint32_t base_u = ptx::smem_u32(sm_raw);
    unsigned char* stage0 = sm_raw + ((1024 - (base_u & 1023)) & 1023);
    int* s_thr = reinterpret_cast<int*>(sm_raw + P.thr_off);
    float* s_tab = reinterpret_cast<float*>(sm_raw + P.tab_off);
    int* s_cmap = reinterpret_cast<int*>(s_tab + 3 * g.nk);
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm_raw + P.bar_off);
    const int tid = threadIdx.x;
    const int r = tid / TPR, q = tid - r * TPR;
    for (int i = tid; i <= g.nrbins; i += NT) s_thr[i] = thresh[i];
    for (int i = tid; i < g.nrbins; i += NT) s_cmap[i] = cmapg[i];
    for (int i = tid; i < g.nk; i += NT) {
        s_tab[i] = corr.xf[i];
        s_tab[g.nk + i] = corr.rn[i];
        s_tab[2 * g.nk + i] = corr.sn[i];
    }
    if (tid == 0) {
        s_abort = 0;
        for (int st = 0; st < STAGES; st++) ptx::mbar_init(&bars[st], 1);
        ptx::mbar_init_fence();
    }
    __syncthreads();
    CorrSmem T{s_thr, s_cmap, s_tab, s_tab + g.nk, s_tab + 2 * g.nk};
    const int my_n = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    if (tid == 0) {
        for (int k = 0; k < STAGES - 1 && k < my_n; k++) {
            const int tile = blockIdx.x + k * gridDim.x;
            ptx::mbar_expect_tx(&bars[k], ROWS * 128);
            ptx::tma_load_2d(stage0 + (size_t)k * ROWS * 128, &tmap, &bars[k], 0, tile * ROWS);
        }
    }
    unsigned flags = 0;
    SegTrack seg;
    int k = 0;
    for (; k < my_n; k++) {
        const int st = k % STAGES;
        const int tile = blockIdx.x + k * gridDim.x;
        if (tid == 0) {
            if (!ptx::mbar_wait_bounded(&bars[st], (k / STAGES) & 1)) s_abort = 1;
            const long long m = (long long)tile * ROWS * 16;
            s_rowbase = m / g.nz;
            s_zbase = (int)(m - s_rowbase * g.nz);
        }
        __syncthreads();
        if (s_abort) break;
        const long long row = (long long)tile * ROWS + r;
        if (row < g.nrows16) {
            unsigned char* rp = stage0 + (size_t)st * ROWS * 128 + (size_t)r * 128;
            KCursor c;
            c.init(g, s_rowbase, s_zbase, r * 16 + q * MPT);
#pragma unroll
            for (int u = q * (MPT / 2); u < (q + 1) * (MPT / 2); u++) {
                float4* vp = reinterpret_cast<float4*>(rp + ((u ^ (r & 7)) << 4));
                float4 v = *vp;
                {
                    const int k2 = c.kxy2 + c.z * c.z;
                    if (k2 != 0) {
                        const float d = seg.delta(k2, g.lnscale, T, g.nk, flags);
                        v.x = fmaf(v.x, d, v.x);
                        v.y = fmaf(v.y, d, v.y);
                    }
                    c.next(g);
                }
                {
                    const int k2 = c.kxy2 + c.z * c.z;
                    if (k2 != 0) {
                        const float d = seg.delta(k2, g.lnscale, T, g.nk, flags);
                        v.z = fmaf(v.z, d, v.z);
                        v.w = fmaf(v.w, d, v.w);
                    }
                    c.next(g);
                }
                *vp = v;
            }
        }
        ptx::fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            ptx::tma_store_2d(&tmap, stage0 + (size_t)st * ROWS * 128, 0, tile * ROWS);
            ptx::bulk_commit();
            if (k + STAGES - 1 < my_n) {
                const int s2 = (k + STAGES - 1) % STAGES;
                const int nt = blockIdx.x + (k + STAGES - 1) * gridDim.x;
                ptx::bulk_wait_read_le1();  // the store issued from stage s2 one iteration ago has been read
                ptx::mbar_expect_tx(&bars[s2], ROWS * 128);
                ptx::tma_load_2d(stage0 + (size_t)s2 * ROWS * 128, &tmap, &bars[s2], 0, nt * ROWS);
            }
        }
    }
    if (tid == 0) {
        if (s_abort) {
            atomicOr(status, kStTimeout);
            for (int kk = k; kk < my_n && kk < k + STAGES - 1; kk++)
                ptx::mbar_wait_bounded(&bars[kk % STAGES], (kk / STAGES) & 1);
        }
        ptx::bulk_wait_all();
    }
    if (s_abort) return;
    // trailing modes (fewer than 16) by CTA 0
    if (blockIdx.x == 0 && tid == 0) {
        for (long long m = g.nrows16 * 16; m < g.nmodes; m++) {
            const long long rr = m / g.nz;
            const int z = (int)(m - rr * g.nz);
            const int il = (int)(rr / g.N), j = (int)(rr - (long long)il * g.N);
            const int kx = kval(g.slab0 + il, g.N), ky = kval(j, g.N);
            const int k2 = kx * kx + ky * ky + z * z;
            if (k2 != 0) {
                const float d = seg.delta(k2, g.lnscale, T, g.nk, flags);
                grid[2 * m] = fmaf(grid[2 * m], d, grid[2 * m]);
                grid[2 * m + 1] = fmaf(grid[2 * m + 1], d, grid[2 * m + 1]);
            }
        }
    }
    if (flags) atomicOr(status, flags);
}

// ------------------------------------------------------------------ K3 (plain loads)
__global__ void k_correct_plain(GridArgs g, const int* __restrict__ thresh, const int* __restrict__ cmapg,
                                CorrTable corr, float* grid, unsigned* status) {
    extern __shared__ unsigned char sm_raw[];
    // an error of the step so far: the grid stays as it is (as in k_correct_stream)
    if (*reinterpret_cast<volatile unsigned*>(status) & kStAbort) return;
    int* s_thr = reinterpret_cast<int*>(sm_raw);
    int* s_cmap = s_thr + g.nrbins + 1;
    float* s_tab = reinterpret_cast<float*>(s_cmap + g.nrbins);
    for (int i = threadIdx.x; i <= g.nrbins; i += blockDim.x) s_thr[i] = thresh[i];
    for (int i = threadIdx.x; i < g.nrbins; i += blockDim.x) s_cmap[i] = cmapg[i];
    for (int i = threadIdx.x; i < g.nk; i += blockDim.x) {
        s_tab[i] = corr.xf[i];
        s_tab[g.nk + i] = corr.rn[i];
        s_tab[2 * g.nk + i] = corr.sn[i];
    }
    __syncthreads();
    CorrSmem T{s_thr, s_cmap, s_tab, s_tab + g.nk, s_tab + 2 * g.nk};
    unsigned flags = 0;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < g.nmodes;
         m += (long long)gridDim.x * blockDim.x) {
        const long long r = m / g.nz;
        const int z = (int)(m - r * g.nz);
        const int il = (int)(r / g.N), j = (int)(r - (long long)il * g.N);
        const int kx = kval(g.slab0 + il, g.N), ky = kval(j, g.N);
        const int k2 = kx * kx + ky * ky + z * z;
        if (k2 == 0) continue;
        const float d = corr_delta(k2, g, T, flags);
        float2 v = reinterpret_cast<float2*>(grid)[m];
        v.x = fmaf(v.x, d, v.x);
        v.y = fmaf(v.y, d, v.y);
        reinterpret_cast<float2*>(grid)[m] = v;
    }
    if (flags) atomicOr(status, flags);
}

// ------------------------------------------------------------------ geometry
// weighted mode count per integer k^2 over the slab range (weights as powerspectrum.c:56-89)
__global__ void k_k2_hist(int N, int slab0, int nslab, unsigned long long* hist) {
    const long long rows = (long long)nslab * N;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows;
         r += (long long)gridDim.x * blockDim.x) {
        const int il = (int)(r / N), j = (int)(r - (long long)il * N);
        const int kx = kval(slab0 + il, N), ky = kval(j, N);
        const int kxy2 = kx * kx + ky * ky;
        for (int z = 0; z <= N / 2; z++) {
            const int k2 = kxy2 + z * z;
            if (k2 == 0) continue;
            atomicAdd(hist + k2, (unsigned long long)((z == 0 || z == N / 2) ? 1 : 2));
        }
    }
}
void launch_k2_histogram(int N, int slab0, int nslab, unsigned long long* hist, cudaStream_t st) {
    const long long rows = (long long)nslab * N;
    const int blocks = (int)((rows + 255) / 256 < 4096 ? (rows + 255) / 256 : 4096);
    k_k2_hist<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(N, slab0, nslab, hist);
}

// powerspectrum.c:98-115 + interface_gadget.c:96-100
__global__ void k_finalize_power(const double* bin_sum, const double* F0sq, const long long* count,
                                 const double* ksum, const int* compact_bins, int nk, double BoxSize,
                                 double* power_out, double* keff_out, double* dcdm_out, double* keffphys_out,
                                 double scale, double kfac) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nk) return;
    const FinalizeArgs f{bin_sum, F0sq,   count,   ksum,         compact_bins, BoxSize, power_out,
                         keff_out, dcdm_out, keffphys_out, 1, scale, kfac};
    finalize_bin(f, c);
}
void launch_finalize_power(const double* bin_sum, const double* F0sq, const long long* count, const double* ksum,
                           const int* compact_bins, int nk, double BoxSize, double* power_out, double* keff_out,
                           double* dcdm_out, double* keffphys_out, cudaStream_t st) {
    // a warp per block: the FP64 pow, sqrt and divisions of the bins spread over SMs
    k_finalize_power<<<(nk + 31) / 32, 32, 0, st>>>(bin_sum, F0sq, count, ksum, compact_bins, nk, BoxSize, power_out,
                                                    keff_out, dcdm_out, keffphys_out, pow(BoxSize, -3.0),
                                                    2 * 3.14159265358979323846 / BoxSize);
}

// ------------------------------------------------------------------ host launchers
typedef CUresult (*PFN_encodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                     const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                     CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static PFN_encodeTiled get_encode() {
    static PFN_encodeTiled fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_encodeTiled>(p);
    }
    return fn;
}

bool make_grid_tmap(CUtensorMap* map, const void* grid, long long nrows16, int rows) {
    PFN_encodeTiled enc = get_encode();
    if (!enc || nrows16 <= 0) return false;
    if ((reinterpret_cast<uintptr_t>(grid) & 15) != 0) return false;
    cuuint64_t gdim[2] = {32, (cuuint64_t)nrows16};
    cuuint64_t gstride[1] = {128};
    cuuint32_t box[2] = {32, (cuuint32_t)rows};
    cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(grid), gdim, gstride, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

template <int ROWS, int STAGES, int MPT>
static int run_bin_tma(const GridGeom& g, const GridArgs& a, const float* grid, double* bin_sum, double* F0sq,
                       unsigned* status, cudaStream_t st) {
    constexpr int NT = ROWS * (16 / MPT);
    CUtensorMap map;
    if (!make_grid_tmap(&map, grid, a.nrows16, ROWS)) return -1;
    const SmemPlan P = plan_smem(ROWS, STAGES, g.nrbins, 2 * a.nz, NT / 32);
    if (P.total > 220 * 1024) return -1;
    auto kern = k_bin_power_tma<ROWS, STAGES, MPT>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P.total);
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, P.total);
    if (per_sm < 1) per_sm = 1;
    const int ntiles = (int)((a.nrows16 + ROWS - 1) / ROWS);
    int grid_n = sm_count() * per_sm;
    if (grid_n > ntiles) grid_n = ntiles > 0 ? ntiles : 1;
    kern<<<grid_n, NT, P.total, st>>>(map, a, g.thresh, g.w1, grid, bin_sum, F0sq, status, ntiles);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -2;
}

// tile shape: rows per CTA, pipeline stages, modes per thread (16: a thread per row;
// 8: two threads per row)
static int bin_variant(const GridGeom& g, const GridArgs& a, const float* grid, double* bin_sum, double* F0sq,
                       unsigned* status, int rows, int stages, int mpt, cudaStream_t st) {
#define KSP_BIN_CASE(R, S, M) \
    if (rows == R && stages == S && mpt == M) return run_bin_tma<R, S, M>(g, a, grid, bin_sum, F0sq, status, st);
    KSP_BIN_CASE(128, 2, 16) KSP_BIN_CASE(128, 3, 16) KSP_BIN_CASE(128, 4, 16) KSP_BIN_CASE(256, 2, 16)
    KSP_BIN_CASE(256, 3, 16) KSP_BIN_CASE(128, 2, 8) KSP_BIN_CASE(128, 3, 8) KSP_BIN_CASE(128, 4, 8)
    KSP_BIN_CASE(256, 2, 8) KSP_BIN_CASE(256, 3, 8)
#undef KSP_BIN_CASE
    return run_bin_tma<256, 2, 16>(g, a, grid, bin_sum, F0sq, status, st);
}

int launch_bin_power(const GridGeom& g, const float* grid, double* bin_sum, double* F0sq, unsigned* status, int tma,
                     int rows_per_cta, int stages, cudaStream_t st) {
    const GridArgs a = make_grid_args(g, 0, 0.f);
    if (tma >= 5) {
        const int r = launch_bin_rows(g, a, grid, bin_sum, F0sq, status, rows_per_cta / 32, stages, tma == 5, st);
        if (r == 0) return 0;
        if (r == -2) return -2;
    } else if (tma >= 3) {
        const int r = launch_bin_stream(g, a, grid, bin_sum, F0sq, status, rows_per_cta / 32, stages, tma == 3, st);
        if (r == 0) return 0;
        if (r == -2) return -2;
    } else if (tma && a.nrows16 > 0) {
        const int r = bin_variant(g, a, grid, bin_sum, F0sq, status, rows_per_cta, stages, tma == 2 ? 8 : 16, st);
        if (r == 0) return 0;
        if (r == -2) return -2;
    }
    const size_t smem = sizeof(double) * g.nrbins + sizeof(int) * (g.nrbins + 1) + sizeof(float) * a.nz + 16;
    cudaFuncSetAttribute(k_bin_power_plain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    long long blocks = (g.nmodes + 255) / 256;
    const long long cap = 8LL * sm_count();
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    k_bin_power_plain<<<(int)blocks, 256, smem, st>>>(a, g.thresh, g.w1, grid, bin_sum, F0sq);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -2;
}

template <int ROWS, int STAGES, int MPT>
static int run_corr_tma(const GridGeom& g, const GridArgs& a, float* grid, CorrTable corr, unsigned* status,
                        cudaStream_t st) {
    constexpr int NT = ROWS * (16 / MPT);
    CUtensorMap map;
    if (!make_grid_tmap(&map, grid, a.nrows16, ROWS)) return -1;
    const SmemPlan P = plan_smem(ROWS, STAGES, g.nrbins, 3 * a.nk + g.nrbins);
    if (P.total > 220 * 1024) return -1;
    auto kern = k_correct_tma<ROWS, STAGES, MPT>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P.total);
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, P.total);
    if (per_sm < 1) per_sm = 1;
    const int ntiles = (int)((a.nrows16 + ROWS - 1) / ROWS);
    int grid_n = sm_count() * per_sm;
    if (grid_n > ntiles) grid_n = ntiles > 0 ? ntiles : 1;
    kern<<<grid_n, NT, P.total, st>>>(map, a, g.thresh, g.cmap, corr, grid, status, ntiles);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -2;
}

static int corr_variant(const GridGeom& g, const GridArgs& a, float* grid, CorrTable corr, unsigned* status,
                        int rows, int stages, int mpt, cudaStream_t st) {
#define KSP_CORR_CASE(R, S, M) \
    if (rows == R && stages == S && mpt == M) return run_corr_tma<R, S, M>(g, a, grid, corr, status, st);
    KSP_CORR_CASE(128, 2, 16) KSP_CORR_CASE(128, 3, 16) KSP_CORR_CASE(128, 4, 16) KSP_CORR_CASE(256, 2, 16)
    KSP_CORR_CASE(256, 3, 16) KSP_CORR_CASE(128, 2, 8) KSP_CORR_CASE(128, 3, 8) KSP_CORR_CASE(128, 4, 8)
    KSP_CORR_CASE(256, 2, 8) KSP_CORR_CASE(256, 3, 8)
#undef KSP_CORR_CASE
    return run_corr_tma<256, 2, 16>(g, a, grid, corr, status, st);
}

int launch_apply_correction(const GridGeom& g, float* grid, CorrTable corr, float lnscale, unsigned* status, int tma,
                            int rows_per_cta, int stages, cudaStream_t st) {
    const GridArgs a = make_grid_args(g, corr.nk, lnscale);
    if (tma >= 3) {
        const int r = launch_correct_stream(a, grid, corr, status, rows_per_cta / 32, stages, st);
        if (r == 0) return 0;
        if (r == -2) return -2;
    } else if (tma && a.nrows16 > 0) {
        const int r = corr_variant(g, a, grid, corr, status, rows_per_cta, stages, tma == 2 ? 8 : 16, st);
        if (r == 0) return 0;
        if (r == -2) return -2;
    }
    const size_t smem = sizeof(int) * (2 * g.nrbins + 1) + sizeof(float) * 3 * a.nk + 16;
    cudaFuncSetAttribute(k_correct_plain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    long long blocks = (g.nmodes + 255) / 256;
    const long long cap = 8LL * sm_count();
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    k_correct_plain<<<(int)blocks, 256, smem, st>>>(a, g.thresh, g.cmap, corr, grid, status);
    return cudaPeekAtLastError() == cudaSuccess ? 1 : -2;
}

}  // namespace ksp
