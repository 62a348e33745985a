// ksp_batch.cu -- many independent integrator instances advanced by one launch sequence.
//
// Every instance is a complete integrator (its own cosmology and masses, transfer table,
// history of its own length, its own k bins).  One batched call performs, for every
// instance, the same arithmetic as the single-instance kernels of ksp_integrator.cu --
// which follow get_delta_nu_update, delta_tot_table.c:193-250 -- so each instance's
// delta_nu is the one a single-instance call returns:
//   kb_prologue     block per instance: provisional history row (:222), call scalars,
//                   knot factorisation of the history spline
//   kb_fs_segments  every instance's fslength segments (4-point Gauss-Legendre)
//   kb_fs_finish    block per instance: suffix sums of the segments -> fslength table
//   kb_fs_coeffs    thread per (instance, unknown): natural spline of the table
//   kb_dtot_coeffs  thread per (instance, bin): history-row spline coefficients
//   kb_nc_build     thread per (instance, node): node tables of the integrand
//   kb_dnu_qag      persistent warps that pull (instance, species, bin) tasks from an
//                   atomic queue; knots, row and coefficients staged into shared memory
//                   by TMA bulk copies; QAG with the 61-point Gauss-Kronrod rule
//   kb_finish       thread per (instance, bin): species sum, commit, NaN check, clamp
//   kb_corr         block per bound grid: correction table (interface_common.c:134-146)
// All kernels run on fixed launch shapes and read the call's totals from device memory,
// so one captured CUDA graph serves every call.
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>
#include "ksp_batch.h"
#include "ksp_ptx.cuh"

namespace ksp {

// largest i in [0, n) with off[i] <= v (off ascending, off[0] = 0)
__device__ __forceinline__ int owner_of(const int* off, int n, int v) {
    int lo = 0, hi = n;
    while (hi > lo + 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= v) lo = mid; else hi = mid;
    }
    return lo;
}

constexpr int kBatchSmallBlocks = 4 * 152;

// ------------------------------------------------------------------ prologue
// The call scalars (as k_scalars), update_delta_tot's provisional row (as k_update_row)
// and the knot factorisation (as k_scalars).
__global__ void kb_prologue(BatchDev b) {
    if (blockIdx.x == 0 && threadIdx.x == 0) b.hdr->counter = 0;
    for (int i = blockIdx.x; i < b.M; i += gridDim.x) {
        const BatchCall& P = b.calls[i];
        __syncthreads();  // the previous instance's scalars are complete
        if (!P.active) continue;
        const IntegratorDev& I = b.insts[i];
        StepScalars& S = *I.sc;
        const double a = P.a;
        const int Na = P.Na;
        const bool integrate = P.commit_row != -2;
        if (threadIdx.x < 32) call_scalars_warp(*I.B, a, P.loga, P.loga0, P.TimeTransfer, integrate ? Na : 1, S);
        if (threadIdx.x == 0 && integrate) I.scalefact[Na - 1] = P.loga;
        __syncthreads();
        if (!integrate) continue;
        const double OmegaNua3 = S.OmegaNua3, OmegaNu1 = S.OmegaNu1, partnu = S.partnu, Omeganonu = S.Omeganonu;
        for (int ik = threadIdx.x; ik < P.nk; ik += blockDim.x)
            I.dtot[(size_t)ik * I.ld + Na - 1] =
                get_delta_tot(I.nu_last[ik], I.dcdm[ik], OmegaNua3, Omeganonu, OmegaNu1, partnu);
        const double* xk = I.scalefact;
        for (int j = threadIdx.x; j + 1 < Na; j += blockDim.x) {
            const double h = xk[j + 1] - xk[j];
            I.knot_invh[j] = 1.0 / h;
            I.knot_h3[j] = h / 3.0;
            I.knot_ih3[j] = 1.0 / (3.0 * h);
        }
        if (threadIdx.x != 0) continue;
        if (P.nfs == 0) {
            S.fsl_A0a = 0.0;
            S.Nfs = 0;
        }
        const double* x = I.scalefact;
        if (Na > 2) {
            const int m = Na - 2;
            for (int r = P.start_row < 0 ? 0 : P.start_row; r < m; r++) {
                const double h0 = x[r + 1] - x[r], h1 = x[r + 2] - x[r + 1];
                double d = 2.0 * (h0 + h1);
                if (r > 0) {
                    const double f = h0 * I.knot_invdiag[r - 1];
                    d -= f * h0;
                    I.knot_fac[r] = f;
                }
                I.knot_invdiag[r] = 1.0 / d;
            }
        }
    }
}

// ------------------------------------------------------------------ fslength table
struct GL4b { double x[2], w[2]; };

// groups of 4 lanes over the fslength segments of all instances (flat, so that
// instances of any length balance), as k_fs_segments
__global__ void kb_fs_segments(BatchDev b, GL4b gl) {
    const int total = b.hdr->total_segs;  // groups
    const long long stride = (long long)gridDim.x * blockDim.x;  // a multiple of 4
    const long long end = 4LL * total;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < end; base += stride) {
        const long long gt = base + threadIdx.x;
        const int gg = (int)(gt >> 2), q = (int)(gt & 3);
        const bool live = gt < end;
        int i = 0, g = 0;
        if (live) {
            i = owner_of(b.fs_off, b.M, gg);
            g = gg - __ldg(b.fs_off + i);
        }
        const BatchCall& P = b.calls[i];
        const int Nfs = live ? P.nfs : 1;
        const double loga0 = P.loga0, loga = P.loga;
        const int npts = live ? fs_rule_points(Nfs, loga0, loga) : 4;
        fs_group_eval(*b.insts[i].B, Nfs, loga0, loga, npts, g, q, live, gl.x, gl.w, b.insts[i].fs_x,
                      b.insts[i].fs_seg);
    }
}

// block of 1024 threads per instance: the partition and summation order of k_fs_finish
// (which also runs with 1024 threads)
__global__ void __launch_bounds__(1024) kb_fs_finish(BatchDev b) {
    __shared__ double warp_tot[32];
    const int t = threadIdx.x, nt = blockDim.x, lane = t & 31, w = t >> 5;
    for (int i = blockIdx.x; i < b.M; i += gridDim.x) {
        const BatchCall& P = b.calls[i];
        const int Nfs = P.nfs;
        if (!P.active || P.commit_row == -2 || Nfs <= 0) continue;  // uniform over the block
        const IntegratorDev& I = b.insts[i];
        const int per = (Nfs + nt - 1) / nt;
        const int i0 = t * per, i1 = min(Nfs, i0 + per);
        double loc = 0;
        for (int k = i1 - 1; k >= i0; k--) loc += I.fs_seg[k];
        double v = loc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double n = __shfl_down_sync(0xffffffffu, v, o);
            if (lane + o < 32) v += n;
        }
        __syncthreads();  // warp_tot reuse across instances
        if (lane == 0) warp_tot[w] = v;
        __syncthreads();
        if (w == 0) {
            const int nw = nt >> 5;
            double u = lane < nw ? warp_tot[lane] : 0.0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double n = __shfl_down_sync(0xffffffffu, u, o);
                if (lane + o < 32) u += n;
            }
            if (lane < nw) warp_tot[lane] = u;
        }
        __syncthreads();
        const double later = (w + 1 < (nt >> 5)) ? warp_tot[w + 1] : 0.0;
        double run = v - loc + later;
        const double light = I.sc->light;
        for (int k = i1 - 1; k >= i0; k--) {
            run += I.fs_seg[k];
            I.fs_y[k] = light * run;
        }
        __syncthreads();
        if (t == 0) {
            I.sc->fsl_A0a = I.fs_y[0];
            I.sc->Nfs = Nfs;
            I.fs_c[0] = 0.0;
            I.fs_c[Nfs - 1] = 0.0;
        }
    }
}

// warp per instance: the fslength table's spline coefficients, as k_fs_coeffs
__global__ void kb_fs_coeffs(BatchDev b) {
    const int nw = blockDim.x >> 5;
    for (int i = blockIdx.x * nw + (threadIdx.x >> 5); i < b.M; i += gridDim.x * nw) {
        const BatchCall& P = b.calls[i];
        const int Nfs = P.nfs;
        if (!P.active || P.commit_row == -2 || Nfs <= 2) continue;  // uniform over the warp
        const IntegratorDev& I = b.insts[i];
        uniform_spline_warp(I.fs_y, I.fs_c, Nfs, (P.loga - P.loga0) / (Nfs - 1.));
    }
}

// ------------------------------------------------------------------ history splines
// thread per (instance, bin): the same substitutions as k_dtot_coeffs, each thread
// sweeping its own row in global memory.  With a million rows in flight the latency of
// the strided loads is hidden by parallelism, which a warp-per-row solve (one active
// lane per row) cannot match at this size.
__global__ void kb_dtot_coeffs(BatchDev b) {
    const int total = b.hdr->total_bins;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const int i = owner_of(b.bin_off, b.M, g);
        const int ik = g - __ldg(b.bin_off + i);
        const BatchCall& P = b.calls[i];
        const int Na = P.Na;
        if (!P.active || P.commit_row == -2 || Na <= 2) continue;
        const IntegratorDev& I = b.insts[i];
        const double* y = I.dtot + (size_t)ik * I.ld;
        double* c = I.coef + (size_t)ik * I.ld;
        const double* ih = I.knot_invh;
        const int m = Na - 2;
        double prev = 0;
        for (int k = 0; k < m; k++) {
            double r = 3.0 * ((y[k + 2] - y[k + 1]) * ih[k + 1] - (y[k + 1] - y[k]) * ih[k]);
            if (k > 0) r -= I.knot_fac[k] * prev;
            prev = r;
            c[k + 1] = r;
        }
        c[0] = 0.0;
        c[Na - 1] = 0.0;
        double next = c[m] * I.knot_invdiag[m - 1];
        c[m] = next;
        const double* x = I.scalefact;
        for (int k = m - 1; k-- > 0;) {
            const double off = x[k + 2] - x[k + 1];
            next = (c[k + 1] - off * next) * I.knot_invdiag[k];
            c[k + 1] = next;
        }
    }
}

// thread per (instance, slot, node): the node tables (as k_nc_build)
__global__ void kb_nc_build(BatchDev b) {
    const double XK[31] = KSP_GK61_XK_INIT;  // the abscissae of gk61_fill
    const int per = b.nc_slots * 61;
    const long long total = (long long)b.M * per;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
         g += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(g / per);
        const int q = (int)(g - (long long)i * per);
        const BatchCall& P = b.calls[i];
        if (!P.active || P.commit_row == -2 || P.nfs <= 0 || P.Na <= 1) continue;
        const IntegratorDev& I = b.insts[i];
        const StepScalars& S = *I.sc;
        const int slot = q / 61, jn = q - 61 * slot;
        double lo, hi;
        nc_interval(slot, S.loga0, S.loga, &lo, &hi);
        const double c = __dmul_rn(0.5, __dadd_rn(lo, hi));
        const double h = __dmul_rn(0.5, __dsub_rn(hi, lo));
        const double xk = jn < 30 ? -XK[jn] : (jn < 60 ? XK[jn - 30] : 0.0);
        const double x = __dadd_rn(c, __dmul_rn(h, xk));
        const double fs_inv = (S.Nfs - 1.) / (S.loga - S.loga0);
        const NodeTerms t =
            dnu_node_terms(I.B, I.fs_x, I.fs_y, I.fs_c, S.Nfs, S.loga0, fs_inv, I.scalefact, P.Na, x);
        I.nc_g[q] = t.g;
        I.nc_fsl[q] = t.fsl;
        I.nc_dx[q] = t.dx;
        I.nc_j[q] = t.j;
    }
}

size_t batch_qag_smem(int ldmax, int wpb) {
    return ((sizeof(Gk61Nodes) + 15) & ~size_t(15)) + wpb * (sizeof(QagList) + 5 * sizeof(double) * ldmax) +
           wpb * sizeof(uint64_t);
}

// Shared memory: Gk61Nodes | per warp: QagList, knots[ldmax], row[ldmax], coef[ldmax], seg_poly [2 ldmax] |
// mbarriers
__global__ void __launch_bounds__(128) kb_dnu_qag(BatchDev b) {
    extern __shared__ __align__(16) unsigned char sm[];
    Gk61Nodes& N = *reinterpret_cast<Gk61Nodes*>(sm);
    const size_t off = (sizeof(Gk61Nodes) + 15) & ~size_t(15);
    const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t per_warp = sizeof(QagList) + 5 * sizeof(double) * b.ldmax;
    unsigned char* wbase = sm + off + warp * per_warp;
    QagList& L = *reinterpret_cast<QagList*>(wbase);
    double* knots = reinterpret_cast<double*>(wbase + sizeof(QagList));
    double* row = knots + b.ldmax;
    double* rc = row + b.ldmax;
    double* sb = rc + b.ldmax;
    double* sd = sb + b.ldmax;
    uint64_t* mybar = reinterpret_cast<uint64_t*>(sm + off + nw * per_warp) + warp;
    gk61_fill(N, threadIdx.x, blockDim.x);
    if (lane == 0) ptx::mbar_init(mybar, 1);
    ptx::mbar_init_fence();
    __syncthreads();
    const int total = b.hdr->total_tasks;
    unsigned phase = 0;
    for (;;) {
        int task = 0;
        if (lane == 0) task = atomicAdd(&b.hdr->counter, 1);
        task = __shfl_sync(0xffffffffu, task, 0);
        if (task >= total) break;
        const int i = owner_of(b.task_off, b.M, task);
        const int loc = task - __ldg(b.task_off + i);
        const BatchCall& P = b.calls[i];
        const IntegratorDev& I = b.insts[i];
        const int nk = P.nk;
        const int si = loc / nk, ik = loc - si * nk;
        const int mi = P.spec[si];
        const Background* B = I.B;
        const StepScalars& S = *I.sc;
        const int Na = P.Na;
        const double k = I.wavenum[ik];
        // the task's divisions on lane 0
        double mnubykT = 0, kom = 0, fsi = 0;
        if (lane == 0) {
            mnubykT = B->mnu_J[mi] / B->kBtnu;
            kom = k / mnubykT;
            fsi = (S.Nfs - 1.) / (S.loga - S.loga0);
        }
        mnubykT = __shfl_sync(0xffffffffu, mnubykT, 0);
        kom = __shfl_sync(0xffffffffu, kom, 0);
        fsi = __shfl_sync(0xffffffffu, fsi, 0);
        double integral = 0;
        const bool integrate = !S.skip_integral && Na > 1 && mnubykT > 0;
        if (integrate) {
            const unsigned bytes = (unsigned)(((Na + 1) & ~1) * sizeof(double));
            __syncwarp();
            if (lane == 0) {
                ptx::fence_async_smem();
                ptx::mbar_expect_tx(mybar, Na > 2 ? 3 * bytes : 2 * bytes);
                ptx::bulk_g2s(knots, I.scalefact, bytes, mybar);
                ptx::bulk_g2s(row, I.dtot + (size_t)ik * I.ld, bytes, mybar);
                if (Na > 2) ptx::bulk_g2s(rc, I.coef + (size_t)ik * I.ld, bytes, mybar);
            }
            const bool got = __all_sync(0xffffffffu, ptx::mbar_wait_bounded(mybar, phase));  // warp-uniform
            phase ^= 1;
            if (!got) {
                if (lane == 0) atomicOr(I.status, kStTimeout);
                ptx::mbar_wait_bounded(mybar, phase ^ 1);  // the copies still in flight
                return;
            }
            const KnotSeg ks{I.knot_invh, I.knot_h3, I.knot_ih3};
            if (Na > 2) seg_poly(row, rc, Na, ks, sb, sd, lane, 32);
            __syncwarp();
            const double qc = S.partnu_now > 0 ? B->vcrit * mnubykT : 0.0;
            const DnuIntegrandC f = dnu_integrand_pre(I, S, kom, fsi, qc, knots, row, rc, sb, sd, Na);
            const QagResult r = qag_warp_c(f, N, L, S.loga0, S.loga, 0.0, S.relerr, kQagLimit);
            integral = r.result;
            if (!r.ok && lane == 0) atomicOr(I.status, kStGsl);
        }
        if (lane == 0) I.dnu_s[(size_t)mi * I.nk_alloc + ik] = dnu_task_value(I, S, ik, k, mnubykT, integrate, integral);
    }
}

// ------------------------------------------------------------------ finish
// k_combine + k_finish for every bin of every instance
__global__ void kb_finish(BatchDev b) {
    const int total = b.hdr->total_bins;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const int i = owner_of(b.bin_off, b.M, g);
        const int ik = g - __ldg(b.bin_off + i);
        const BatchCall& P = b.calls[i];
        if (!P.active) continue;
        const IntegratorDev& I = b.insts[i];
        const StepScalars& S = *I.sc;
        double out;
        if (P.commit_row == -2) {
            out = I.nu_last[ik];  // same scale factor: delta_nu_last as it is
            I.dnu[ik] = out;
        } else {
            double v = 0;
            for (int mi = 0; mi < kNuSpecies; mi++)
                if (I.B->deg[mi] > 0) v += I.dnu_s[(size_t)mi * I.nk_alloc + ik] * S.omeganu[mi] / S.Omega_nu_tot;
            I.dnu[ik] = v;
            if (!P.dry) I.nu_last[ik] = v;
            if (P.commit_row >= 0 && !P.dry) {
                if (ik == 0) I.scalefact[P.commit_row] = P.loga;
                I.dtot[(size_t)ik * I.ld + P.commit_row] =
                    get_delta_tot(v, I.dcdm[ik], S.OmegaNua3, S.Omeganonu, S.OmegaNu1, S.partnu);
            }
            if (isnan(v)) atomicOr(I.status, kStDnuNaN);
            out = v < 0 ? 0.0 : v;
        }
        b.dnu_pool[__ldg(b.bin_off + i) + ik] = out;
    }
}

// correction tables of the bound grids (the table part of k_finish)
__global__ void kb_corr(BatchDev b, const BatchGridCorr* grids, int ngrid) {
    for (int gi = blockIdx.x; gi < ngrid; gi += gridDim.x) {
        const BatchGridCorr G = grids[gi];
        const BatchCall& P = b.calls[G.inst];
        if (!P.active) continue;
        const IntegratorDev& I = b.insts[G.inst];
        const double norm = I.sc->kspace_prefac;
        const double* dnu_out = b.dnu_pool + b.bin_off[G.inst];
        const int nk = P.nk;
        if (threadIdx.x == 0 && G.norm_out) *G.norm_out = norm;
        for (int j = threadIdx.x; j < nk; j += blockDim.x) {
            const double lk = log(G.keff[j]);
            const double r = dnu_out[j] / I.dcdm[j];
            G.corr.xf[j] = (float)lk;
            G.corr.rn[j] = (float)(norm * r);
            double s = 0;
            if (j + 1 < nk) {
                const double lk1 = log(G.keff[j + 1]);
                const double r1 = dnu_out[j + 1] / I.dcdm[j + 1];
                s = norm * (r1 - r) / (lk1 - lk);
            }
            G.corr.sn[j] = (float)s;
            if (!isfinite(norm * r) || !isfinite(s)) atomicOr(I.status, kStGridNaN);
        }
    }
}

// ------------------------------------------------------------------ launchers
static void gl_nodes_b(int n, double* X, double* Wt) {  // Newton on P_n, positive half
    for (int i = 0; i < n / 2; i++) {
        double x = cos(3.14159265358979323846 * (i + 0.75) / (n + 0.5)), dp = 0;
        for (int it = 0; it < 100; it++) {
            double p0 = 1, p1 = x;
            for (int k = 2; k <= n; k++) {
                const double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (x * p1 - p0) / (x * x - 1);
            const double dx = p1 / dp;
            x -= dx;
            if (fabs(dx) < 1e-16) break;
        }
        X[i] = x;
        Wt[i] = 2 / ((1 - x * x) * dp * dp);
    }
}

void batch_set_attributes() {
    raise_dynamic_smem_limit(reinterpret_cast<const void*>(kb_dnu_qag));
}

void launch_batch_update(const BatchDev& b, cudaStream_t st) {
    static GL4b gl;
    static bool init = false;
    if (!init) {
        gl_nodes_b(4, gl.x, gl.w);
        init = true;
    }
    const int nb = kBatchSmallBlocks;
    kb_prologue<<<b.M < nb ? b.M : nb, 128, 0, st>>>(b);
    kb_fs_segments<<<nb, 256, 0, st>>>(b, gl);
    kb_fs_finish<<<b.M < 2 * 152 ? b.M : 2 * 152, 1024, 0, st>>>(b);
    kb_fs_coeffs<<<nb, 128, 0, st>>>(b);
    kb_dtot_coeffs<<<nb, 128, 0, st>>>(b);
    kb_nc_build<<<nb, 128, 0, st>>>(b);
    kb_dnu_qag<<<b.qag_blocks, 32 * b.wpb, batch_qag_smem(b.ldmax, b.wpb), st>>>(b);
    kb_finish<<<nb, 256, 0, st>>>(b);
}

void launch_batch_corr(const BatchDev& b, const BatchGridCorr* g, int ngrid, cudaStream_t st) {
    if (ngrid > 0) kb_corr<<<ngrid, 256, 0, st>>>(b, g, ngrid);
}

}  // namespace ksp
