// ksp_adjoint.cu -- hand-written adjoint of one neutrino-correction step.
//
// The differentiated function is one step at scale factor a with the integrator state
// (delta_nu_init, delta_nu_last) held fixed:
//   P_b    = S_b(x) / (|x_0|^2 C_b)                          (binning, K1)
//   dcdm_b = sqrt(P_b L^3)
//   D_b,Na-1 = get_delta_tot(delta_nu_last_b, dcdm_b, ...)     (provisional row)
//   dnu_b  = sum_s w_s [ J(k_b fsl0/m_s) nu_init_b (1+..) + prefac QAG_s,b(D_b, m_s) ]
//   r_b    = max(dnu_b, 0) / dcdm_b,   P_nu,b = max(dnu_b,0)^2
//   y_m    = x_m (1 + norm interp_r(log|k_m|))                (correction, K3)
// Adjoint (subdivision of every QAG held fixed, background Omega_nu(a), H(a) fixed):
//   B1  k_adj_reduce8        rbar_j = norm sum_m (gbar_m . x_m) dinterp/dr_j   (reads gbar, x)
//   B2a k_adj_bins           dnubar_b from rbar and the P_nu cotangent
//   B2  k_dnu_adj            warp per (species, bin): history row and spline
//                            coefficients staged by TMA bulk copies; the GK61 nodes of the
//                            stored (or recomputed) final QAG intervals give
//                            d/d(row) through the spline (cubic basis + transposed
//                            natural-spline solve) and d/dm through J's argument
//   B2c k_adj_bins2          dcdm/P cotangents -> per-bin Q_b and the DC term
//   B3  k_adj_grid_plain     xbar_m = gbar_m smth_m + Q_b w_m W_m^4 x_m   (reads gbar, x; writes xbar)
#include <cuda_runtime.h>
#include <stdint.h>
#include "ksp_internal.h"
#include "ksp_gridutil.cuh"
#include "ksp_ptx.cuh"

namespace ksp {

// d specialJ_fit / dx (derivative of the rational fit of delta_tot_table.c:417-428)
__device__ __forceinline__ double specialJ_fit_deriv(double x) {
    if (x <= 0.) return 0.;
    const double x2 = x * x, x4 = x2 * x2, x8 = x4 * x4;
    const double p = exp(4.1811 * log(x));
    const double N = 1. + 0.0168 * x2 + 0.0407 * x4;
    const double D = 1. + 2.1734 * x2 + 1.6787 * p + 0.1467 * x8;
    const double dN = 0.0336 * x + 0.1628 * x2 * x;
    const double dD = 4.3468 * x + 1.6787 * 4.1811 * p / x + 1.1736 * x4 * x2 * x;
    return (dN * D - N * dD) / (D * D);
}

// ------------------------------------------------------------------ B1
// Interpolation weights of the correction for integer k^2 (same segment choice and
// clamping as corr_delta): node j0 gets w0, node j0+1 gets w1.
__device__ __forceinline__ void corr_weights(int k2, const GridArgs& g, const CorrSmem& t, int& j0, float& w0,
                                             float& w1) {
    const int b = bin_of(k2, g.c1, t.thr, g.nrbins);
    const int c = t.cmap[b];
    const float x = fmaf(0.5f, __logf((float)k2), g.lnscale);
    const int nk = g.nk;
    if (c < 0) { j0 = 0; w0 = 0.f; w1 = 0.f; return; }
    if (x < t.xf[c]) {
        if (c == 0) { j0 = 0; w0 = 1.f; w1 = 0.f; return; }
        j0 = c - 1;
    } else {
        if (c >= nk - 1) { j0 = nk - 2; w0 = 0.f; w1 = 1.f; return; }
        j0 = c;
    }
    const float tt = (x - t.xf[j0]) / (t.xf[j0 + 1] - t.xf[j0]);
    w0 = 1.f - tt;
    w1 = tt;
}

// B1, 8 consecutive modes per thread: the table segment of the modes is followed in
// x = log k (as the correction pass does), and a run of modes in one segment j
// accumulates A = sum u and B = sum u t (u = gbar . x, t the position in the segment) in
// FP32, so d/dr_j gets A - B and d/dr_{j+1} gets B once per run, into the warp's own
// float totals; each block adds its warps' totals to the FP64 node sums once.
__global__ void __launch_bounds__(256) k_adj_reduce8(GridArgs g, CorrTable corr, const float* __restrict__ gbar,
                                                     const float* __restrict__ x, double* node_sum, long long nchunks,
                                                     int adv_il, int adv_j, int adv_z) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5;
    float* s_xf = reinterpret_cast<float*>(sm_raw);
    float* s_acc = s_xf + g.nk;  // [nw][nk]
    for (int i = threadIdx.x; i < g.nk; i += blockDim.x) s_xf[i] = corr.xf[i];
    for (int i = threadIdx.x; i < nw * g.nk; i += blockDim.x) s_acc[i] = 0.f;
    __syncthreads();
    float* acc = s_acc + warp * g.nk;
    const int nk = g.nk;
    // current segment: node j0, t = (x - x0) * inv + tadd, valid for xlo <= x < xhi
    int j0 = -1;
    float xlo = 3.0e38f, xhi = -3.0e38f, x0 = 0.f, inv = 0.f, tadd = 0.f;
    float A = 0.f, B = 0.f;
    auto flush = [&]() {
        if (j0 >= 0 && (A != 0.f || B != 0.f)) {
            atomicAdd(acc + j0, A - B);
            atomicAdd(acc + j0 + 1, B);
        }
        A = 0.f;
        B = 0.f;
    };
    auto locate = [&](float xm) {
        int lo = -1, hi = nk;  // largest j with xf[j] <= xm
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (s_xf[mid] <= xm) lo = mid; else hi = mid;
        }
        if (lo < 0) {  // constant below the first node: all to node 0
            j0 = 0; xlo = -3.0e38f; xhi = s_xf[0]; x0 = 0.f; inv = 0.f; tadd = 0.f;
        } else if (lo >= nk - 1) {  // constant from the last node: all to node nk-1
            j0 = nk - 2; xlo = s_xf[nk - 1]; xhi = 3.0e38f; x0 = 0.f; inv = 0.f; tadd = 1.f;
        } else {
            j0 = lo; xlo = s_xf[lo]; xhi = s_xf[lo + 1]; x0 = xlo; inv = 1.f / (xhi - xlo); tadd = 0.f;
        }
    };
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long ci = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (ci < nchunks) {
        const long long m0 = ci * 8;
        KCursor c;
        c.init(g, m0 / g.nz, (int)(m0 % g.nz), 0);
        for (; ci < nchunks; ci += stride) {
            const long long mb = ci * 8;
            const bool full = mb + 8 <= g.nmodes;
            float gv[16], xv[16];
            if (full) {
                const float4* gp = reinterpret_cast<const float4*>(gbar + 2 * mb);
                const float4* xp = reinterpret_cast<const float4*>(x + 2 * mb);
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float4 a = __ldg(gp + q), bq = __ldg(xp + q);
                    gv[4 * q] = a.x; gv[4 * q + 1] = a.y; gv[4 * q + 2] = a.z; gv[4 * q + 3] = a.w;
                    xv[4 * q] = bq.x; xv[4 * q + 1] = bq.y; xv[4 * q + 2] = bq.z; xv[4 * q + 3] = bq.w;
                }
            } else {
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const bool in = mb * 2 + q < 2 * g.nmodes;
                    gv[q] = in ? gbar[2 * mb + q] : 0.f;
                    xv[q] = in ? x[2 * mb + q] : 0.f;
                }
            }
            KCursor cc = c;
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const int k2 = cc.kxy2 + cc.z * cc.z;
                if (k2 != 0 && mb + e < g.nmodes) {
                    const float xm = fmaf(0.5f, __logf((float)k2), g.lnscale);
                    if (xm < xlo || xm >= xhi) {
                        flush();
                        locate(xm);
                    }
                    const float u = fmaf(gv[2 * e], xv[2 * e], gv[2 * e + 1] * xv[2 * e + 1]);
                    const float t = fmaf(xm - x0, inv, tadd);
                    A += u;
                    B = fmaf(u, t, B);
                }
                cc.next(g);
            }
            // advance the cursor by the grid stride (stride * 8 modes = adv_il slabs, adv_j
            // rows, adv_z modes)
            c.z += adv_z;
            int carry = 0;
            if (c.z >= g.nz) { c.z -= g.nz; carry = 1; }
            c.j += adv_j + carry;
            carry = 0;
            if (c.j >= g.N) { c.j -= g.N; carry = 1; }
            c.il += adv_il + carry;
            c.set_row(g);
        }
    }
    flush();
    __syncthreads();
    for (int i = threadIdx.x; i < nk; i += blockDim.x) {
        double v = 0.0;
        for (int w = 0; w < nw; w++) v += (double)s_acc[w * nk + i];
        if (v != 0.0) atomicAdd(node_sum + i, v);
    }
}

__global__ void k_adj_reduce_plain(GridArgs g, const int* __restrict__ thresh, const int* __restrict__ cmapg,
                                   CorrTable corr, const float* __restrict__ gbar, const float* __restrict__ x,
                                   double* node_sum) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    double* s_acc = reinterpret_cast<double*>(sm_raw);  // doubles first: 8-byte aligned
    int* s_thr = reinterpret_cast<int*>(s_acc + g.nk);
    int* s_cmap = s_thr + g.nrbins + 1;
    float* s_tab = reinterpret_cast<float*>(s_cmap + g.nrbins);
    for (int i = threadIdx.x; i <= g.nrbins; i += blockDim.x) s_thr[i] = thresh[i];
    for (int i = threadIdx.x; i < g.nrbins; i += blockDim.x) s_cmap[i] = cmapg[i];
    for (int i = threadIdx.x; i < g.nk; i += blockDim.x) {
        s_tab[i] = corr.xf[i];
        s_tab[g.nk + i] = corr.rn[i];
        s_tab[2 * g.nk + i] = corr.sn[i];
        s_acc[i] = 0.0;
    }
    __syncthreads();
    CorrSmem T{s_thr, s_cmap, s_tab, s_tab + g.nk, s_tab + 2 * g.nk};
    // runs keyed by the segment's first node, Kahan-summed in FP32 per node pair
    int rj = -1;
    float a0 = 0.f, c0 = 0.f, a1 = 0.f, c1 = 0.f;
    auto flush = [&]() {
        if (rj >= 0) {
            atomicAdd(&s_acc[rj], (double)a0 - (double)c0);
            if (rj + 1 < g.nk) atomicAdd(&s_acc[rj + 1], (double)a1 - (double)c1);
        }
    };
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < g.nmodes;
         m += (long long)gridDim.x * blockDim.x) {
        const long long r = m / g.nz;
        const int z = (int)(m - r * g.nz);
        const int il = (int)(r / g.N), j = (int)(r - (long long)il * g.N);
        const int kx = kval(g.slab0 + il, g.N), ky = kval(j, g.N);
        const int k2 = kx * kx + ky * ky + z * z;
        if (k2 == 0) continue;
        const float2 gv = reinterpret_cast<const float2*>(gbar)[m];
        const float2 xv = reinterpret_cast<const float2*>(x)[m];
        const float v = fmaf(gv.x, xv.x, gv.y * xv.y);
        int j0;
        float w0, w1;
        corr_weights(k2, g, T, j0, w0, w1);
        if (j0 != rj) {
            flush();
            rj = j0; a0 = c0 = a1 = c1 = 0.f;
        }
        {
            const float y = v * w0 - c0, t = a0 + y;
            c0 = (t - a0) - y; a0 = t;
        }
        {
            const float y = v * w1 - c1, t = a1 + y;
            c1 = (t - a1) - y; a1 = t;
        }
    }
    flush();
    __syncthreads();
    for (int i = threadIdx.x; i < g.nk; i += blockDim.x)
        if (s_acc[i] != 0.0) atomicAdd(node_sum + i, s_acc[i]);
}

// ------------------------------------------------------------------ B2a / B2c
struct AdjBins {
    const double* node_sum;  // sum over modes of (gbar.x) dinterp/dr_j   [nk]
    const double* pnu_bar;   // cotangent of P_nu                         [nk]
    const double* dnu;       // combined delta_nu (unclamped)             [nk]
    const double* dcdm;      // [nk]
    const double* power;     // P_b normalised                           [nk]
    const long long* count;  // mode count per bin (indexed by bin)
    const int* compact;      // compact -> bin
    const double* F0sq;
    double* dnu_bar;         // out [nk]
    const double* dprov_bar; // provisional-row cotangent (from k_dnu_adj), stride ld
    double* rbar;            // out [nk]
    double* Q;               // out: 2 Pbar_b / (F0 C_b), indexed by bin [nrbins]
    double* dc_sum;          // out: sum_b Pbar_b P_b (DC term)
    double norm, L3, fcdm;
    int ld;
};

__global__ void k_adj_bins(AdjBins A, int nk) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nk) return;
    const double rb = A.norm * A.node_sum[b];
    A.rbar[b] = rb;
    const double v = A.dnu[b];
    const double out = v < 0 ? 0.0 : v;
    A.dnu_bar[b] = v > 0 ? (2.0 * out * A.pnu_bar[b] + rb / A.dcdm[b]) : 0.0;
}

__global__ void k_adj_bins2(AdjBins A, int nk) {
    __shared__ double red[256];
    double acc = 0;
    for (int b = threadIdx.x; b < nk; b += blockDim.x) {
        const double v = A.dnu[b];
        const double out = v < 0 ? 0.0 : v;
        const double dc = A.dcdm[b];
        const double dcbar = -A.rbar[b] * out / (dc * dc) + A.dprov_bar[(size_t)b * A.ld] * A.fcdm;
        const double Pbar = dcbar * A.L3 / (2.0 * dc);
        const int bin = A.compact[b];
        A.Q[bin] = 2.0 * Pbar / (*A.F0sq * (double)A.count[bin]);
        acc += Pbar * A.power[b];
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int i = 0; i < (int)blockDim.x; i++) s += red[i];
        *A.dc_sum = s;
    }
}

// ------------------------------------------------------------------ B2
struct DnuAdjArgs {
    const double* dnu_bar;   // [nk]
    double* Dbar;            // [nk][ld] history cotangent (columns < Na)
    double* mbar;            // [kNuSpecies]
    const double* ivals;     // stored intervals [kNuSpecies][nk][kQagLimit][2] or null
    const int* nivals;       // [kNuSpecies][nk]
    int recompute;
};

// Node quantities of the delta_nu integrand for one bin (delta_tot_table.c:492-500).
struct DnuNode {
    double g, J, Jd, S, xj;
    int seg;
    double dx, h;
};

__device__ __forceinline__ DnuNode dnu_node(const Background* B, double k, double mnubykT, double qc, double nfl,
                                            const double* fs_x, const double* fs_y, const double* fs_c, int nfs,
                                            double fs_x0, double fs_inv, const double* kx, const double* ky,
                                            const double* kc, int na, double logai) {
    DnuNode o;
    int i = (int)((logai - fs_x0) * fs_inv);
    i = i < 0 ? 0 : (i > nfs - 2 ? nfs - 2 : i);
    while (i > 0 && logai < __ldg(fs_x + i)) i--;
    while (i < nfs - 2 && logai >= __ldg(fs_x + i + 1)) i++;
    double fsl;
    {
        const double x0 = __ldg(fs_x + i), x1 = __ldg(fs_x + i + 1);
        const double y0 = __ldg(fs_y + i), y1 = __ldg(fs_y + i + 1);
        const double c0 = __ldg(fs_c + i), c1 = __ldg(fs_c + i + 1);
        const double h = x1 - x0, dx = logai - x0;
        const double b = (y1 - y0) / h - h * (c1 + 2.0 * c0) / 3.0;
        const double d = (c1 - c0) / (3.0 * h);
        fsl = y0 + dx * (b + dx * (c0 + dx * d));
    }
    const int j = seg_bsearch(kx, na, logai);
    o.seg = j;
    o.h = kx[j + 1] - kx[j];
    o.dx = logai - kx[j];
    o.S = na > 2 ? cspline_seg(kx, ky, kc, j, logai) : linear_seg(kx, ky, j, logai);
    o.xj = k * fsl / mnubykT;
    o.J = specialJ(o.xj, qc, nfl);
    o.Jd = qc > 0 ? 0.0 : specialJ_fit_deriv(o.xj);
    const double ai = exp(logai);
    o.g = fsl / (ai * hubble(*B, ai));
    return o;
}

// The 61 nodes of one interval [a_i, b_i] of the final subdivision, by one warp (lane
// order = ascending x): each node's weight w g J times the spline weights of its
// history segment goes to ybar / cbar (cotangents of the delta_tot row values and of
// its spline second derivatives), and its mass derivative to mder (per lane).
__device__ __forceinline__ void adj_interval(const DnuIntegrandC& fi, const Gk61Nodes& N, const double* knots,
                                             const double* row, const double* rc, int Na, double qc, double a_i,
                                             double b_i, double loga0, double loga, int nc_slots, double ckm,
                                             double* ybar, double* cbar, double& mder, int lane) {
    const double c = __dmul_rn(0.5, __dadd_rn(a_i, b_i));
    const double h = __dmul_rn(0.5, __dsub_rn(b_i, a_i));
    const int slot = nc_slot_of(a_i, b_i, loga0, loga, nc_slots);
    // nodes in ascending x (lane order): the history segments grow with the
    // lane, so a segmented warp sum per segment replaces atomic updates
    for (int m = 0; m < 2; m++) {
        const int sidx = lane + 32 * m;
        double ya = 0.0, yb = 0.0, ca = 0.0, cb = 0.0;
        int key = -1;
        if (sidx < 61) {
            const int jn = sidx < 30 ? sidx : (sidx == 30 ? 60 : 90 - sidx);
            const double xn = __dadd_rn(c, __dmul_rn(h, N.x[jn]));
            const NodeTerms t = fi.terms(slot, jn, xn);
            double J, Jd;
            if (qc > 0) {
                J = specialJ(t.fsl * fi.k_over_m, qc, fi.nfl);
                Jd = 0.0;
            } else {
                specialJ_fit_tab_d(t.fsl * fi.k_over_m, J, Jd);
            }
            const double hh = knots[t.j + 1] - knots[t.j];
            const double dx = t.dx;
            const double wt = N.wk[jn] * h;
            const double u = wt * t.g * J;
            const double tt = dx / hh;
            ya = u * (1 - tt);
            yb = u * tt;
            if (Na > 2) {
                ca = u * (dx * (-2 * hh / 3) + dx * dx - dx * dx * dx / (3 * hh));
                cb = u * (dx * (-hh / 3) + dx * dx * dx / (3 * hh));
            }
            key = t.j;
            mder += ckm * wt * t.g * Jd * t.fsl * dnu_S_poly(t, row, rc, fi.sb, fi.sd, Na, fi.ks);
        }
        bool tail;
        warp_seg_sum4(key, ya, yb, ca, cb, tail);
        // each run's last lane adds its run; left ends first, then right ends
        // (two runs may share a knot), so no two lanes touch one entry at once
        if (tail && key >= 0) { ybar[key] += ya; cbar[key] += ca; }
        __syncwarp();
        if (tail && key >= 0) { ybar[key + 1] += yb; cbar[key + 1] += cb; }
        __syncwarp();
    }
}

// Shared memory per CTA: Gk61Nodes | knots[ld] | per warp: QagList, row[ld], coef[ld], ybar[ld], cbar[ld],
// seg_poly [2 ld] | bars
__global__ void __launch_bounds__(128) k_dnu_adj(IntegratorDev I, DnuAdjArgs A, int nk, int Na, int nspec,
                                                 int4 spec_ids) {
    extern __shared__ __align__(16) unsigned char sm[];
    Gk61Nodes& N = *reinterpret_cast<Gk61Nodes*>(sm);
    size_t off = (sizeof(Gk61Nodes) + 15) & ~size_t(15);
    double* knots = reinterpret_cast<double*>(sm + off);
    off += sizeof(double) * I.ld;
    const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t per_warp = sizeof(QagList) + 6 * sizeof(double) * I.ld;
    unsigned char* wbase = sm + off + warp * per_warp;
    QagList& L = *reinterpret_cast<QagList*>(wbase);
    double* row = reinterpret_cast<double*>(wbase + sizeof(QagList));
    double* rc = row + I.ld;
    double* ybar = rc + I.ld;
    double* cbar = ybar + I.ld;
    double* sb = cbar + I.ld;
    double* sd = sb + I.ld;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + off + nw * per_warp);
    uint64_t* mybar = bars + warp;
    gk61_fill(N, threadIdx.x, blockDim.x);
    for (int i = threadIdx.x; i < Na; i += blockDim.x) knots[i] = I.scalefact[i];
    if (lane == 0) ptx::mbar_init(mybar, 1);
    ptx::mbar_init_fence();
    __syncthreads();
    const Background* B = I.B;
    const StepScalars& S = *I.sc;
    const unsigned row_bytes = (unsigned)(((Na + 1) & ~1) * sizeof(double));
    unsigned phase = 0;
    for (int task = blockIdx.x * nw + warp; task < nspec * nk; task += gridDim.x * nw) {
        const int si = task / nk, ik = task % nk;
        const int mi = si == 0 ? spec_ids.x : (si == 1 ? spec_ids.y : spec_ids.z);
        const double mnu = B->mnu_J[mi];
        const double mnubykT = mnu / B->kBtnu;
        const double k = I.wavenum[ik];
        const double sbar = A.dnu_bar[ik] * S.omeganu[mi] / S.Omega_nu_tot;
        if (sbar == 0.0) continue;
        double mder = 0.0;
        // initial-condition piece (delta_tot_table.c:525-535)
        if (lane == 0 && mnubykT > 0) {
            const double x0 = k * S.fsl_A0a / mnubykT;
            mder += sbar * specialJ_fit_deriv(x0) * (-x0 / mnu) * I.nu_init[ik] * (1. + S.deriv_prefac * S.fsl_A0a);
        }
        const bool integrate = !S.skip_integral && Na > 1 && mnubykT > 0;
        if (integrate) {
            __syncwarp();
            if (lane == 0) {
                ptx::fence_async_smem();
                ptx::mbar_expect_tx(mybar, Na > 2 ? 2 * row_bytes : row_bytes);
                ptx::bulk_g2s(row, I.dtot + (size_t)ik * I.ld, row_bytes, mybar);
                if (Na > 2) ptx::bulk_g2s(rc, I.coef + (size_t)ik * I.ld, row_bytes, mybar);
            }
            for (int i = lane; i < Na; i += 32) { ybar[i] = 0.0; cbar[i] = 0.0; }
            const bool got = __all_sync(0xffffffffu, ptx::mbar_wait_bounded(mybar, phase));  // warp-uniform
            phase ^= 1;
            if (!got) {
                if (lane == 0) atomicOr(I.status, kStTimeout);
                ptx::mbar_wait_bounded(mybar, phase ^ 1);
                return;
            }
            const KnotSeg ks{I.knot_invh, I.knot_h3, I.knot_ih3};
            if (Na > 2) seg_poly(row, rc, Na, ks, sb, sd, lane, 32);
            __syncwarp();
            const double qc = S.partnu_now > 0 ? B->vcrit * mnubykT : 0.0;
            // the final subdivision of the forward QAG: stored, or recomputed (same decisions)
            int nint;
            const double* iv = nullptr;
            if (!A.recompute && A.ivals) {
                nint = A.nivals[(size_t)mi * I.nk_alloc + ik];
                iv = A.ivals + ((size_t)mi * I.nk_alloc + ik) * kQagLimit * 2;
            } else {
                const DnuIntegrandC f = dnu_integrand(I, S, k, mnubykT, qc, knots, row, rc, sb, sd, Na);
                QagResult r = qag_warp_c(f, N, L, S.loga0, S.loga, 0.0, S.relerr, kQagLimit);
                nint = r.nint;
            }
            const DnuIntegrandC fi = dnu_integrand(I, S, k, mnubykT, qc, knots, row, rc, sb, sd, Na);
            const double ckm = -sbar * S.prefac * fi.k_over_m / mnu;  // d(J's argument)/dm per fsl
            for (int q = 0; q < nint; q++)
                adj_interval(fi, N, knots, row, rc, Na, qc, iv ? iv[2 * q] : L.a[q], iv ? iv[2 * q + 1] : L.b[q],
                             S.loga0, S.loga, I.nc_slots, ckm, ybar, cbar, mder, lane);
            __syncwarp();
            if (Na > 2) {
                // z = A^-1 cbar_int with the shared factorisation (A is symmetric, so the
                // solve of the forward pass applies); then ybar += rhs^T z, gathered per
                // entry in the order the scatter over rows would add them
                const int m = Na - 2;
                spline_solve_scan(I, m, cbar);
                const double* ih = I.knot_invh;
                for (int j = lane; j < Na; j += 32) {
                    double v = ybar[j];
                    if (j >= 2 && j <= m + 1) v += 3 * cbar[j - 1] * ih[j - 1];
                    if (j >= 1 && j <= m) v -= 3 * cbar[j] * (ih[j - 1] + ih[j]);
                    if (j < m) v += 3 * cbar[j + 1] * ih[j];
                    ybar[j] = v;
                }
            }
            __syncwarp();
            for (int j = lane; j < Na; j += 32)  // column Na-1: the provisional row
                atomicAdd(&A.Dbar[(size_t)ik * I.ld + j], S.prefac * sbar * ybar[j]);
        }
        mder = warp_sum_to0(mder);
        if (lane == 0 && mder != 0.0) atomicAdd(&A.mbar[mi], mder);
    }
}

// ------------------------------------------------------------------ B3
__global__ void k_adj_grid_plain(GridArgs g, const int* __restrict__ thresh, const int* __restrict__ cmapg,
                                 const float* __restrict__ w1g, CorrTable corr, const float* __restrict__ gbar,
                                 const float* __restrict__ x, float* xbar, const double* __restrict__ Q,
                                 const double* dc_sum, const double* F0sq) {
    extern __shared__ unsigned char sm_raw[];
    int* s_thr = reinterpret_cast<int*>(sm_raw);
    int* s_cmap = s_thr + g.nrbins + 1;
    float* s_tab = reinterpret_cast<float*>(s_cmap + g.nrbins);
    float* s_w1 = s_tab + 3 * g.nk;
    float* s_Q = s_w1 + g.nz;
    for (int i = threadIdx.x; i <= g.nrbins; i += blockDim.x) s_thr[i] = thresh[i];
    for (int i = threadIdx.x; i < g.nrbins; i += blockDim.x) {
        s_cmap[i] = cmapg[i];
        s_Q[i] = (float)Q[i];
    }
    for (int i = threadIdx.x; i < g.nk; i += blockDim.x) {
        s_tab[i] = corr.xf[i];
        s_tab[g.nk + i] = corr.rn[i];
        s_tab[2 * g.nk + i] = corr.sn[i];
    }
    for (int i = threadIdx.x; i < g.nz; i += blockDim.x) s_w1[i] = w1g[i];
    __syncthreads();
    CorrSmem T{s_thr, s_cmap, s_tab, s_tab + g.nk, s_tab + 2 * g.nk};
    unsigned flags = 0;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < g.nmodes;
         m += (long long)gridDim.x * blockDim.x) {
        const long long r = m / g.nz;
        ModeCursor c;
        c.z = (int)(m - r * g.nz);
        c.il = (int)(r / g.N);
        c.j = (int)(r - (long long)c.il * g.N);
        c.set_row(g, s_w1);
        const int k2 = c.kxy2 + c.z * c.z;
        const float2 gv = reinterpret_cast<const float2*>(gbar)[m];
        const float2 xv = reinterpret_cast<const float2*>(x)[m];
        float2 o;
        if (k2 == 0) {
            // DC: y_0 = x_0, and |x_0|^2 normalises every P_b
            const double f = -2.0 * (*dc_sum) / (*F0sq);
            o.x = (float)(gv.x + f * xv.x);
            o.y = (float)(gv.y + f * xv.y);
        } else {
            const float d = corr_delta(k2, g, T, flags);
            const float t = __fmul_rn(c.iwxy, s_w1[c.z]);
            const float inv = __fmul_rn(t, t);
            float wW = __fmul_rn(inv, inv);
            if (c.z != 0 && c.z != g.half) wW = wW + wW;
            const float q = s_Q[bin_of(k2, g.c1, s_thr, g.nrbins)] * wW;
            o.x = fmaf(gv.x, d, gv.x) + q * xv.x;
            o.y = fmaf(gv.y, d, gv.y) + q * xv.y;
        }
        reinterpret_cast<float2*>(xbar)[m] = o;
    }
}

// ------------------------------------------------------------------ launchers
// Few tasks (fewer than four per SM): a block of NW warps per task.  The final
// subdivision is recomputed with the block-cooperative QAG (the same decisions and
// sums as the forward pass's block kernel) or read back; its intervals are dealt out
// to the warps, each warp scatters into its own copy of the row cotangents, and the
// copies are summed before the transposed spline solve.
// Shared memory: Gk61Nodes | knots, row, coef, seg_poly [5 ld] | QagList | QagBlockSmem | per warp
// ybar[ld], cbar[ld] | mbarrier
size_t dnu_adj_blk_smem(int ld, int nw) {
    return ((sizeof(Gk61Nodes) + 15) & ~size_t(15)) + 5 * sizeof(double) * ld + ((sizeof(QagList) + 15) & ~size_t(15)) +
           ((sizeof(QagBlockSmem) + 15) & ~size_t(15)) + (size_t)nw * 2 * sizeof(double) * ld + 16;
}

__global__ void __launch_bounds__(128) k_dnu_adj_blk(IntegratorDev I, DnuAdjArgs A, int nk, int Na, int nspec,
                                                     int4 spec_ids) {
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ double s_red[4];
    Gk61Nodes& N = *reinterpret_cast<Gk61Nodes*>(sm);
    size_t off = (sizeof(Gk61Nodes) + 15) & ~size_t(15);
    double* knots = reinterpret_cast<double*>(sm + off);
    double* row = knots + I.ld;
    double* rc = row + I.ld;
    double* sb = rc + I.ld;
    double* sd = sb + I.ld;
    off += 5 * sizeof(double) * I.ld;
    QagList& L = *reinterpret_cast<QagList*>(sm + off);
    off += (sizeof(QagList) + 15) & ~size_t(15);
    QagBlockSmem& sh = *reinterpret_cast<QagBlockSmem*>(sm + off);
    off += (sizeof(QagBlockSmem) + 15) & ~size_t(15);
    const int tid = threadIdx.x, nw = blockDim.x >> 5, warp = tid >> 5, lane = tid & 31;
    double* wy = reinterpret_cast<double*>(sm + off);  // [nw][ld]
    double* wc = wy + (size_t)nw * I.ld;                // [nw][ld]
    off += (size_t)nw * 2 * sizeof(double) * I.ld;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + off);
    gk61_fill(N, tid, blockDim.x);
    for (int i = tid; i < Na; i += blockDim.x) knots[i] = I.scalefact[i];
    if (tid == 0) ptx::mbar_init(bar, 1);
    ptx::mbar_init_fence();
    __syncthreads();
    const Background* B = I.B;
    const StepScalars& S = *I.sc;
    const unsigned row_bytes = (unsigned)(((Na + 1) & ~1) * sizeof(double));
    unsigned phase = 0;
    for (int task = blockIdx.x; task < nspec * nk; task += gridDim.x) {
        const int si = task / nk, ik = task % nk;
        const int mi = si == 0 ? spec_ids.x : (si == 1 ? spec_ids.y : spec_ids.z);
        const double mnu = B->mnu_J[mi];
        const double mnubykT = mnu / B->kBtnu;
        const double k = I.wavenum[ik];
        const double sbar = A.dnu_bar[ik] * S.omeganu[mi] / S.Omega_nu_tot;
        if (sbar == 0.0) continue;  // block-uniform
        double mder = 0.0;
        // initial-condition piece (delta_tot_table.c:525-535)
        if (tid == 0 && mnubykT > 0) {
            const double x0 = k * S.fsl_A0a / mnubykT;
            mder += sbar * specialJ_fit_deriv(x0) * (-x0 / mnu) * I.nu_init[ik] * (1. + S.deriv_prefac * S.fsl_A0a);
        }
        const bool integrate = !S.skip_integral && Na > 1 && mnubykT > 0;
        if (integrate) {
            __syncthreads();  // the previous task's readers of row / rc / wy / wc are done
            if (tid == 0) {
                ptx::fence_async_smem();
                ptx::mbar_expect_tx(bar, Na > 2 ? 2 * row_bytes : row_bytes);
                ptx::bulk_g2s(row, I.dtot + (size_t)ik * I.ld, row_bytes, bar);
                if (Na > 2) ptx::bulk_g2s(rc, I.coef + (size_t)ik * I.ld, row_bytes, bar);
            }
            for (int i = tid; i < nw * I.ld; i += blockDim.x) {
                wy[i] = 0.0;
                wc[i] = 0.0;
            }
            const bool got = __syncthreads_and(ptx::mbar_wait_bounded(bar, phase));  // block-uniform
            phase ^= 1;
            if (!got) {
                if (tid == 0) atomicOr(I.status, kStTimeout);
                ptx::mbar_wait_bounded(bar, phase ^ 1);
                return;
            }
            const KnotSeg ks{I.knot_invh, I.knot_h3, I.knot_ih3};
            if (Na > 2) seg_poly(row, rc, Na, ks, sb, sd, tid, blockDim.x);
            __syncthreads();
            const double qc = S.partnu_now > 0 ? B->vcrit * mnubykT : 0.0;
            int nint;
            const double* iv = nullptr;
            if (!A.recompute && A.ivals) {
                nint = A.nivals[(size_t)mi * I.nk_alloc + ik];
                iv = A.ivals + ((size_t)mi * I.nk_alloc + ik) * kQagLimit * 2;
            } else {
                const DnuIntegrandC f = dnu_integrand(I, S, k, mnubykT, qc, knots, row, rc, sb, sd, Na);
                const QagResult r = qag_block_c(f, N, L, S.loga0, S.loga, 0.0, S.relerr, kQagLimit, sh);
                nint = r.nint;
            }
            __syncthreads();
            const DnuIntegrandC fi = dnu_integrand(I, S, k, mnubykT, qc, knots, row, rc, sb, sd, Na);
            const double ckm = -sbar * S.prefac * fi.k_over_m / mnu;
            double* yb = wy + (size_t)warp * I.ld;
            double* cb = wc + (size_t)warp * I.ld;
            for (int q = warp; q < nint; q += nw)
                adj_interval(fi, N, knots, row, rc, Na, qc, iv ? iv[2 * q] : L.a[q], iv ? iv[2 * q + 1] : L.b[q],
                             S.loga0, S.loga, I.nc_slots, ckm, yb, cb, mder, lane);
            __syncthreads();
            for (int j = tid; j < Na; j += blockDim.x) {
                double y = wy[j], c = wc[j];
                for (int w = 1; w < nw; w++) {
                    y += wy[(size_t)w * I.ld + j];
                    c += wc[(size_t)w * I.ld + j];
                }
                wy[j] = y;
                wc[j] = c;
            }
            __syncthreads();
            const int m = Na - 2;
            if (warp == 0 && Na > 2) spline_solve_scan(I, m, wc);
            __syncthreads();
            const double* ih = I.knot_invh;
            for (int j = tid; j < Na; j += blockDim.x) {  // column Na-1: the provisional row
                double v = wy[j];
                if (Na > 2) {
                    if (j >= 2 && j <= m + 1) v += 3 * wc[j - 1] * ih[j - 1];
                    if (j >= 1 && j <= m) v -= 3 * wc[j] * (ih[j - 1] + ih[j]);
                    if (j < m) v += 3 * wc[j + 1] * ih[j];
                }
                atomicAdd(&A.Dbar[(size_t)ik * I.ld + j], S.prefac * sbar * v);
            }
        }
        mder = warp_sum_to0(mder);
        if (lane == 0) s_red[warp] = mder;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int w = 0; w < nw; w++) t += s_red[w];
            if (t != 0.0) atomicAdd(&A.mbar[mi], t);
        }
        __syncthreads();
    }
}

size_t dnu_adj_smem(int ld, int wpb) {
    return ((sizeof(Gk61Nodes) + 15) & ~size_t(15)) + sizeof(double) * ld +
           wpb * (sizeof(QagList) + 6 * sizeof(double) * ld) + wpb * sizeof(uint64_t);
}

static int sm_count_a() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

void launch_adj_reduce(const GridGeom& gg, CorrTable corr, float lnscale, const float* gbar, const float* x,
                       double* node_sum, cudaStream_t st) {
    GridArgs a = make_grid_args(gg, corr.nk, lnscale);
    const bool aligned = ((reinterpret_cast<uintptr_t>(gbar) | reinterpret_cast<uintptr_t>(x)) & 15) == 0;
    if (aligned && corr.nk >= 2) {
        const long long nchunks = (gg.nmodes + 7) / 8;
        long long blocks = (nchunks + 255) / 256;
        if (blocks > 4LL * sm_count_a()) blocks = 4LL * sm_count_a();
        if (blocks < 1) blocks = 1;
        const long long adv = blocks * 256 * 8;  // modes per grid stride
        const int nz = gg.N / 2 + 1;
        const size_t smem = sizeof(float) * corr.nk * (1 + 8);
        cudaFuncSetAttribute(k_adj_reduce8, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        const long long adv_rows = adv / nz;
        k_adj_reduce8<<<(int)blocks, 256, smem, st>>>(a, corr, gbar, x, node_sum, nchunks, (int)(adv_rows / gg.N),
                                                      (int)(adv_rows % gg.N), (int)(adv % nz));
        return;
    }
    const size_t smem = sizeof(double) * corr.nk + sizeof(int) * (2 * gg.nrbins + 1) + sizeof(float) * 3 * corr.nk + 64;
    cudaFuncSetAttribute(k_adj_reduce_plain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    long long blocks = (gg.nmodes + 255) / 256;
    if (blocks > 4LL * sm_count_a()) blocks = 4LL * sm_count_a();
    k_adj_reduce_plain<<<(int)(blocks > 0 ? blocks : 1), 256, smem, st>>>(a, gg.thresh, gg.cmap, corr, gbar, x,
                                                                          node_sum);
}

void launch_adj_bins(const AdjBinsHost& h, cudaStream_t st) {
    AdjBins A{h.node_sum, h.pnu_bar, h.dnu, h.dcdm, h.power, h.count, h.compact, h.F0sq, h.dnu_bar, h.dprov_bar,
              h.rbar, h.Q, h.dc_sum, h.norm, h.L3, h.fcdm, h.ld};
    k_adj_bins<<<(h.nk + 127) / 128, 128, 0, st>>>(A, h.nk);
}

void launch_adj_bins2(const AdjBinsHost& h, cudaStream_t st) {
    AdjBins A{h.node_sum, h.pnu_bar, h.dnu, h.dcdm, h.power, h.count, h.compact, h.F0sq, h.dnu_bar, h.dprov_bar,
              h.rbar, h.Q, h.dc_sum, h.norm, h.L3, h.fcdm, h.ld};
    k_adj_bins2<<<1, 256, 0, st>>>(A, h.nk);
}

void launch_dnu_adj(const IntegratorDev& I, const double* dnu_bar, double* Dbar, double* mbar, const double* ivals,
                    const int* nivals, int recompute, int nk, int Na, int nspec, const int* spec_ids, int wpb,
                    cudaStream_t st) {
    DnuAdjArgs A{dnu_bar, Dbar, mbar, ivals, nivals, recompute};
    wpb = wpb < 1 ? 1 : (wpb > 4 ? 4 : wpb);
    while (wpb > 1 && dnu_adj_smem(I.ld, wpb) > 227 * 1024 - 256) wpb--;
    const size_t smem = dnu_adj_smem(I.ld, wpb);
    static bool attr = false;
    if (!attr) {
        raise_dynamic_smem_limit(reinterpret_cast<const void*>(k_dnu_adj));
        attr = true;
    }
    const int ntask = nspec * nk;
    if (ntask <= 0) return;
    const size_t bsmem = dnu_adj_blk_smem(I.ld, 4);
    if (ntask < 4 * sm_count_a() && bsmem <= 227 * 1024 - 256) {
        static bool blk_attr = false;
        if (!blk_attr) {
            raise_dynamic_smem_limit(reinterpret_cast<const void*>(k_dnu_adj_blk));
            blk_attr = true;
        }
        k_dnu_adj_blk<<<ntask, 128, bsmem, st>>>(I, A, nk, Na, nspec,
                                                 make_int4(spec_ids[0], spec_ids[1], spec_ids[2], 0));
        return;
    }
    k_dnu_adj<<<(ntask + wpb - 1) / wpb, 32 * wpb, smem, st>>>(I, A, nk, Na, nspec,
                                                               make_int4(spec_ids[0], spec_ids[1], spec_ids[2], 0));
}

void launch_adj_grid(const GridGeom& gg, CorrTable corr, float lnscale, const float* gbar, const float* x, float* xbar,
                     const double* Q, const double* dc_sum, const double* F0sq, cudaStream_t st) {
    GridArgs a = make_grid_args(gg, corr.nk, lnscale);
    const size_t smem = sizeof(int) * (2 * gg.nrbins + 1) + sizeof(float) * (3 * corr.nk + a.nz + gg.nrbins) + 64;
    cudaFuncSetAttribute(k_adj_grid_plain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    long long blocks = (gg.nmodes + 255) / 256;
    if (blocks > 8LL * sm_count_a()) blocks = 8LL * sm_count_a();
    k_adj_grid_plain<<<(int)(blocks > 0 ? blocks : 1), 256, smem, st>>>(a, gg.thresh, gg.cmap, gg.w1, corr, gbar, x,
                                                                        xbar, Q, dc_sum, F0sq);
}

}  // namespace ksp
