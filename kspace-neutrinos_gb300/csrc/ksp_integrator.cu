// ksp_integrator.cu -- the linear-response neutrino integrator on the GPU.
//
//   k_rho_points / k_spline1    Omega_nu(a) tables (omega_nu_single.c:117-153)
//   k_nufrac_low                hybrid-neutrino fractions (omega_nu_single.c:214-240)
//   k_update_row                update_delta_tot (delta_tot_table.c:177-191)
//   k_delta_tot_init            delta_tot_init's per-bin part (delta_tot_table.c:94-129)
//   k_scalars                   per-call scalars + factorised knot spline system
//   k_fs_segments/k_fs_finish   the fslength table (delta_tot_table.c:574-591): a
//                               cumulative fixed-order Gauss-Legendre sum over the 16*Na
//                               uniform nodes replaces 16*Na adaptive integrals; spline
//                               coefficients by the closed-form inverse of tridiag(1,4,1)
//   k_nc_build                  the integrand's bin-independent terms on QAG's right spine
//   k_dtot_coeffs               natural spline of every history row (shared knots); in a
//                               prepared step also the binning pass's normalisation and
//                               the provisional row
//   k_dnu_qag                   one warp per (species, bin): history row staged into
//                               shared memory by a TMA bulk copy, then QAG/GK61 of the
//                               delta_nu time integral (delta_tot_table.c:492-500,592-599)
//   k_dnu_qag_blk               the same with a block per task (few tasks), one bisection
//                               level evaluated ahead
//   k_combine / k_finish        species sum, row commit, NaN check, clamp, ratio table
#include <cuda_runtime.h>
#include <stdio.h>
#include "ksp_internal.h"
#include "ksp_ptx.cuh"

namespace ksp {

// ------------------------------------------------------------------ background tables
struct RhoIntegrand {  // omega_nu_single.c:89-96
    double amnu, kT;
    __device__ double operator()(double q) const {
        const double epsilon = sqrt(q * q + amnu * amnu);
        const double f0 = 1. / (exp(q / kT) + 1);
        return q * q * epsilon * f0;
    }
};

// one warp per (species, table point): rhonu[i] = qag(...)/a^4 * conversion
__global__ void k_rho_points(Background* B, unsigned* status) {
    __shared__ Gk61Nodes N;
    extern __shared__ unsigned char smraw[];
    QagList* lists = reinterpret_cast<QagList*>(smraw);
    gk61_fill(N, threadIdx.x, blockDim.x);
    __syncthreads();
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int task = blockIdx.x * nw + warp;
    const int s = task / kNRhoTab, i = task % kNRhoTab;
    if (s >= kNuSpecies) return;
    RhoTable& T = B->tab[s];
    if (!B->deg[s] || !T.has_table) return;
    RhoIntegrand f{T.mnu * exp(T.loga[i]), B->kBtnu};
    QagResult r = qag_warp(f, N, lists[warp], 0.0, 500 * B->kBtnu, 0.0, 1e-9, kQagLimit);
    if ((threadIdx.x & 31) == 0) {
        const double ea = exp(T.loga[i]);
        T.rhonu[i] = r.result / (ea * ea * ea * ea) * B->conv;
        if (!r.ok) atomicOr(status, kStGsl);
    }
}

__global__ void k_rho_splines(Background* B, double* scratch) {
    const int s = threadIdx.x;
    if (s >= kNuSpecies) return;
    RhoTable& T = B->tab[s];
    T.imnu = 1.0 / T.mnu;
    if (!B->deg[s] || !T.has_table) return;
    natural_spline_coeffs(T.loga, T.rhonu, kNRhoTab, T.c, scratch + s * 2 * kNRhoTab);
    // the node-independent terms of cspline_seg, per segment
    for (int i = 0; i + 1 < kNRhoTab; i++) {
        const double h = T.loga[i + 1] - T.loga[i];
        T.sb[i] = (T.rhonu[i + 1] - T.rhonu[i]) / h - h * (T.c[i + 1] + 2.0 * T.c[i]) / 3.0;
        T.sd[i] = (T.c[i + 1] - T.c[i]) / (3.0 * h);
    }
    T.inv_dx = (kNRhoTab - 1) / (T.loga[kNRhoTab - 1] - T.loga[0]);
}

void launch_background_tables(Background* dB, double a0, cudaStream_t st, unsigned* status) {
    (void)a0;
    const int warps = 4;
    const int tasks = kNuSpecies * kNRhoTab;
    k_rho_points<<<(tasks + warps - 1) / warps, 32 * warps, warps * sizeof(QagList), st>>>(dB, status);
    double* scratch = nullptr;
    cudaMallocAsync(&scratch, sizeof(double) * 2 * kNRhoTab * kNuSpecies, st);
    k_rho_splines<<<1, 32, 0, st>>>(dB, scratch);
    cudaFreeAsync(scratch, st);
}

// Natural cubic spline of log H on n uniform knots (spacing h), as per-segment
// polynomial coefficients (y_i, b_i, c_i, d_i): one thread (a one-time set-up).
__global__ void k_hubble_table(const double* H, int n, double h, double* coef, double* m) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    // second derivatives: m[i-1] + 4 m[i] + m[i+1] = 6 (y[i+1] - 2 y[i] + y[i-1]) / h^2,
    // m[0] = m[n-1] = 0 (Thomas algorithm; coef[4i+1] holds the modified diagonal ratio)
    double* cp = coef;  // scratch for the forward sweep, overwritten below
    m[0] = 0;
    m[n - 1] = 0;
    double prev_c = 0, prev_d = 0;
    for (int i = 1; i < n - 1; i++) {
        const double r = 6.0 * (log(H[i + 1]) - 2.0 * log(H[i]) + log(H[i - 1])) / (h * h);
        const double den = 4.0 - prev_c;
        const double ci = 1.0 / den;
        const double di = (r - prev_d) / den;
        cp[4 * i] = ci;
        cp[4 * i + 1] = di;
        prev_c = ci;
        prev_d = di;
    }
    for (int i = n - 2; i >= 1; i--) m[i] = cp[4 * i + 1] - cp[4 * i] * m[i + 1];
    for (int i = 0; i < n - 1; i++) {
        const double y0 = log(H[i]), y1 = log(H[i + 1]);
        coef[4 * i] = y0;
        coef[4 * i + 1] = (y1 - y0) / h - h * (2.0 * m[i] + m[i + 1]) / 6.0;
        coef[4 * i + 2] = 0.5 * m[i];
        coef[4 * i + 3] = (m[i + 1] - m[i]) / (6.0 * h);
    }
}
void launch_hubble_table(const double* H, int n, double h, double* coef, double* scratch, cudaStream_t st) {
    k_hubble_table<<<1, 32, 0, st>>>(H, n, h, coef, scratch);
}

__global__ void k_spline1(const double* x, const double* y, double* c, double* scratch, int n) {
    if (threadIdx.x == 0 && blockIdx.x == 0) natural_spline_coeffs(x, y, n, c, scratch);
}
void launch_spline_coeffs_1thread(const double* x, const double* y, double* c, double* scratch, int n,
                                  cudaStream_t st) {
    k_spline1<<<1, 32, 0, st>>>(x, y, c, scratch, n);
}

struct FermiDirac {  // omega_nu_single.c:207-210
    __device__ double operator()(double x) const { return x * x / (exp(x) + 1); }
};

// omega_nu_single.c:214-228 (qag limit 100) and :230-240
__global__ void k_nufrac_low(Background* B, double light, double vcrit, unsigned* status) {
    __shared__ Gk61Nodes N;
    __shared__ QagList L[kNuSpecies];
    gk61_fill(N, threadIdx.x, blockDim.x);
    __syncthreads();
    const int s = threadIdx.x >> 5;
    if (s >= kNuSpecies) return;
    const double qc = B->mnu[s] * vcrit / light / B->kBtnu;
    QagResult r = qag_warp(FermiDirac{}, N, L[s], 0.0, qc, 0.0, 1e-6, 100);
    if ((threadIdx.x & 31) == 0) {
        B->nufrac_low[s] = r.result / (1.5 * kZeta3);
        if (!r.ok) atomicOr(status, kStGsl);
    }
}
void launch_nufrac_low(Background* dB, double light, double vcrit, cudaStream_t st, unsigned* status) {
    k_nufrac_low<<<1, 32 * kNuSpecies, 0, st>>>(dB, light, vcrit, status);
}

// nufrac_low(qc) of n momenta (omega_nu_single.c:214-228): a warp per value
__global__ void k_nufrac_low_values(const double* qc, int n, double* out, unsigned* status) {
    __shared__ Gk61Nodes N;
    __shared__ QagList L[4];
    gk61_fill(N, threadIdx.x, blockDim.x);
    __syncthreads();
    const int w = threadIdx.x >> 5;
    const int i = blockIdx.x * 4 + w;
    if (i >= n) return;
    QagResult r = qag_warp(FermiDirac{}, N, L[w], 0.0, qc[i], 0.0, 1e-6, 100);
    if ((threadIdx.x & 31) == 0) {
        out[i] = r.result / (1.5 * kZeta3);
        if (!r.ok) atomicOr(status, kStGsl);
    }
}
void launch_nufrac_low_values(const double* qc, int n, double* out, unsigned* status, cudaStream_t st) {
    if (n > 0) k_nufrac_low_values<<<(n + 3) / 4, 128, 0, st>>>(qc, n, out, status);
}

// specialJ of n arguments (the device function the integrator uses)
__global__ void k_special_j(const double* x, int n, double qc, double nfl, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = specialJ(x[i], qc, nfl);
}
void launch_special_j(const double* x, int n, double qc, double nufrac_low, double* out, cudaStream_t st) {
    if (n > 0) k_special_j<<<(n + 127) / 128, 128, 0, st>>>(x, n, qc, nufrac_low, out);
}

// ------------------------------------------------------------------ history rows
// delta_tot_table.c:177-191: row `row` = get_delta_tot(dnu, dcdm) at a
__global__ void k_update_row(IntegratorDev I, int nk, int row, double a, double loga, const double* dcdm,
                             const double* dnu) {
    __shared__ double s3[3];
    const Background& B = *I.B;
    if (threadIdx.x == 0) {
        s3[0] = omega_nu_nopart(B, a) * (a * a * a);
        s3[1] = omega_nu(B, 1);
        s3[2] = particle_nu_fraction(B, a, 0);
        if (blockIdx.x == 0) I.scalefact[row] = loga;
    }
    __syncthreads();
    const double Omeganonu = I.sc->Omeganonu;
    for (int ik = blockIdx.x * blockDim.x + threadIdx.x; ik < nk; ik += gridDim.x * blockDim.x)
        I.dtot[(size_t)ik * I.ld + row] = get_delta_tot(dnu[ik], dcdm[ik], s3[0], Omeganonu, s3[1], s3[2]);
}
void launch_update_row(const IntegratorDev& I, int nk, int row, double a, double loga, const double* dcdm,
                       const double* dnu, cudaStream_t st) {
    k_update_row<<<(nk + 255) / 256, 256, 0, st>>>(I, nk, row, a, loga, dcdm, dnu);
}

// the same row from the call's scalars (after k_scalars), delta_nu_last and delta_cdm
__global__ void k_update_row_s(IntegratorDev I, int nk, int row) {
    const StepScalars& S = *I.sc;
    for (int ik = blockIdx.x * blockDim.x + threadIdx.x; ik < nk; ik += gridDim.x * blockDim.x)
        I.dtot[(size_t)ik * I.ld + row] =
            get_delta_tot(I.nu_last[ik], I.dcdm[ik], S.OmegaNua3, S.Omeganonu, S.OmegaNu1, S.partnu);
}
void launch_update_row_scalars(const IntegratorDev& I, int nk, int row, cudaStream_t st) {
    k_update_row_s<<<(nk + 255) / 256, 256, 0, st>>>(I, nk, row);
}

// delta_tot_table.c:94-129: transfer spline, first row (fresh start), delta_nu_init
__global__ void k_delta_tot_init(IntegratorDev I, int nk, const double* wavenum, const double* dcdm, int fresh,
                                 double TimeTransfer) {
    __shared__ double s4[4];
    const Background& B = *I.B;
    if (threadIdx.x == 0) {
        s4[0] = omega_nu_nopart(B, TimeTransfer) * (TimeTransfer * TimeTransfer * TimeTransfer);
        s4[1] = omega_nu(B, 1);
        s4[2] = particle_nu_fraction(B, TimeTransfer, 0);
        s4[3] = I.sc->Omeganonu;
        // k beyond the transfer table (delta_tot_table.c:113-114)
        if (log(wavenum[nk - 1]) > I.t_logk[I.ntrans - 1]) atomicOr(I.status, kStKmax);
    }
    __syncthreads();
    const double OmegaNua3 = s4[0], OmegaNu1 = s4[1], Omeganonu = s4[3];
    const double OmegaMa = Omeganonu + OmegaNua3;
    for (int ik = blockIdx.x * blockDim.x + threadIdx.x; ik < nk; ik += gridDim.x * blockDim.x) {
        const double lk = log(wavenum[ik]);
        double T;
        if (lk < I.t_logk[0] || lk > I.t_logk[I.ntrans - 1]) {
            atomicOr(I.status, kStGsl);  // GSL interpolation domain error -> 2001
            T = 0;
        } else {
            const int i = seg_bsearch(I.t_logk, I.ntrans, lk);
            T = cspline_seg(I.t_logk, I.t_T, I.t_c, i, lk);
        }
        double* row = I.dtot + (size_t)ik * I.ld;
        if (fresh) row[0] = get_delta_tot(dcdm[ik] * T, dcdm[ik], OmegaNua3, Omeganonu, OmegaNu1, s4[2]);
        I.nu_init[ik] = row[0] * OmegaMa / (OmegaMa - OmegaNua3 + T * OmegaNua3) * fabs(T);
        I.wavenum[ik] = wavenum[ik];
    }
}
void launch_delta_tot_init(const IntegratorDev& I, int nk, const double* wavenum, const double* dcdm, int fresh,
                           double TimeTransfer, cudaStream_t st) {
    k_delta_tot_init<<<(nk + 255) / 256, 256, 0, st>>>(I, nk, wavenum, dcdm, fresh, TimeTransfer);
}

// ------------------------------------------------------------------ per-call scalars
// Scalars of the call and the factorised natural-spline system of the history knots
// x = scalefact[0..Na-1] (shared by every row).  Rows below `start_row` were factorised
// by an earlier call with the same leading knots and are kept.  Reciprocals are stored
// so the per-row sweeps need no divisions.
__global__ void k_scalars(IntegratorDev I, int Na, double a, double loga, double loga0, double TimeTransfer,
                          int start_row, int write_knot) {
    if (threadIdx.x == 0) {  // this call's QAG statistics start from zero
        *I.qag_max = 0;
        *I.qag_total = 0;
    }
    if (write_knot) {  // the provisional knot (update_row writes the same value)
        if (threadIdx.x == 0) I.scalefact[Na - 1] = loga;
        __syncthreads();
    }
    const double* xk = I.scalefact;
    for (int i = threadIdx.x; i + 1 < Na; i += blockDim.x) {
        const double h = xk[i + 1] - xk[i];
        I.knot_invh[i] = 1.0 / h;
        I.knot_h3[i] = h / 3.0;
        I.knot_ih3[i] = 1.0 / (3.0 * h);
    }
    if (threadIdx.x < 32) call_scalars_warp(*I.B, a, loga, loga0, TimeTransfer, Na, *I.sc);
    if (threadIdx.x != 0) return;
    const double* x = I.scalefact;
    if (Na > 2) {
        const int m = Na - 2;
        for (int i = start_row < 0 ? 0 : start_row; i < m; i++) {
            const double h0 = x[i + 1] - x[i], h1 = x[i + 2] - x[i + 1];
            double d = 2.0 * (h0 + h1);
            if (i > 0) {
                const double f = h0 * I.knot_invdiag[i - 1];
                d -= f * h0;
                I.knot_fac[i] = f;
            }
            I.knot_invdiag[i] = 1.0 / d;
        }
    }
}

// ------------------------------------------------------------------ fslength table
struct GL4 { double x[2], w[2]; };  // positive half of the 4-point Gauss-Legendre rule

struct FslIntegrand {  // delta_tot_table.c:378-383
    const Background* B;
    __device__ double operator()(double loga) const { return fsl_integrand(*B, loga); }
};

// The segment integrals of the fslength table, 4 lanes per group (fs_group_eval).
__global__ void k_fs_segments(IntegratorDev I, int Nfs, double loga0, double loga, GL4 gl, int npts, int ngroups) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    fs_group_eval(*I.B, Nfs, loga0, loga, npts, gt >> 2, gt & 3, (gt >> 2) < ngroups, gl.x, gl.w, I.fs_x, I.fs_seg);
}

// One block: suffix sums of the segment integrals -> fslength at every node.
__global__ void k_fs_finish(IntegratorDev I, int Nfs) {
    __shared__ double warp_tot[32];
    const int t = threadIdx.x, nt = blockDim.x, lane = t & 31, w = t >> 5;
    const int per = (Nfs + nt - 1) / nt;
    const int i0 = t * per, i1 = min(Nfs, i0 + per);
    double loc = 0;
    for (int i = i1 - 1; i >= i0; i--) loc += I.fs_seg[i];
    // inclusive suffix scan over the threads of a warp, then over warps
    double v = loc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double n = __shfl_down_sync(0xffffffffu, v, o);
        if (lane + o < 32) v += n;
    }
    if (lane == 0) warp_tot[w] = v;
    __syncthreads();
    if (w == 0) {
        const int nwarps = nt >> 5;
        double u = lane < nwarps ? warp_tot[lane] : 0.0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double n = __shfl_down_sync(0xffffffffu, u, o);
            if (lane + o < 32) u += n;
        }
        if (lane < nwarps) warp_tot[lane] = u;  // inclusive suffix over warps
    }
    __syncthreads();
    const double later_warps = (w + 1 < (nt >> 5)) ? warp_tot[w + 1] : 0.0;
    double run = v - loc + later_warps;  // exclusive suffix of this thread's chunk
    const double light = I.sc->light;
    for (int i = i1 - 1; i >= i0; i--) {
        run += I.fs_seg[i];
        I.fs_y[i] = light * run;  // fslength(x_i, log a)
    }
    __syncthreads();
    if (t == 0) {
        I.sc->fsl_A0a = I.fs_y[0];
        I.sc->Nfs = Nfs;
        I.fs_c[0] = 0.0;
        I.fs_c[Nfs - 1] = 0.0;
    }
}

// Natural-spline coefficients of the (uniformly spaced) fslength table, one thread per
// unknown.  The system is tridiag(1,4,1) c = 3 D^2 y / h^2 with known inverse: for
// mu = 2 - sqrt(3) and 1-based i <= j,
//   (T^-1)_{ij} = (-1)^{i+j} mu^{j-i} (1-mu^{2i}) (1-mu^{2(m+1-j)}) / (2 sqrt3 (1-mu^{2(m+1)})).
// Terms with |i-j| > 40 are below 1e-22 relative and dropped.  (Fully parallel: a single
// table is solved faster this way than by one warp's substitution, whose loads are
// serial; the batch path, with thousands of tables, uses uniform_spline_warp.)
__global__ void k_fs_coeffs(IntegratorDev I, int Nfs, double loga0, double loga) {
    __shared__ double mupow[82];
    for (int e = threadIdx.x; e < 82; e += blockDim.x) {  // any block size
        const double mu = 2.0 - sqrt(3.0);
        double p = 1.0;
        for (int k = 0; k < e; k++) p *= mu;
        mupow[e] = p;
    }
    __syncthreads();
    const int m = Nfs - 2;
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= m) return;
    const double h = (loga - loga0) / (Nfs - 1.);
    const double scale = 3.0 / (h * h) / (2.0 * sqrt(3.0));
    const double D = (2 * (m + 1) < 82) ? 1.0 - mupow[2 * (m + 1)] : 1.0;
    const double* y = I.fs_y;
    double acc = 0;
    const int vlo = max(0, u - 40), vhi = min(m - 1, u + 40);
    for (int v = vlo; v <= vhi; v++) {
        const int d = v > u ? v - u : u - v;
        const int lo1 = min(u, v) + 1, hi1 = max(u, v) + 1;
        const double A = (2 * lo1 < 82) ? 1.0 - mupow[2 * lo1] : 1.0;
        const int e2 = 2 * (m + 1 - hi1);
        const double Bf = (e2 < 82) ? 1.0 - mupow[e2] : 1.0;
        const double r = __ldg(y + v + 2) - 2.0 * __ldg(y + v + 1) + __ldg(y + v);
        acc += ((d & 1) ? -mupow[d] : mupow[d]) * A * Bf * r;
    }
    I.fs_c[u + 1] = acc * scale / D;
}

// ------------------------------------------------------------------ history splines
// Forward/back substitution of every history row against the shared factorisation,
// warp per row (warp-parallel affine scans when the row fits in shared memory).
__global__ void k_dtot_coeffs(IntegratorDev I, int nk, int Na, int staged, int update_row, FinalizeArgs fin) {
    extern __shared__ __align__(16) double sdc[];
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double* sy = staged ? sdc + (size_t)warp * 2 * I.ld : nullptr;
    double* sc = staged ? sy + I.ld : nullptr;
    for (int ik = blockIdx.x * nw + warp; ik < nk; ik += gridDim.x * nw) {
        if (fin.active && (threadIdx.x & 31) == 0) finalize_bin(fin, ik);  // this bin's delta_cdm first
        if (update_row >= 0) {  // update_delta_tot (delta_tot_table.c:177-191), as k_update_row
            if ((threadIdx.x & 31) == 0) {
                const StepScalars& S = *I.sc;
                I.dtot[(size_t)ik * I.ld + update_row] =
                    get_delta_tot(I.nu_last[ik], I.dcdm[ik], S.OmegaNua3, S.Omeganonu, S.OmegaNu1, S.partnu);
            }
            __syncwarp();
        }
        if (staged) dtot_row_coeffs_scan(I, ik, Na, sy, sc);
        else dtot_row_coeffs_warp(I, ik, Na, nullptr, nullptr);
    }
}

// ------------------------------------------------------------------ row splines in two parts
// A history row's natural spline is linear in the row, and the provisional (last) knot
// enters the spline system through its last right-hand side only, so
//   c = c_base + (y_new - y_base) c_unit,
// with c_base the coefficients of the row whose last knot is y_base (the knot before it)
// and c_unit those of a unit last knot with all other knots zero.  Both depend only on
// the committed rows and the knots: k_dtot_base solves them beside the binning pass
// (block nk: c_unit).  After it, k_row_update forms y_new (update_delta_tot,
// delta_tot_table.c:177-191) from this step's delta_cdm and adds the correction, in
// place of the solve.  y_new - y_base is one step's growth of delta_tot, so the sum does
// not cancel.
__global__ void k_dtot_base(IntegratorDev I, int nk, int Na) {
    // in place in the coefficient rows (global memory, L1-cached): the binning pass holds
    // nearly all of every SM's shared memory, and these blocks run beside it
    const int lane = threadIdx.x & 31;
    const int m = Na - 2;  // unknowns c[1..m]
    const double* ih = I.knot_invh;
    double* c;
    if (blockIdx.x == nk) {
        c = I.coef_unit;
        for (int u = lane; u < m; u += 32) c[u + 1] = u == m - 1 ? 3.0 * ih[m] : 0.0;
    } else {
        const double* y = I.dtot + (size_t)blockIdx.x * I.ld;
        c = I.coef + (size_t)blockIdx.x * I.ld;
        for (int u = lane; u < m; u += 32) {
            const double y2 = u == m - 1 ? y[m] : y[u + 2];  // the last knot taken equal to the one before
            c[u + 1] = 3.0 * ((y2 - y[u + 1]) * ih[u + 1] - (y[u + 1] - y[u]) * ih[u]);
        }
    }
    __syncwarp();
    spline_solve_scan(I, m, c);
    if (lane == 0) {
        c[0] = 0.0;
        c[Na - 1] = 0.0;
    }
}

// block per bin: this bin's delta_cdm (a deferred normalisation), the provisional row
// `row` = Na - 1, and its spline as c_base + (y_new - y_base) c_unit
__global__ void k_row_update(IntegratorDev I, int nk, int Na, int row, FinalizeArgs fin) {
    __shared__ double s_dy;
    const int ik = blockIdx.x;
    if (threadIdx.x == 0) {
        if (fin.active) finalize_bin(fin, ik);
        const StepScalars& S = *I.sc;
        double* y = I.dtot + (size_t)ik * I.ld;
        const double yn = get_delta_tot(I.nu_last[ik], I.dcdm[ik], S.OmegaNua3, S.Omeganonu, S.OmegaNu1, S.partnu);
        y[row] = yn;
        s_dy = yn - y[Na - 2];
    }
    __syncthreads();
    const double dy = s_dy;
    double* c = I.coef + (size_t)ik * I.ld;
    for (int k = 1 + threadIdx.x; k < Na - 1; k += blockDim.x) c[k] = fma(dy, __ldg(I.coef_unit + k), c[k]);
}

bool launch_dtot_base(const IntegratorDev& I, int nk, int Na, cudaStream_t st) {
    if (Na <= 2 || nk <= 0) return false;
    k_dtot_base<<<nk + 1, 32, 0, st>>>(I, nk, Na);
    return cudaPeekAtLastError() == cudaSuccess;
}

// ------------------------------------------------------------------ node table
// The k-independent terms of the delta_nu integrand at the 61 nodes of the first
// kNcLevels levels of QAG's bisection of [log a0, log a]: thread per (slot, node).
__global__ void k_nc_build(IntegratorDev I, int Na) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= I.nc_slots * 61) return;
    const StepScalars& S = *I.sc;
    const int slot = q / 61, jn = q - 61 * slot;
    double lo, hi;
    nc_interval(slot, S.loga0, S.loga, &lo, &hi);
    const double c = __dmul_rn(0.5, __dadd_rn(lo, hi));
    const double h = __dmul_rn(0.5, __dsub_rn(hi, lo));
    const double XK[31] = KSP_GK61_XK_INIT;  // the abscissae of gk61_fill
    const double xk = jn < 30 ? -XK[jn] : (jn < 60 ? XK[jn - 30] : 0.0);
    const double x = __dadd_rn(c, __dmul_rn(h, xk));
    const double fs_inv = (S.Nfs - 1.) / (S.loga - S.loga0);
    const NodeTerms t = dnu_node_terms(I.B, I.fs_x, I.fs_y, I.fs_c, S.Nfs, S.loga0, fs_inv, I.scalefact, Na, x);
    I.nc_g[q] = t.g;
    I.nc_fsl[q] = t.fsl;
    I.nc_dx[q] = t.dx;
    I.nc_j[q] = t.j;
}

// ------------------------------------------------------------------ delta_nu integral
// Shared memory per CTA: Gk61Nodes | knots[ld] | per warp: QagList, row[ld], coef[ld], seg_poly [2 ld] |
// mbarriers
__global__ void __launch_bounds__(128) k_dnu_qag(IntegratorDev I, int nk, int Na, int nspec, int4 spec_ids) {
    extern __shared__ __align__(16) unsigned char sm[];
    Gk61Nodes& N = *reinterpret_cast<Gk61Nodes*>(sm);
    size_t off = (sizeof(Gk61Nodes) + 15) & ~size_t(15);
    double* knots = reinterpret_cast<double*>(sm + off);
    off += sizeof(double) * I.ld;
    const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t per_warp = sizeof(QagList) + 4 * sizeof(double) * I.ld;
    unsigned char* wbase = sm + off + warp * per_warp;
    QagList& L = *reinterpret_cast<QagList*>(wbase);
    double* row = reinterpret_cast<double*>(wbase + sizeof(QagList));
    double* rc = row + I.ld;
    double* sb = rc + I.ld;
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
    const int ntask = nspec * nk;
    const unsigned row_bytes = (unsigned)(((Na + 1) & ~1) * sizeof(double));
    unsigned phase = 0;
    int my_max = 0;
    long long my_tot = 0;
    for (int task = blockIdx.x * nw + warp; task < ntask; task += gridDim.x * nw) {
        const int si = task / nk, ik = task % nk;
        const int mi = si == 0 ? spec_ids.x : (si == 1 ? spec_ids.y : spec_ids.z);
        const double k = I.kq ? I.kq[ik] : I.wavenum[ik];
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
            // stage the history row and its spline coefficients (TMA bulk copies)
            __syncwarp();
            if (lane == 0) {
                // order this warp's earlier generic reads of the buffers before the async writes
                ptx::fence_async_smem();
                ptx::mbar_expect_tx(mybar, Na > 2 ? 2 * row_bytes : row_bytes);
                ptx::bulk_g2s(row, I.dtot + (size_t)ik * I.ld, row_bytes, mybar);
                if (Na > 2) ptx::bulk_g2s(rc, I.coef + (size_t)ik * I.ld, row_bytes, mybar);
            }
            const bool got = __all_sync(0xffffffffu, ptx::mbar_wait_bounded(mybar, phase));  // warp-uniform
            phase ^= 1;
            if (!got) {
                if (lane == 0) atomicOr(I.status, kStTimeout);
                // wait (bounded) for the copy still in flight before leaving
                ptx::mbar_wait_bounded(mybar, phase ^ 1);
                return;
            }
            const KnotSeg ks{I.knot_invh, I.knot_h3, I.knot_ih3};
            if (Na > 2) seg_poly(row, rc, Na, ks, sb, sd, lane, 32);
            __syncwarp();
            const double qc = S.partnu_now > 0 ? B->vcrit * mnubykT : 0.0;
            const DnuIntegrandC f = dnu_integrand_pre(I, S, kom, fsi, qc, knots, row, rc, sb, sd, Na);
            QagResult r = qag_warp_c(f, N, L, S.loga0, S.loga, 0.0, S.relerr, kQagLimit);
            integral = r.result;
            if (I.ivals) {  // keep the final subdivision for the adjoint
                double* dst = I.ivals + ((size_t)mi * I.nk_alloc + ik) * kQagLimit * 2;
                for (int q = lane; q < r.nint; q += 32) {
                    dst[2 * q] = L.a[q];
                    dst[2 * q + 1] = L.b[q];
                }
                if (lane == 0) I.nivals[(size_t)mi * I.nk_alloc + ik] = r.nint;
            }
            if (!r.ok && lane == 0) atomicOr(I.status, kStGsl);
            my_max = max(my_max, r.nint);
            my_tot += r.nint;
        }
        if (lane == 0) I.dnu_s[(size_t)mi * I.nk_alloc + ik] = dnu_task_value(I, S, ik, k, mnubykT, integrate, integral);
    }
    if (lane == 0 && my_tot) {
        atomicMax(I.qag_max, my_max);
        atomicAdd(reinterpret_cast<unsigned long long*>(I.qag_total), (unsigned long long)my_tot);
    }
}

// One (species, bin) task per block of 8 warps: the same integral as k_dnu_qag with the
// GK61 nodes of each step spread over the block and one bisection level evaluated ahead
// (qag_block_spec_c: the same decisions, sums equal to the last bits).  For calls with few tasks, where one warp
// per task leaves the SMs' FP64 pipes idle between the long dependent chains of a single
// warp and the sequential QAG rounds set the time.
// SPEC = false: blocks of 4 warps and qag_block_c (no look-ahead).
// Shared memory: Gk61Nodes | knots[ld] | row[ld] | coef[ld] | QagList | QagSpecSmem or QagBlockSmem | mbarrier
template <bool SPEC>
struct QagBlkSmemOf { typedef QagSpecSmem type; };
template <>
struct QagBlkSmemOf<false> { typedef QagBlockSmem type; };

template <bool SPEC>
__global__ void __launch_bounds__(SPEC ? 256 : 128, SPEC ? 2 : 4)
    k_dnu_qag_blk(IntegratorDev I, int nk, int Na, int nspec, int4 spec_ids) {
    typedef typename QagBlkSmemOf<SPEC>::type Smem;
    extern __shared__ __align__(16) unsigned char sm[];
    Gk61Nodes& N = *reinterpret_cast<Gk61Nodes*>(sm);
    size_t off = (sizeof(Gk61Nodes) + 15) & ~size_t(15);
    double* knots = reinterpret_cast<double*>(sm + off);
    off += sizeof(double) * I.ld;
    double* row = reinterpret_cast<double*>(sm + off);
    off += sizeof(double) * I.ld;
    double* rc = reinterpret_cast<double*>(sm + off);
    off += sizeof(double) * I.ld;
    double* sb = reinterpret_cast<double*>(sm + off);
    double* sd = sb + I.ld;
    off += 2 * sizeof(double) * I.ld;
    QagList& L = *reinterpret_cast<QagList*>(sm + off);
    off += (sizeof(QagList) + 15) & ~size_t(15);
    Smem& sh = *reinterpret_cast<Smem*>(sm + off);
    off += (sizeof(Smem) + 15) & ~size_t(15);
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + off);
    __shared__ double s_task[4];  // m/kT, k/(m/kT), (Nfs-1)/(log a - log a0), integrate? of the current task
    const int tid = threadIdx.x;
    const Background* B = I.B;
    const StepScalars& S = *I.sc;
    const int ntask = nspec * nk;
    const unsigned row_bytes = (unsigned)(((Na + 1) & ~1) * sizeof(double));
    // Thread 0 starts a task: the copies of its history row and spline coefficients, then
    // the task's divisions while they land.
    auto start_task = [&](int task) {
        const int si = task / nk, ik = task % nk;
        const int mi = si == 0 ? spec_ids.x : (si == 1 ? spec_ids.y : spec_ids.z);
        const double mnu = B->mnu_J[mi];
        const bool integ = !S.skip_integral && Na > 1 && mnu / B->kBtnu > 0;
        if (integ) {
            ptx::fence_async_smem();
            ptx::mbar_expect_tx(bar, Na > 2 ? 2 * row_bytes : row_bytes);
            ptx::bulk_g2s(row, I.dtot + (size_t)ik * I.ld, row_bytes, bar);
            if (Na > 2) ptx::bulk_g2s(rc, I.coef + (size_t)ik * I.ld, row_bytes, bar);
        }
        const double m = mnu / B->kBtnu;
        s_task[0] = m;
        s_task[1] = (I.kq ? I.kq[ik] : I.wavenum[ik]) / m;
        s_task[2] = (S.Nfs - 1.) / (S.loga - S.loga0);
        s_task[3] = integ ? 1.0 : 0.0;
    };
    // the first task's copies are in flight while the block fills its tables
    if (tid == 0) {
        ptx::mbar_init(bar, 1);
        ptx::mbar_init_fence();
        if (blockIdx.x < ntask) start_task(ntask - 1 - (int)blockIdx.x);
    }
    gk61_fill(N, tid, blockDim.x);
    for (int i = tid; i < Na; i += blockDim.x) knots[i] = I.scalefact[i];
    __syncthreads();
    unsigned phase = 0;
    int my_max = 0;
    long long my_tot = 0;
    // Blocks take the tasks from the last: the high-k bins of the last species, among the
    // deepest QAG subdivisions, start first, and the blocks that wait for a free slot
    // (more tasks than resident blocks) get the shallow low-k bins of the first species.
    for (int task = blockIdx.x; task < ntask; task += gridDim.x) {
        const int si = (ntask - 1 - task) / nk, ik = (ntask - 1 - task) % nk;
        const int mi = si == 0 ? spec_ids.x : (si == 1 ? spec_ids.y : spec_ids.z);
        const double k = I.kq ? I.kq[ik] : I.wavenum[ik];
        if (task != (int)blockIdx.x) {  // later tasks: after the previous task's reads of row / rc
            __syncthreads();
            if (tid == 0) start_task(ntask - 1 - task);
            __syncthreads();
        }
        const double mnubykT = s_task[0];
        double integral = 0;
        const bool integrate = s_task[3] != 0.0;
        if (integrate) {
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
            const DnuIntegrandC f = dnu_integrand_pre(I, S, s_task[1], s_task[2], qc, knots, row, rc, sb, sd, Na);
            QagResult r;
            if constexpr (SPEC) r = qag_block_spec_c(f, N, L, S.loga0, S.loga, 0.0, S.relerr, kQagLimit, sh);
            else r = qag_block_c(f, N, L, S.loga0, S.loga, 0.0, S.relerr, kQagLimit, sh);
            integral = r.result;
            if (I.ivals) {  // keep the final subdivision for the adjoint
                double* dst = I.ivals + ((size_t)mi * I.nk_alloc + ik) * kQagLimit * 2;
                for (int q = tid; q < r.nint; q += blockDim.x) {
                    dst[2 * q] = L.a[q];
                    dst[2 * q + 1] = L.b[q];
                }
                if (tid == 0) I.nivals[(size_t)mi * I.nk_alloc + ik] = r.nint;
            }
            if (!r.ok && tid == 0) atomicOr(I.status, kStGsl);
            my_max = max(my_max, r.nint);
            my_tot += r.nint;
        }
        if (tid == 0) I.dnu_s[(size_t)mi * I.nk_alloc + ik] = dnu_task_value(I, S, ik, k, mnubykT, integrate, integral);
    }
    if (tid == 0 && my_tot) {
        atomicMax(I.qag_max, my_max);
        atomicAdd(reinterpret_cast<unsigned long long*>(I.qag_total), (unsigned long long)my_tot);
    }
}

size_t dnu_qag_blk_smem(int ld, bool spec) {
    return ((sizeof(Gk61Nodes) + 15) & ~size_t(15)) + 5 * sizeof(double) * ld + ((sizeof(QagList) + 15) & ~size_t(15)) +
           (((spec ? sizeof(QagSpecSmem) : sizeof(QagBlockSmem)) + 15) & ~size_t(15)) + sizeof(uint64_t);
}

// delta_tot_table.c:155-170: combine the species
__global__ void k_combine(IntegratorDev I, int nk) {
    const int ik = blockIdx.x * blockDim.x + threadIdx.x;
    if (ik >= nk) return;
    const StepScalars& S = *I.sc;
    double acc = 0;
    for (int mi = 0; mi < kNuSpecies; mi++)
        if (I.B->deg[mi] > 0) acc += I.dnu_s[(size_t)mi * I.nk_alloc + ik] * S.omeganu[mi] / S.Omega_nu_tot;
    I.dnu[ik] = acc;
}

// Gauss-Legendre nodes by Newton iteration on P_n (positive half)
static void gl_nodes(int n, double* X, double* Wt) {
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

// fslength(logai, logaf) = light * int_{logai}^{logaf} dlna / (a^2 H(a)) (delta_tot_table.c:378-407)
// for n intervals, a warp each: the interval is cut into segments of at most 0.01 in
// log a, each integrated with the 8-point Gauss-Legendre rule (the integrand is smooth on
// a scale of ~1 in log a, so the rule error is far below double rounding); lanes take
// segments in turn and the warp sums them.  0 where logai >= logaf, as the reference.
struct GL8 {
    double x[8], w[8];
};
__global__ void k_fslength_values(const Background* B, const double* lai, const double* laf, int n, double light,
                                  GL8 gl, double* out) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (i >= n) return;
    const double a0 = lai[i], a1 = laf[i];
    double acc = 0;
    if (a0 < a1) {
        const int nseg = (int)ceil((a1 - a0) / 0.01);
        const double h = (a1 - a0) / nseg;
        for (int sgi = lane; sgi < nseg; sgi += 32) {
            const double c = a0 + (sgi + 0.5) * h;
            double sseg = 0;
            for (int q = 0; q < 8; q++) {
                const double la = c + 0.5 * h * gl.x[q];
                const double a = exp(la);
                sseg += gl.w[q] / (a * (a * hubble(*B, a, la)));
            }
            acc += 0.5 * h * sseg;
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) out[i] = a0 < a1 ? light * acc : 0.0;
}
void launch_fslength_values(const Background* dB, const double* logai, const double* logaf, int n, double light,
                            double* out, cudaStream_t st) {
    static GL8 gl;
    static bool have = false;
    if (!have) {
        double X[4], Wt[4];  // the positive half; nodes come in +-x pairs
        gl_nodes(8, X, Wt);
        for (int q = 0; q < 4; q++) {
            gl.x[2 * q] = X[q];
            gl.x[2 * q + 1] = -X[q];
            gl.w[2 * q] = gl.w[2 * q + 1] = Wt[q];
        }
        have = true;
    }
    if (n > 0) k_fslength_values<<<(n + 3) / 4, 128, 0, st>>>(dB, logai, logaf, n, light, gl, out);
}
static GL4 gl4_host() {
    GL4 g;
    gl_nodes(4, g.x, g.w);
    return g;
}

size_t dnu_qag_smem(int ld, int wpb) {
    return ((sizeof(Gk61Nodes) + 15) & ~size_t(15)) + sizeof(double) * ld +
           wpb * (sizeof(QagList) + 4 * sizeof(double) * ld) + wpb * sizeof(uint64_t);
}

// The part of a call that does not depend on the current delta_cdm: the scalars and the
// knot factorisation, the fslength table, the node table.  Can run concurrently with
// the binning pass (write_knot = 1 also stores the provisional knot, log a).
void launch_integrator_prepare(const IntegratorDev& I, int Na, double a, double loga, double loga0,
                               double TimeTransfer, int start_row, int write_knot, bool scalars_only,
                               cudaStream_t st) {
    static const GL4 gl = gl4_host();
    k_scalars<<<1, 256, 0, st>>>(I, Na, a, loga, loga0, TimeTransfer, start_row, write_knot);
    if (scalars_only) return;
    // the fslength table (always built: it also gives fslength(log a0, log a))
    const int Nfs = 16 * (Na > 1 ? Na : 1);
    if (loga > loga0) {
        const int npts = fs_rule_points(Nfs, loga0, loga), ngroups = fs_groups(Nfs, loga0, loga);
        const long long threads = 4LL * ngroups;
        k_fs_segments<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(I, Nfs, loga0, loga, gl, npts, ngroups);
        k_fs_finish<<<1, 1024, 0, st>>>(I, Nfs);
        if (Nfs > 2) k_fs_coeffs<<<(Nfs - 2 + 31) / 32, 32, 0, st>>>(I, Nfs, loga0, loga);
    } else {
        cudaMemsetAsync(&I.sc->fsl_A0a, 0, sizeof(double), st);
        cudaMemsetAsync(&I.sc->Nfs, 0, sizeof(int), st);
    }
    if (loga > loga0 && Na > 1 && I.nc_slots > 0)
        k_nc_build<<<(I.nc_slots * 61 + 63) / 64, 64, 0, st>>>(I, Na);
}

// The rest, after the provisional history row: spline coefficients of the rows, the
// integrals, the species sum.
void launch_integrator_rest(const IntegratorDev& I, int nk, int Na, int nspec, const int* spec_ids,
                            int warps_per_block, cudaStream_t st, int qag_split, int update_row, bool defer_combine,
                            const FinalizeArgs* fin, bool base_ready) {
    // a deferred normalisation runs in the row-spline kernel, or on its own without one
    FinalizeArgs fa{};
    if (fin && fin->active) {
        if (Na > 2) fa = *fin;
        else
            launch_finalize_power(fin->bin_sum, fin->F0sq, fin->count, fin->ksum, fin->compact_bins, nk, fin->BoxSize,
                                  fin->power_out, fin->keff_out, fin->dcdm_out, fin->keffphys_out, st);
    }
    if (update_row >= 0 && Na <= 2) {
        launch_update_row_scalars(I, nk, update_row, st);
        update_row = -1;
    }
    if (Na > 2 && base_ready && update_row == Na - 1) {
        k_row_update<<<nk, 128, 0, st>>>(I, nk, Na, update_row, fa);
    } else if (Na > 2) {
        static bool dc_attr = false;
        if (!dc_attr) {
            raise_dynamic_smem_limit(reinterpret_cast<const void*>(k_dtot_coeffs));
            dc_attr = true;
        }
        // a warp (one row at a time) per block: the latency-bound solves spread over SMs
        const size_t smem = 2 * sizeof(double) * I.ld;
        const int staged = smem <= 200 * 1024;
        k_dtot_coeffs<<<nk, 32, staged ? smem : 0, st>>>(I, nk, Na, staged, update_row, fa);
    }
    int wpb = warps_per_block < 1 ? 1 : (warps_per_block > 4 ? 4 : warps_per_block);
    while (wpb > 1 && dnu_qag_smem(I.ld, wpb) > 227 * 1024 - 256) wpb--;
    const size_t smem = dnu_qag_smem(I.ld, wpb);
    static bool attr_set = false;
    if (!attr_set) {
        raise_dynamic_smem_limit(reinterpret_cast<const void*>(k_dnu_qag));
        attr_set = true;
    }
    const int ntask = nspec * nk;
    if (ntask > 0) {
        static int nsm = 0;
        if (!nsm) {
            int dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
            if (nsm <= 0) nsm = 1;
        }
        // a block per task: 8 warps with look-ahead (split 8) below 4 tasks per SM, 4 warps
        // without up to 6 tasks per SM, 2 warps from there (at 128 registers a thread, 4
        // blocks of 4 warps fit an SM: 1221 tasks of 3 species x 407 bins take two waves
        // of 4-warp blocks and one of 2-warp blocks, measured 0.211 against 0.223 ms; a
        // warp per task, split 1, 0.231 ms)
        const int split = qag_split > 0 ? qag_split : (ntask < 4 * nsm ? 8 : (ntask < 6 * nsm ? 4 : 2));
        const bool spec = split >= 8;
        const size_t bsmem = dnu_qag_blk_smem(I.ld, spec);
        if (split > 1 && bsmem <= 227 * 1024 - 256) {
            static bool blk_attr = false;
            if (!blk_attr) {
                raise_dynamic_smem_limit(reinterpret_cast<const void*>(k_dnu_qag_blk<true>));
                raise_dynamic_smem_limit(reinterpret_cast<const void*>(k_dnu_qag_blk<false>));
                blk_attr = true;
            }
            const int4 sp = make_int4(spec_ids[0], spec_ids[1], spec_ids[2], 0);
            if (spec) k_dnu_qag_blk<true><<<ntask, 256, bsmem, st>>>(I, nk, Na, nspec, sp);
            else k_dnu_qag_blk<false><<<ntask, split >= 4 ? 128 : 64, bsmem, st>>>(I, nk, Na, nspec, sp);
        } else {
            const int blocks = (ntask + wpb - 1) / wpb;
            k_dnu_qag<<<blocks, 32 * wpb, smem, st>>>(I, nk, Na, nspec,
                                                      make_int4(spec_ids[0], spec_ids[1], spec_ids[2], 0));
        }
    }
    if (!defer_combine) k_combine<<<(nk + 255) / 256, 256, 0, st>>>(I, nk);
}

void launch_delta_nu_combined(const IntegratorDev& I, int nk, int Na, double a, double loga, double loga0,
                              double TimeTransfer, int start_row, int nspec, const int* spec_ids,
                              int warps_per_block, cudaStream_t st, int qag_split) {
    launch_integrator_prepare(I, Na, a, loga, loga0, TimeTransfer, start_row, 0, nk <= 0, st);
    if (nk <= 0) return;  // scalars only
    launch_integrator_rest(I, nk, Na, nspec, spec_ids, warps_per_block, st, qag_split);
}

// ------------------------------------------------------------------ end of an update
// commit_row >= 0: overwrite that row with the final delta_tot (delta_tot_table.c:229-233);
// -1: the provisional row is dropped; -2: delta_nu_last is returned as is (the
// same-scale-factor path, delta_tot_table.c:209-213: no NaN check, no clamp);
// -3: a differentiable step: like -1 but delta_nu_last is left unchanged.
__global__ void k_finish(IntegratorDev I, int nk, int commit_row, double a, double loga, const double* keff,
                         double* dnu_out, double* logk_out, double* ratio_out, CorrTable corr, double* norm_out,
                         int combine) {
    const StepScalars& S = *I.sc;
    const bool pass = commit_row == -2;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (commit_row >= 0) I.scalefact[commit_row] = loga;
        if (norm_out) *norm_out = S.kspace_prefac;
    }
    const double norm = S.kspace_prefac;
    // delta_nu of bin ik: k_combine's species sum (same arithmetic) or the combined value
    auto dnu_of = [&](int ik) -> double {
        if (!combine) return I.dnu[ik];
        double acc = 0;
        for (int mi = 0; mi < kNuSpecies; mi++)
            if (I.B->deg[mi] > 0) acc += I.dnu_s[(size_t)mi * I.nk_alloc + ik] * S.omeganu[mi] / S.Omega_nu_tot;
        return acc;
    };
    // Bin ik's slope needs bin ik+1's final value: recomputed here rather than read back,
    // so the bins are independent and spread over many blocks (their FP64 logs and
    // divisions would otherwise queue on one SM).
    for (int ik = blockIdx.x * blockDim.x + threadIdx.x; ik < nk; ik += gridDim.x * blockDim.x) {
        const double v = dnu_of(ik);
        if (combine) I.dnu[ik] = v;
        double out = v;
        if (!pass) {
            if (commit_row != -3) I.nu_last[ik] = v;
            if (commit_row >= 0)
                I.dtot[(size_t)ik * I.ld + commit_row] =
                    get_delta_tot(v, I.dcdm[ik], S.OmegaNua3, S.Omeganonu, S.OmegaNu1, S.partnu);
            if (isnan(v)) atomicOr(I.status, kStDnuNaN);
            out = v < 0 ? 0.0 : v;  // delta_tot_table.c:246-247
        }
        dnu_out[ik] = out;
        if (keff) {
            const double lk = log(keff[ik]);
            const double r = out / I.dcdm[ik];
            if (logk_out) logk_out[ik] = lk;
            if (ratio_out) ratio_out[ik] = r;
            if (corr.xf) {
                corr.xf[ik] = (float)lk;
                corr.rn[ik] = (float)(norm * r);
                double sl = 0;
                if (ik + 1 < nk) {
                    const double v1 = dnu_of(ik + 1);
                    const double out1 = pass ? v1 : (v1 < 0 ? 0.0 : v1);
                    const double lk1 = log(keff[ik + 1]);
                    const double r1 = out1 / I.dcdm[ik + 1];
                    sl = norm * (r1 - r) / (lk1 - lk);
                }
                corr.sn[ik] = (float)sl;
                if (!isfinite(norm * r) || !isfinite(sl)) atomicOr(I.status, kStGridNaN);
            }
        }
    }
}

void launch_finish_update(const IntegratorDev& I, int nk, int commit_row, double a, double loga,
                          const double* keff, double* dnu_out, double* logk_out, double* ratio_out,
                          CorrTable corr, double* norm_out, cudaStream_t st, bool combine) {
    k_finish<<<(nk + 31) / 32 > 0 ? (nk + 31) / 32 : 1, 32, 0, st>>>(I, nk, commit_row, a, loga, keff, dnu_out,
                                                                     logk_out, ratio_out, corr, norm_out,
                                                                     combine ? 1 : 0);
}

}  // namespace ksp
