// ksp_internal.h -- host-visible structures and kernel launchers shared by the
// translation units of libkspace_gb300.so.  Not part of the public C ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "ksp_device.cuh"

namespace ksp {

// Scalars of one integrator call at scale factor a (delta_tot_table.c:153-172,507-548,
// interface_common.c:139-145), computed on the device by k_scalars.
struct StepScalars {
    double a, loga, loga0;           // inputs (logs taken on the host, as the reference does)
    double light, prefac, Omeganonu; // delta_tot_table.c:52-57
    double OmegaNua3, OmegaNu1, partnu;  // get_delta_tot coefficients at a (:179-181)
    double Omega_nu_tot;             // get_omega_nu_nopart(a) (:155)
    double omeganu[kNuSpecies];      // deg * omega_nu_single(a, mi) (:162)
    double fsl_A0a;                  // fslength(log a0, log a) (:522)
    double deriv_prefac;             // a0 * H(a0)/c * a0 (:524)
    double relerr;                   // 1e-6, loosened for hybrid neutrinos (:547)
    double partnu_now;               // particle_nu_fraction(a, 0) (:539)
    double kspace_prefac;            // interface_common.c:139-145
    int skip_integral;               // particles carry everything (:542-543)
    int Na, Nfs;
};

// One integrator instance (the reference's delta_tot_table + omega_nu + transfer table).
struct IntegratorDev {
    Background* B;                   // device
    int nk_alloc, namax, ld;         // ld: padded row length of the history table
    double* scalefact;               // [namax]
    double* dtot;                    // [nk_alloc][ld]
    double* coef;                    // [nk_alloc][ld]  spline coefficients of each row
    double* nu_init;                 // [nk_alloc]
    double* nu_last;                 // [nk_alloc]
    double* wavenum;                 // [nk_alloc]
    const double* kq;                // k of the bins of the current call (the reference integrates at
                                     // the wavenum argument, delta_tot_table.c:526,593); null = wavenum
    double* dcdm;                    // [nk_alloc] sqrt(P_cdm) of the current call
    double* dnu_s;                   // [kNuSpecies][nk_alloc] per-species delta_nu
    double* dnu;                     // [nk_alloc] combined
    double* knot_invdiag;            // [namax] factorised spline system of the knots
    double* knot_fac;                // [namax]
    double* knot_invh;               // [namax] 1/(x_{i+1}-x_i)
    double* knot_h3;                 // [namax] (x_{i+1}-x_i)/3
    double* knot_ih3;                // [namax] 1/(3 (x_{i+1}-x_i))
    double* nc_g;                    // [kNcNodes] node table of the delta_nu integrand (NodeCache)
    double* nc_fsl;
    double* nc_dx;
    int* nc_j;
    int nc_slots;                    // slots of the node table in use (1 + 2 levels, 0 = none)
    double* fs_x;                    // [fs_cap]
    double* fs_y;                    // [fs_cap]
    double* fs_c;                    // [fs_cap]
    double* fs_seg;                  // [fs_cap]
    int fs_cap;
    double* t_logk;                  // transfer table [ntrans]
    double* t_T;
    double* t_c;
    int ntrans;
    StepScalars* sc;                 // device scalars
    unsigned* status;                // device status bits
    int* qag_max;                    // diagnostics: max intervals of any bin in the last call
    long long* qag_total;
    double* ivals;                   // optional: final QAG intervals [kNuSpecies][nk_alloc][kQagLimit][2]
    int* nivals;                     // [kNuSpecies][nk_alloc]
    double* coef_unit;               // [ld] spline coefficients of a unit provisional (last) knot,
                                     // the other knots zero (k_dtot_base)
};

#ifdef __CUDACC__
// The scalars of a call at a (as k_scalars, delta_tot_table.c:153-172,507-548,
// interface_common.c:139-145), by one warp: the background evaluations, which are long
// FP64 dependency chains, run on different lanes; lane 0 combines them.
__device__ __forceinline__ void call_scalars_warp(const Background& B, double a, double loga, double loga0,
                                                  double TT, int Na, StepScalars& S) {
    const int lane = threadIdx.x & 31;
    double v = 0.0;
    if (lane == 0) v = omega_nu(B, a);
    else if (lane == 1) v = omega_nu(B, 1);
    else if (lane < 2 + kNuSpecies) v = B.deg[lane - 2] > 0 ? B.deg[lane - 2] * omega_nu_single(B, a, lane - 2) : 0.0;
    else if (lane == 2 + kNuSpecies) v = hubble(B, TT);
    const double om_a = __shfl_sync(0xffffffffu, v, 0);
    const double om_1 = __shfl_sync(0xffffffffu, v, 1);
    double om_s[kNuSpecies];
    for (int mi = 0; mi < kNuSpecies; mi++) om_s[mi] = __shfl_sync(0xffffffffu, v, 2 + mi);
    const double h_tt = __shfl_sync(0xffffffffu, v, 2 + kNuSpecies);
    if (lane != 0) return;
    const double partnu = particle_nu_fraction(B, a, 0);
    const double nop = om_a - om_1 * partnu / (a * a * a);  // omega_nu_nopart (omega_nu_single.c:69-74)
    S.a = a;
    S.loga = loga;
    S.loga0 = loga0;
    S.Na = Na;
    S.OmegaNua3 = nop * (a * a * a);
    S.OmegaNu1 = om_1;
    S.partnu = partnu;
    S.Omega_nu_tot = nop;
    for (int mi = 0; mi < kNuSpecies; mi++) S.omeganu[mi] = om_s[mi];
    S.deriv_prefac = TT * (h_tt / S.light) * TT;
    S.relerr = 1e-6;
    S.partnu_now = partnu;
    S.skip_integral = 0;
    if (S.partnu_now > 0) {
        if (1 - S.partnu_now < 1e-3) S.skip_integral = 1;
        S.relerr /= (1. + 1e-5 - S.partnu_now);
    }
    S.kspace_prefac = nop / (S.Omeganonu / (a * a * a) + (om_a - nop));
}

// Natural-spline coefficients of one history row against the shared factorisation of
// the knot system (knot_fac, knot_invdiag from k_scalars), by one warp: the row is
// staged in shared memory with coalesced loads, lane 0 runs the forward and back
// substitutions there, and the warp writes the coefficients back coalesced.
// sy, sc: ld doubles of shared memory each, or null to work in global memory (rows
// too long for shared memory).
__device__ __forceinline__ void dtot_row_coeffs_warp(const IntegratorDev& I, int ik, int Na, double* sy,
                                                     double* sc) {
    const int lane = threadIdx.x & 31;
    const double* y = I.dtot + (size_t)ik * I.ld;
    double* c = I.coef + (size_t)ik * I.ld;
    const bool staged = sy != nullptr;
    if (staged) {
        for (int k = lane; k < Na; k += 32) sy[k] = y[k];
    } else {
        sy = const_cast<double*>(y);
        sc = c;
    }
    __syncwarp();
    if (lane == 0) {
        const double* ih = I.knot_invh;
        const int m = Na - 2;
        double prev = 0;
        for (int k = 0; k < m; k++) {
            double r = 3.0 * ((sy[k + 2] - sy[k + 1]) * ih[k + 1] - (sy[k + 1] - sy[k]) * ih[k]);
            if (k > 0) r -= I.knot_fac[k] * prev;
            prev = r;
            sc[k + 1] = r;
        }
        sc[0] = 0.0;
        sc[Na - 1] = 0.0;
        double next = sc[m] * I.knot_invdiag[m - 1];
        sc[m] = next;
        const double* x = I.scalefact;
        for (int k = m - 1; k-- > 0;) {
            const double off = x[k + 2] - x[k + 1];
            next = (sc[k + 1] - off * next) * I.knot_invdiag[k];
            sc[k + 1] = next;
        }
    }
    __syncwarp();
    if (staged)
        for (int k = lane; k < Na; k += 32) c[k] = sc[k];
    __syncwarp();
}

// The fslength table's segment integrals (the segments between its 16*Na uniform knots
// in log a): a group of 4 lanes takes one segment with the 4-point Gauss-Legendre rule
// or, where the knots are closer than 1.5e-3 in log a (the 2-point rule's relative
// error per segment is then below ~3e-14 for this smooth integrand), two segments with
// the 2-point rule.
__host__ __device__ inline int fs_rule_points(int Nfs, double loga0, double loga) {
    return (loga - loga0) / (Nfs - 1.) < 1.5e-3 ? 2 : 4;
}
__host__ __device__ inline int fs_groups(int Nfs, double loga0, double loga) {
    return fs_rule_points(Nfs, loga0, loga) == 4 ? Nfs : (Nfs + 1) / 2;
}
#ifdef __CUDACC__
// lane q (0..3) of group g; called by whole warps (groups are aligned to 4 lanes).
// gx, gw: the positive half of the 4-point rule.
__device__ __forceinline__ void fs_group_eval(const Background& B, int Nfs, double loga0, double loga, int npts,
                                              int g, int q, bool live, const double* gx, const double* gw,
                                              double* fs_x, double* fs_seg) {
    double v = 0.0;
    int seg = -1;
    if (live) {
        const int node = npts == 4 ? q : (q & 1);
        seg = npts == 4 ? g : 2 * g + (q >> 1);
        if (seg < Nfs) {
            const double xa = loga0 + seg * (loga - loga0) / (Nfs - 1.);
            double xb = loga0 + (seg + 1) * (loga - loga0) / (Nfs - 1.);
            if (seg == Nfs - 1) xb = loga;
            if (xb > xa) {
                const double c = 0.5 * (xa + xb), h = 0.5 * (xb - xa);
                double x, w;
                if (npts == 4) {
                    const int j = node & 1;
                    x = node < 2 ? c - h * gx[j] : c + h * gx[j];
                    w = gw[j];
                } else {
                    x = node ? c + h * 0.57735026918962576451 : c - h * 0.57735026918962576451;  // 1/sqrt(3)
                    w = 1.0;
                }
                v = w * h * fsl_integrand(B, x);
            }
            if (node == 0) fs_x[seg] = xa;
        } else {
            seg = -1;
        }
    }
    const double s1 = v + __shfl_down_sync(0xffffffffu, v, 1, 4);
    const double s2 = s1 + __shfl_down_sync(0xffffffffu, s1, 2, 4);
    if (seg >= 0) {
        if (npts == 4 && q == 0) fs_seg[seg] = s2;
        if (npts == 2 && (q & 1) == 0) fs_seg[seg] = s1;
    }
}
#endif

// Natural-spline second derivatives c[0..n-1] of a table y on uniform spacing h, by
// one warp: tridiag(1,4,1) c[1..n-2] = 3/h^2 (y[u+2] - 2 y[u+1] + y[u]), c[0] = c[n-1]
// = 0.  Gaussian elimination has pivots d_0 = 4, d_u = 4 - 1/d_{u-1}; they reach
// 2 + sqrt(3) to double precision by u = 40, and d_u = d_40 is used from there on.
// Forward and back substitution are chains of affine maps, composed per lane over a
// stretch of rows, then across lanes by a warp scan, then replayed (as
// spline_solve_scan).  c holds the forward pass's results in between.
struct UniformPivots {
    double inv[41];  // 1 / d_u, u = 0..40
    constexpr UniformPivots() : inv() {
        double d = 4.0;
        for (int u = 0; u <= 40; u++) {
            if (u > 0) d = 4.0 - 1.0 / d;
            inv[u] = 1.0 / d;
        }
    }
};
static __constant__ UniformPivots kUniformPivots{};
__device__ __forceinline__ double uniform_inv_pivot(int u) { return kUniformPivots.inv[u < 40 ? u : 40]; }
__device__ __forceinline__ void uniform_spline_warp(const double* y, double* c, int n, double h) {
    const int lane = threadIdx.x & 31;
    const int m = n - 2;
    if (m >= 1) {
        const double s3 = 3.0 / (h * h);
        const int per = (m + 31) / 32;
        const int u0 = min(m, lane * per), u1 = min(m, u0 + per);
        // forward: z_u = r_u - z_{u-1} / d_{u-1}
        double A = 1.0, B = 0.0;
        for (int u = u0; u < u1; u++) {
            const double f = u > 0 ? uniform_inv_pivot(u - 1) : 0.0;
            B = s3 * (y[u + 2] - 2.0 * y[u + 1] + y[u]) - f * B;
            A = -f * A;
        }
        double pa = A, pb = B;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const double qa = __shfl_up_sync(0xffffffffu, pa, d), qb = __shfl_up_sync(0xffffffffu, pb, d);
            if (lane >= d) {
                pb = pa * qb + pb;
                pa = pa * qa;
            }
        }
        double zin = __shfl_up_sync(0xffffffffu, pb, 1);
        if (lane == 0) zin = 0.0;
        for (int u = u0; u < u1; u++) {
            const double f = u > 0 ? uniform_inv_pivot(u - 1) : 0.0;
            zin = s3 * (y[u + 2] - 2.0 * y[u + 1] + y[u]) - f * zin;
            c[u + 1] = zin;
        }
        __syncwarp();
        // back: x_u = (z_u - x_{u+1}) / d_u, x_m = 0
        A = 1.0;
        B = 0.0;
        for (int u = u1 - 1; u >= u0; u--) {
            const double iv = uniform_inv_pivot(u);
            const double off = u < m - 1 ? 1.0 : 0.0;
            B = (c[u + 1] - off * B) * iv;
            A = -off * iv * A;
        }
        pa = A;
        pb = B;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const double qa = __shfl_down_sync(0xffffffffu, pa, d), qb = __shfl_down_sync(0xffffffffu, pb, d);
            if (lane + d < 32) {
                pb = pa * qb + pb;
                pa = pa * qa;
            }
        }
        double cin = __shfl_down_sync(0xffffffffu, pb, 1);
        if (lane == 31) cin = 0.0;
        __syncwarp();
        for (int u = u1 - 1; u >= u0; u--) {
            const double off = u < m - 1 ? 1.0 : 0.0;
            cin = (c[u + 1] - off * cin) * uniform_inv_pivot(u);
            c[u + 1] = cin;
        }
    }
    if (lane == 0) {
        c[0] = 0.0;
        c[n - 1] = 0.0;
    }
    __syncwarp();
}

// The same solve with all 32 lanes: both substitutions are linear recurrences
// z_u = r_u - f_u z_{u-1} and c_u = (z_u - o_u c_{u+1}) / d_u, i.e. chains of affine
// maps; each lane composes the maps of its stretch of rows, a warp scan composes the
// stretches, and each lane then replays its stretch from the value entering it.  The
// results equal the sequential sweep's up to rounding.  sy, sc: ld doubles of shared
// memory each (staged rows).
// Solve the natural-spline system of the knots (factorised by k_scalars) for the
// right-hand side sc[1..m], m = Na - 2, in place, with all 32 lanes of a warp.
__device__ __forceinline__ void spline_solve_scan(const IntegratorDev& I, int m, double* sc) {
    const int lane = threadIdx.x & 31;
    const double* x = I.scalefact;
    const int per = (m + 31) / 32;
    const int u0 = min(m, lane * per), u1 = min(m, u0 + per);
    // forward: z_u = r_u - fac_u z_{u-1} (fac_0 = 0)
    double A = 1.0, B = 0.0;
    for (int u = u0; u < u1; u++) {
        const double f = u > 0 ? I.knot_fac[u] : 0.0;
        B = sc[u + 1] - f * B;
        A = -f * A;
    }
    double pa = A, pb = B;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {  // inclusive scan of the maps, left to right
        const double qa = __shfl_up_sync(0xffffffffu, pa, d), qb = __shfl_up_sync(0xffffffffu, pb, d);
        if (lane >= d) {
            pb = pa * qb + pb;
            pa = pa * qa;
        }
    }
    double zin = __shfl_up_sync(0xffffffffu, pb, 1);  // z entering this stretch (z_{-1} = 0)
    if (lane == 0) zin = 0.0;
    for (int u = u0; u < u1; u++) {
        const double f = u > 0 ? I.knot_fac[u] : 0.0;
        zin = sc[u + 1] - f * zin;
        sc[u + 1] = zin;
    }
    __syncwarp();
    // backward: c_u = (z_u - off_u c_{u+1}) * invdiag_u, c_m = 0
    A = 1.0;
    B = 0.0;
    for (int u = u1 - 1; u >= u0; u--) {
        const double off = u < m - 1 ? x[u + 2] - x[u + 1] : 0.0;
        const double iv = I.knot_invdiag[u];
        B = (sc[u + 1] - off * B) * iv;
        A = -off * iv * A;
    }
    pa = A;
    pb = B;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {  // right to left
        const double qa = __shfl_down_sync(0xffffffffu, pa, d), qb = __shfl_down_sync(0xffffffffu, pb, d);
        if (lane + d < 32) {
            pb = pa * qb + pb;
            pa = pa * qa;
        }
    }
    double cin = __shfl_down_sync(0xffffffffu, pb, 1);  // c entering from the right
    if (lane == 31) cin = 0.0;
    __syncwarp();
    for (int u = u1 - 1; u >= u0; u--) {
        const double off = u < m - 1 ? x[u + 2] - x[u + 1] : 0.0;
        cin = (sc[u + 1] - off * cin) * I.knot_invdiag[u];
        sc[u + 1] = cin;
    }
    __syncwarp();
}

// The same solve with all 32 lanes: both substitutions are linear recurrences
// z_u = r_u - f_u z_{u-1} and c_u = (z_u - o_u c_{u+1}) / d_u, i.e. chains of affine
// maps; each lane composes the maps of its stretch of rows, a warp scan composes the
// stretches, and each lane then replays its stretch from the value entering it.  The
// results equal the sequential sweep's up to rounding.  sy, sc: ld doubles of shared
// memory each (staged rows).
__device__ __forceinline__ void dtot_row_coeffs_scan(const IntegratorDev& I, int ik, int Na, double* sy,
                                                     double* sc) {
    const int lane = threadIdx.x & 31;
    const double* y = I.dtot + (size_t)ik * I.ld;
    double* c = I.coef + (size_t)ik * I.ld;
    for (int k = lane; k < Na; k += 32) sy[k] = y[k];
    __syncwarp();
    const int m = Na - 2;  // unknowns c[1..m]
    const double* ih = I.knot_invh;
    for (int u = lane; u < m; u += 32)
        sc[u + 1] = 3.0 * ((sy[u + 2] - sy[u + 1]) * ih[u + 1] - (sy[u + 1] - sy[u]) * ih[u]);
    __syncwarp();
    spline_solve_scan(I, m, sc);
    for (int k = lane; k < Na; k += 32) c[k] = (k == 0 || k == Na - 1) ? 0.0 : sc[k];
    __syncwarp();
}

// The delta_nu integrand of one (species, bin) with the instance's node table; knots,
// row and rc may be staged copies (shared memory) of the instance's arrays.
// sb, sd: seg_poly of (row, rc), filled by the caller
// k_over_m = k / (m / kT) and fs_inv = (Nfs - 1) / (log a - log a0) given: the integral
// kernels form those divisions on one lane per task and broadcast them
__device__ __forceinline__ DnuIntegrandC dnu_integrand_pre(const IntegratorDev& I, const StepScalars& S,
                                                           double k_over_m, double fs_inv, double qc,
                                                           const double* knots, const double* row, const double* rc,
                                                           const double* sb, const double* sd, int Na) {
    DnuIntegrandC f;
    f.B = I.B; f.k_over_m = k_over_m; f.qc = qc; f.nfl = I.B->nufrac_low[0];
    f.fs_x = I.fs_x; f.fs_y = I.fs_y; f.fs_c = I.fs_c; f.nfs = S.Nfs; f.fs_x0 = S.loga0;
    f.fs_inv = fs_inv;
    f.kx = knots; f.ky = row; f.kc = rc; f.na = Na;
    f.sb = sb; f.sd = sd;
    f.ks = KnotSeg{I.knot_invh, I.knot_h3, I.knot_ih3};
    f.nc = NodeCache{I.nc_g, I.nc_fsl, I.nc_dx, I.nc_j, I.nc_slots};
    return f;
}
__device__ __forceinline__ DnuIntegrandC dnu_integrand(const IntegratorDev& I, const StepScalars& S, double k,
                                                       double mnubykT, double qc, const double* knots,
                                                       const double* row, const double* rc, const double* sb,
                                                       const double* sd, int Na) {
    return dnu_integrand_pre(I, S, k / mnubykT, (S.Nfs - 1.) / (S.loga - S.loga0), qc, knots, row, rc, sb, sd, Na);
}
// The delta_nu of one (species, bin) task (delta_tot_table.c:525-535 and :597-603): the
// initial-condition term plus prefac times the integral; one lane forms it (FP64 log and
// exp of the J fit are issued per active lane).
__device__ __forceinline__ double dnu_task_value(const IntegratorDev& I, const StepScalars& S, int ik,
                                                 double k, double mnubykT, bool integrated, double integral) {
    const double specJ0 = specialJ(k * S.fsl_A0a / (mnubykT > 0 ? mnubykT : 1), 0.0, I.B->nufrac_low[0]);
    double val = specJ0 * I.nu_init[ik] * (1. + S.deriv_prefac * S.fsl_A0a);
    if (integrated) val += S.prefac * integral;
    return val;
}
#endif

// Interpolation table for the grid correction (delta_pow.c:19-37), float, per
// non-empty bin, plus the bin -> compact index map.
// K1's normalisation of one compact bin (powerspectrum.c:98-115 + interface_gadget.c:
// 96-100): P = sum / |F(0)|^2 / count, keff = sum|k| / count (grid units), delta_cdm =
// sqrt(P L^3), keff in physical units.  k_finalize_power applies it to every bin; the
// step's row-spline kernel applies it to its bin when the binning pass deferred it.
struct FinalizeArgs {
    const double* bin_sum;
    const double* F0sq;
    const long long* count;
    const double* ksum;
    const int* compact_bins;
    double BoxSize;
    double* power_out;
    double* keff_out;
    double* dcdm_out;
    double* keffphys_out;
    int active;  // 0: nothing to do
    // formed on the host, as the reference forms them there (interface_gadget.c:84,96-99):
    // scale = BoxSize^-3 (pow), kfac = 2 pi / BoxSize
    double scale, kfac;
};
#ifdef __CUDACC__
__device__ __forceinline__ void finalize_bin(const FinalizeArgs& f, int c) {
    const int b = f.compact_bins[c];
    double p = f.bin_sum[b];
    p /= *f.F0sq;
    const double cnt = (double)f.count[b];
    const double ke = f.ksum[b] / cnt;
    p /= cnt;
    if (f.power_out) f.power_out[c] = p;
    if (f.keff_out) f.keff_out[c] = ke;
    if (f.dcdm_out) f.dcdm_out[c] = sqrt(p / f.scale);
    if (f.keffphys_out) f.keffphys_out[c] = ke * f.kfac;
}
#endif

struct CorrTable {
    float* xf;   // log k of node j
    float* rn;   // norm * ratio_j
    float* sn;   // norm * (ratio_{j+1}-ratio_j)/(logk_{j+1}-logk_j)
    int nk;
};

// Raise a kernel's dynamic shared-memory limit to the most a block may have beside the
// kernel's own static shared memory (the device's opt-in maximum minus it), once per
// kernel and device (ksp_api.cu).  A fixed 227 KB request fails for a kernel with static
// shared memory, and the failure would surface as the error of a later, unrelated launch.
int raise_dynamic_smem_limit(const void* kernel);

// ---- integrator launchers (ksp_integrator.cu)
void launch_background_tables(Background* dB, double a0, cudaStream_t st, unsigned* status);
void launch_spline_coeffs_1thread(const double* x, const double* y, double* c, double* scratch, int n,
                                  cudaStream_t st);
void launch_nufrac_low(Background* dB, double light, double vcrit, cudaStream_t st, unsigned* status);
// natural cubic spline of log H on n uniform knots of spacing h: coef[4 (n-1)], scratch[n]
void launch_hubble_table(const double* H, int n, double h, double* coef, double* scratch, cudaStream_t st);
// nufrac_low (omega_nu_single.c:214-228) of n momenta, a warp each
void launch_nufrac_low_values(const double* qc, int n, double* out, unsigned* status, cudaStream_t st);
// specialJ (delta_tot_table.c:457-463) of n arguments
void launch_special_j(const double* x, int n, double qc, double nufrac_low, double* out, cudaStream_t st);
// fslength (delta_tot_table.c:394-407) of n intervals [logai, logaf], a warp each
void launch_fslength_values(const Background* dB, const double* logai, const double* logaf, int n, double light,
                            double* out, cudaStream_t st);
// update_delta_tot (delta_tot_table.c:177-191) for row `row` at scale factor a
void launch_update_row(const IntegratorDev& I, int nk, int row, double a, double loga, const double* dcdm,
                       const double* dnu, cudaStream_t st);
// delta_tot_init part that needs the device (delta_tot_table.c:94-129)
void launch_delta_tot_init(const IntegratorDev& I, int nk, const double* wavenum, const double* dcdm,
                           int fresh, double TimeTransfer, cudaStream_t st);
// get_delta_nu_combined (delta_tot_table.c:153-172) with Na rows: writes I.dnu
// start_row: leading rows of the knot factorisation still valid from an earlier call
// qag_split: warps per (species, bin) task (1, 2 or 4; 0 = chosen by the task count)
void launch_delta_nu_combined(const IntegratorDev& I, int nk, int Na, double a, double loga, double loga0,
                              double TimeTransfer, int start_row, int nspec, const int* spec_ids,
                              int warps_per_block, cudaStream_t st, int qag_split = 0);
// the same in two parts: what does not depend on delta_cdm (may overlap the binning
// pass; write_knot stores the provisional knot log a), and the rest
void launch_integrator_prepare(const IntegratorDev& I, int Na, double a, double loga, double loga0,
                               double TimeTransfer, int start_row, int write_knot, bool scalars_only,
                               cudaStream_t st);
// update_row >= 0: write the provisional row `update_row` (update_delta_tot, from
// delta_nu_last and delta_cdm with the call's scalars) as each row's spline is solved;
// defer_combine: leave the species sum to launch_finish_update(..., combine = true)
// base_ready: launch_dtot_base ran for this Na (the rows' splines then take the
// provisional row as a correction)
void launch_integrator_rest(const IntegratorDev& I, int nk, int Na, int nspec, const int* spec_ids,
                            int warps_per_block, cudaStream_t st, int qag_split, int update_row = -1,
                            bool defer_combine = false, const FinalizeArgs* fin = nullptr,
                            bool base_ready = false);
// Before the provisional row is known (beside the binning pass, after
// launch_integrator_prepare): every row's spline with its last knot equal to the one
// before, and the spline of a unit last knot.  False for histories of two knots or fewer.
bool launch_dtot_base(const IntegratorDev& I, int nk, int Na, cudaStream_t st);
size_t dnu_qag_smem(int ld, int wpb);
// end of get_delta_nu_update (delta_tot_table.c:226-248) + interface_common.c:134-146:
// delta_nu_last, committed row, NaN check, clamp, ratio/log k/kspace_prefac, grid table
void launch_finish_update(const IntegratorDev& I, int nk, int commit_row, double a, double loga,
                          const double* keff, double* dnu_out, double* logk_out, double* ratio_out,
                          CorrTable corr, double* norm_out, cudaStream_t st, bool combine = false);

// ---- adjoint (ksp_adjoint.cu)
struct AdjBinsHost {
    const double* node_sum; const double* pnu_bar; const double* dnu; const double* dcdm; const double* power;
    const long long* count; const int* compact; const double* F0sq;
    double* dnu_bar; double* dprov_bar; double* rbar; double* Q; double* dc_sum;
    double norm, L3, fcdm;
    int nk, ld;  // dprov_bar has stride ld
};
size_t dnu_adj_smem(int ld, int wpb);

// ---- grid launchers (ksp_grid.cu)
struct GridGeom {
    int N, nrbins, slab0, nslab;
    long long nmodes;               // nslab * N * (N/2+1)
    int* thresh;                    // device [nrbins+1]: min k^2 of each bin
    float* w1;                      // device [N/2+1]: 1-D inverse CIC window (float)
    int* cmap;                      // device [nrbins]: bin -> compact index (-1 empty)
    float bin_c1;                   // binsperunit * ln2 / 2 (approximate bin estimate)
    unsigned* runtab = nullptr;     // device run table of the binning pass (or null)
    int run_Rp = 0;                 // its row length: runs of 17 modes per grid row, rounded up to 4
};
// the run table of a geometry (ksp_stream.cu): 0 built, 1 not applicable (2^15 bins or
// more, or over 1 GiB), -1 error
int build_run_table(GridGeom& g, cudaStream_t st);
// histogram of weighted mode counts over integer k^2 for the slab range
void launch_k2_histogram(int N, int slab0, int nslab, unsigned long long* hist, cudaStream_t st);
// K1: per-bin sum of w |F|^2 W^4 (double), and |F(0)|^2 when slab0 == 0
// returns 0 (TMA kernel), 1 (plain kernel) or -2 (launch error)
int launch_bin_power(const GridGeom& g, const float* grid, double* bin_sum, double* F0sq, unsigned* status, int tma,
                     int rows_per_cta, int stages, cudaStream_t st);
// K3: grid *= 1 + norm * interp(log k)
// Every variant leaves the grid as it is when the status word holds an error (kStAbort).
int launch_apply_correction(const GridGeom& g, float* grid, CorrTable corr, float lnscale, unsigned* status, int tma,
                            int rows_per_cta, int stages, cudaStream_t st);
// normalisation of K1's sums into P(k), delta_cdm, keff (powerspectrum.c:98-115,
// interface_gadget.c:96-100)
void launch_finalize_power(const double* bin_sum, const double* F0sq, const long long* count, const double* ksum,
                           const int* compact_bins, int nk, double BoxSize, double* power_out, double* keff_out,
                           double* dcdm_out, double* keffphys_out, cudaStream_t st);

struct GridGeom;
void launch_adj_reduce(const GridGeom& gg, CorrTable corr, float lnscale, const float* gbar, const float* x,
                       double* node_sum, cudaStream_t st);
void launch_adj_bins(const AdjBinsHost& h, cudaStream_t st);
void launch_adj_bins2(const AdjBinsHost& h, cudaStream_t st);
void launch_dnu_adj(const IntegratorDev& I, const double* dnu_bar, double* Dbar, double* mbar, const double* ivals,
                    const int* nivals, int recompute, int nk, int Na, int nspec, const int* spec_ids, int wpb,
                    cudaStream_t st);
void launch_adj_grid(const GridGeom& gg, CorrTable corr, float lnscale, const float* gbar, const float* x, float* xbar,
                     const double* Q, const double* dc_sum, const double* F0sq, cudaStream_t st);

}  // namespace ksp
