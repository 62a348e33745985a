// ksp_device.cuh -- device-side numerics of the linear-response neutrino integrator.
//
// Background cosmology (Omega_nu(a) from Fermi-Dirac tables, H(a)), natural cubic
// splines, the Fermi-Dirac kernel J(x), and a warp-cooperative QAG integrator that
// makes the same adaptive decisions as QUADPACK's QAG with the 61-point Gauss-Kronrod
// rule (the integrator the reference calls through GSL, delta_tot_table.c:404,597).
// Each function names the reference file:line whose arithmetic it follows.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <float.h>
#include "gk61_table.h"

#define KSP_HD __host__ __device__ __forceinline__

namespace ksp {

// kspace_neutrino_const.h:9-19, gadget_defines.h:8, omega_nu_single.c:10-14,85
constexpr int kNuSpecies = 3;
constexpr int kNRhoTab = 200;
constexpr int kQagLimit = 200;  // GSL_VAL
constexpr double kLightCgs = 2.99792458e10;
constexpr double kBolEvK = 8.61734e-5;
constexpr double kHubble = 3.24077929e-18;
constexpr double kHbar = 6.582119e-16;
constexpr double kStefanBoltzmann = 5.670373e-5;
constexpr double kGravity = 6.67408e-8;
constexpr double kNuSw = 100.0;
constexpr double kFloatAcc = 1e-6;
constexpr double kPi = 3.14159265358979323846;
constexpr double kZeta3 = 1.202056903159594;

// Status bits written by kernels (host maps them to reference error codes).
enum : unsigned {
    kStGsl = 1u << 0,        // QAG failed / interpolation out of range  -> 2001
    kStDnuNaN = 1u << 1,     // delta_nu is NaN                          -> 2004
    kStGridNaN = 1u << 2,    // correction factor is NaN                 -> 5
    kStKmax = 1u << 3,       // k beyond transfer table                  -> 2
    kStKWarn = 1u << 4,      // k < keff_0 / 2 (reference prints to stderr, continues)
    kStTimeout = 1u << 5,    // a bounded wait expired
};
// the errors after which the reference terminates before it corrects the grid: the
// correction pass leaves the grid as it is when one of them is set
constexpr unsigned kStAbort = kStGsl | kStDnuNaN | kStGridNaN | kStKmax | kStTimeout;

// omega_nu_single.h:27-34: tabulated rho_nu(a) of one species (natural cubic spline in log a)
struct RhoTable {
    int has_table;
    double mnu;
    double loga[kNRhoTab], rhonu[kNRhoTab], c[kNRhoTab];
    // filled with c (k_rho_splines): the node-independent spline terms of each segment
    // (as cspline_seg forms them), 1 / knot spacing and 1 / mnu, for fsl_integrand
    double sb[kNRhoTab], sd[kNRhoTab];
    double inv_dx, imnu;
};

// omega_nu_single.h:100-113 (_omega_nu, _hybrid_nu) plus the parameters of the host's
// hubble_function (delta_tot_table_test.c:33-45; curvature as gadget-2/0003 patch:38).
struct Background {
    double rhocrit, kBtnu, tcmb0, conv, omegag0;
    double irhocrit;  // 1 / rhocrit
    int deg[kNuSpecies];
    double mnu[kNuSpecies];
    double mnu_J[kNuSpecies];  // mass inside J's argument (get_delta_nu's mnu, delta_tot_table.c:507)
    int hyb_enabled;
    double nufrac_low[kNuSpecies], nu_crit_time, vcrit;
    double Omega_nonu_H, OmegaLambda, OmegaK, hubble;
    int radiation;
    RhoTable tab[kNuSpecies];
    // A host H(a) of another form, tabulated: log H as a natural cubic spline in log a on
    // htab_n uniform knots from htab_lo with spacing htab_h, 4 coefficients per segment
    // (device copy for kernels, host copy for host-side evaluation); htab_n = 0: the
    // analytic form above.
    const double* htab_d;
    const double* htab_h;
    int htab_n;
    double htab_lo, htab_dx;
};

// ------------------------------------------------------------------ splines
// Segment i with x[i] <= v < x[i+1] (v == x[n-1] -> n-2), as GSL's bsearch.
KSP_HD int seg_bsearch(const double* x, int n, double v) {
    int lo = 0, hi = n - 1;
    while (hi > lo + 1) {
        const int mid = (lo + hi) >> 1;
        if (x[mid] > v) hi = mid; else lo = mid;
    }
    return lo;
}

// Natural cubic spline (c = S''/2 at the knots) evaluated on segment i.
KSP_HD double cspline_seg(const double* x, const double* y, const double* c, int i, double v) {
    const double h = x[i + 1] - x[i], dx = v - x[i];
    const double b = (y[i + 1] - y[i]) / h - h * (c[i + 1] + 2.0 * c[i]) / 3.0;
    const double d = (c[i + 1] - c[i]) / (3.0 * h);
    return y[i] + dx * (b + dx * (c[i] + dx * d));
}

KSP_HD double linear_seg(const double* x, const double* y, int i, double v) {
    return y[i] + (v - x[i]) * ((y[i + 1] - y[i]) / (x[i + 1] - x[i]));
}

// Natural cubic spline coefficients by Gaussian elimination (sequential; small n).
// scratch: 2*(n-2) doubles.  Same equations as a natural spline anywhere.
KSP_HD void natural_spline_coeffs(const double* x, const double* y, int n, double* c, double* scratch) {
    const int m = n - 2;
    c[0] = 0.0;
    c[n - 1] = 0.0;
    if (m <= 0) return;
    double* diag = scratch;
    double* rhs = scratch + m;
    for (int i = 0; i < m; i++) {
        const double h0 = x[i + 1] - x[i], h1 = x[i + 2] - x[i + 1];
        diag[i] = 2.0 * (h0 + h1);
        rhs[i] = 3.0 * ((y[i + 2] - y[i + 1]) / h1 - (y[i + 1] - y[i]) / h0);
    }
    for (int i = 1; i < m; i++) {
        const double off = x[i + 1] - x[i];
        const double f = off / diag[i - 1];
        diag[i] -= f * off;
        rhs[i] -= f * rhs[i - 1];
    }
    c[m] = rhs[m - 1] / diag[m - 1];
    for (int i = m - 1; i-- > 0;) {
        const double off = x[i + 2] - x[i + 1];
        c[i + 1] = (rhs[i] - off * c[i + 2]) / diag[i];
    }
}

// ------------------------------------------------------------------ background
// omega_nu_single.c:100-114 (rho_nu conversion factor)
KSP_HD double rho_nu_conversion() {
    double convert = 4 * kPi * 2;
    const double chbar = 1. / (2 * kPi * kLightCgs * kHbar);
    convert *= (chbar * chbar * chbar);
    convert *= (1.60217646e-12 / kLightCgs / kLightCgs);
    return convert;
}

// omega_nu_single.c:156-160
KSP_HD double non_rel_rho_nu(double a, double kT, double amnu, double kTamnu2, double conv) {
    return amnu * (kT * kT * kT) / (a * a * a * a) *
           (1.5 * kZeta3 + kTamnu2 * 45. / 4. * 1.0369277551433704 +
            2835. / 32. * kTamnu2 * kTamnu2 * 1.0083492773819229 +
            80325 / 32. * kTamnu2 * kTamnu2 * kTamnu2 * 1.0020083928260826) * conv;
}

// omega_nu_single.c:164-167
KSP_HD double rel_rho_nu(double a, double kT, double conv) {
    const double t = kPi * kT / a, t2 = t * t;
    return 7 * (t2 * t2) / 120. * conv;
}

// omega_nu_single.c:171-202
// loga_in: log(a) when the caller has it (NaN: computed here)
KSP_HD double rho_nu(const RhoTable& T, double a, double kT, double conv, double loga_in = NAN) {
    const double amnu = a * T.mnu;
    const double kTamnu2 = (kT * kT / amnu / amnu);
    if (kNuSw * kNuSw * kTamnu2 < 1) return non_rel_rho_nu(a, kT, amnu, kTamnu2, conv);
    if (amnu < 1e-6 * kT) return rel_rho_nu(a, kT, conv);
    const double loga = loga_in == loga_in ? loga_in : log(a);
    if (!T.has_table || loga < T.loga[0]) {
        if (amnu < 1e-4 * kT) return rel_rho_nu(a, kT, conv);
        return non_rel_rho_nu(a, kT, amnu, kTamnu2, conv);
    }
    // uniform knots: guess the segment, then settle it against the stored knots
    const double inv = (kNRhoTab - 1) / (T.loga[kNRhoTab - 1] - T.loga[0]);
    int i = (int)((loga - T.loga[0]) * inv);
    i = i < 0 ? 0 : (i > kNRhoTab - 2 ? kNRhoTab - 2 : i);
    while (i > 0 && loga < T.loga[i]) i--;
    while (i < kNRhoTab - 2 && loga >= T.loga[i + 1]) i++;
    return cspline_seg(T.loga, T.rhonu, T.c, i, loga);
}

// omega_nu_single.c:246-257
KSP_HD double particle_nu_fraction(const Background& B, double a, int i) {
    if (!B.hyb_enabled) return 0;
    if (a > B.nu_crit_time) return B.nufrac_low[i];
    return 0;
}

// omega_nu_single.c:55-65
KSP_HD double omega_nu(const Background& B, double a, double loga = NAN) {
    double rhonu = 0;
    for (int mi = 0; mi < kNuSpecies; mi++)
        if (B.deg[mi] > 0) rhonu += B.deg[mi] * rho_nu(B.tab[mi], a, B.kBtnu, B.conv, loga);
    return rhonu / B.rhocrit;
}

// omega_nu_single.c:69-74
KSP_HD double omega_nu_nopart(const Background& B, double a) {
    return omega_nu(B, a) - omega_nu(B, 1) * particle_nu_fraction(B, a, 0) / (a * a * a);
}

// omega_nu_single.c:262-279
KSP_HD double omega_nu_single(const Background& B, double a, int i) {
    if (B.deg[i] == 0) {
        for (int j = i; j >= 0; j--)
            if (B.deg[j]) { i = j; break; }
    }
    const double om = rho_nu(B.tab[i], a, B.kBtnu, B.conv) / B.rhocrit;
    double part = rho_nu(B.tab[i], 1, B.kBtnu, B.conv) / B.rhocrit;
    part *= particle_nu_fraction(B, a, i) / (a * a * a);
    return om - part;
}

// log H at log a from the tabulated spline (the end segments continue past the table)
KSP_HD double hubble_tab_log(const Background& B, double la) {
#ifdef __CUDA_ARCH__
    const double* t = B.htab_d;
#else
    const double* t = B.htab_h;
#endif
    int i = (int)floor((la - B.htab_lo) / B.htab_dx);
    i = i < 0 ? 0 : (i > B.htab_n - 2 ? B.htab_n - 2 : i);
    const double dx = la - (B.htab_lo + i * B.htab_dx);
    const double* c = t + 4 * i;
    return c[0] + dx * (c[1] + dx * (c[2] + dx * c[3]));
}

// delta_tot_table_test.c:33-45 (+ curvature, gadget-2/0003 patch:38); Omega_g as
// omega_nu_single.c:77-81.
KSP_HD double hubble(const Background& B, double a, double loga = NAN) {
    if (B.htab_n > 0) return exp(hubble_tab_log(B, loga == loga ? loga : log(a)));
    const double a3 = a * a * a;
    double om = B.Omega_nonu_H / a3 + B.OmegaLambda;
    if (B.OmegaK != 0.0) om += B.OmegaK / (a * a);
    om += omega_nu(B, a, loga);
    if (B.radiation) om += B.omegag0 / (a3 * a);
    return B.hubble * sqrt(om);
}

#ifdef __CUDACC__
// rho_nu for fsl_integrand: the same branches as rho_nu, with 1/a given and the table
// spline in per-segment polynomial form (RhoTable::sb, sd).
__device__ __forceinline__ double rho_nu_ia(const RhoTable& T, double a, double ia, double loga, double kT,
                                            double conv) {
    const double amnu = a * T.mnu;
    const double kTamnu = kT * ia * T.imnu, kTamnu2 = kTamnu * kTamnu;
    bool nonrel = kNuSw * kNuSw * kTamnu2 < 1;
    bool rel = !nonrel && amnu < 1e-6 * kT;
    if (!nonrel && !rel && (!T.has_table || loga < T.loga[0])) {
        rel = amnu < 1e-4 * kT;
        nonrel = !rel;
    }
    if (nonrel) {
        const double ia4 = (ia * ia) * (ia * ia);
        return amnu * (kT * kT * kT) * ia4 *
               (1.5 * kZeta3 + kTamnu2 * 45. / 4. * 1.0369277551433704 +
                2835. / 32. * kTamnu2 * kTamnu2 * 1.0083492773819229 +
                80325 / 32. * kTamnu2 * kTamnu2 * kTamnu2 * 1.0020083928260826) * conv;
    }
    if (rel) {
        const double t = kPi * kT * ia, t2 = t * t;
        return 7 * (t2 * t2) / 120. * conv;
    }
    int i = (int)((loga - T.loga[0]) * T.inv_dx);
    i = i < 0 ? 0 : (i > kNRhoTab - 2 ? kNRhoTab - 2 : i);
    while (i > 0 && loga < T.loga[i]) i--;
    while (i < kNRhoTab - 2 && loga >= T.loga[i + 1]) i++;
    const double dx = loga - T.loga[i];
    return T.rhonu[i] + dx * (T.sb[i] + dx * (T.c[i] + dx * T.sd[i]));
}

// The fslength integrand 1/(a^2 H(a)) at a = e^x (delta_tot_table.c:378-383) with H as
// hubble() forms it, 1/a computed once (one exp, one sqrt, two divisions per node).
__device__ __forceinline__ double fsl_integrand(const Background& B, double x) {
    if (B.htab_n > 0) return exp(-2.0 * x - hubble_tab_log(B, x));
    const double a = exp(x);
    const double ia = 1.0 / a;
    const double ia2 = ia * ia, ia3 = ia2 * ia;
    double om = B.Omega_nonu_H * ia3 + B.OmegaLambda;
    if (B.OmegaK != 0.0) om += B.OmegaK * ia2;
    double rhonu = 0;
    for (int mi = 0; mi < kNuSpecies; mi++)
        if (B.deg[mi] > 0) rhonu += B.deg[mi] * rho_nu_ia(B.tab[mi], a, ia, x, B.kBtnu, B.conv);
    om += rhonu * B.irhocrit;
    if (B.radiation) om += B.omegag0 * (ia3 * ia);
    return ia2 / (B.hubble * sqrt(om));
}
#endif

// delta_tot_table.c:613-617
KSP_HD double get_delta_tot(double dnu, double dcdm, double OmegaNua3, double Omeganonu, double Omeganu1,
                            double partnu) {
    const double fcdm = 1 - OmegaNua3 / (Omeganonu + Omeganu1);
    return fcdm * (dcdm + dnu * OmegaNua3 / (Omeganonu + Omeganu1 * partnu));
}

// ------------------------------------------------------------------ J(x)
// delta_tot_table.c:417-428
KSP_HD double specialJ_fit(double x) {
    if (x <= 0.) return 1.;
    const double x2 = x * x, x4 = x2 * x2, x8 = x4 * x4;
    return (1. + 0.0168 * x2 + 0.0407 * x4) / (1. + 2.1734 * x2 + 1.6787 * exp(4.1811 * log(x)) + 0.1467 * x8);
}

// sin(y)/y: Taylor series 1 - y^2/6 + y^4/120 - y^6/5040 + y^8/362880 near 0.
KSP_HD double sinc_j0(double y) {
    if (fabs(y) < 0.05) {
        const double t = y * y;
        return 1.0 - t / 6.0 * (1.0 - t / 20.0 * (1.0 - t / 42.0 * (1.0 - t / 72.0)));
    }
    return sin(y) / y;
}

// delta_tot_table.c:431-434
KSP_HD double II(double x, double qc, int n) {
    return (n * n + n * n * n * qc + n * qc * x * x - x * x) * qc * sinc_j0(qc * x) +
           (2 * n + n * n * qc + qc * x * x) * cos(qc * x);
}

// delta_tot_table.c:442-463
KSP_HD double specialJ(double x, double qc, double nufrac_low) {
    if (qc > 0) {
        double integ = 0;
        for (int n = 1; n < 20; n++) {
            const double s = (n & 1) ? 1.0 : -1.0;  // -(-1)^n
            const double d = n * n + x * x;
            integ += s * exp(-n * qc) / d / d * II(x, qc, n);
        }
        return integ / (1.5 * kZeta3 * (1 - nufrac_low));
    }
    return specialJ_fit(x);
}

// Index of the largest error among e[0..n) (lowest index on ties), on every lane of
// the warp.  Errors are >= 0, so their IEEE bit patterns order as the numbers do: the
// comparisons run on the integer pipe (a NaN, never chosen by the floating-point
// comparison, gets key -1).
__device__ __forceinline__ long long err_key(double e) {
    const long long b = __double_as_longlong(e);
    return (b & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL ? -1LL : b;
}
__device__ __forceinline__ int warp_argmax_err(const double* e, int n) {
    const int lane = threadIdx.x & 31;
    long long best = -1;
    int bk = 0x7fffffff;
    for (int i = lane; i < n; i += 32) {
        const long long v = err_key(e[i]);
        if (v > best) { best = v; bk = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const long long ob = __shfl_down_sync(0xffffffffu, best, o);
        const int ok = __shfl_down_sync(0xffffffffu, bk, o);
        if (ob > best || (ob == best && ok < bk)) { best = ob; bk = ok; }
    }
    return __shfl_sync(0xffffffffu, bk, 0);
}

// ------------------------------------------------------------------ QAG (GK61)
#ifdef __CUDACC__
struct Gk61Nodes {  // expanded 61-node table: slot j<30: -x_j, 30<=j<60: +x_{j-30}, 60: centre
    double x[61], wk[61], wg[61];
};

__device__ __forceinline__ void gk61_fill(Gk61Nodes& n, int tid, int nthreads) {
    const double XK[31] = KSP_GK61_XK_INIT;
    const double WK[31] = KSP_GK61_WK_INIT;
    const double WG[31] = KSP_GK61_WG_INIT;
    for (int j = tid; j < 61; j += nthreads) {
        if (j < 30) { n.x[j] = -XK[j]; n.wk[j] = WK[j]; n.wg[j] = WG[j]; }
        else if (j < 60) { n.x[j] = XK[j - 30]; n.wk[j] = WK[j - 30]; n.wg[j] = WG[j - 30]; }
        else { n.x[j] = 0.0; n.wk[j] = WK[30]; n.wg[j] = 0.0; }
    }
}

__device__ __forceinline__ double warp_sum_to0(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double bcast0(double v) { return __shfl_sync(0xffffffffu, v, 0); }

// QUADPACK error estimate: err = resasc * min(1, (200 |err|/resasc)^1.5), floored at
// 50 eps resabs (Piessens et al. 1983, qk rules).  t^1.5 as t sqrt(t): within an ulp of
// pow(t, 1.5), without pow's long FP64 dependency chain on the QAG's critical path.
__device__ __forceinline__ double rescale_error(double err, double resabs, double resasc) {
    err = fabs(err);
    if (resasc != 0.0 && err != 0.0) {
        const double t = 200.0 * err / resasc;
        const double s = t * sqrt(t);
        err = s < 1.0 ? resasc * s : resasc;
    }
    if (resabs > DBL_MIN / (50.0 * DBL_EPSILON)) {
        const double fl = 50.0 * DBL_EPSILON * resabs;
        if (fl > err) err = fl;
    }
    return err;
}

struct GkOut { double result, abserr, resabs, resasc; };

// Evaluate the GK61 rule on `nint` (1 or 2) intervals [a_t, b_t] with one warp.
// Every lane returns identical values (sums are reduced to lane 0 and broadcast).
template <class F>
__device__ __forceinline__ void gk61_warp(const F& f, const Gk61Nodes& N, int nint, const double* a, const double* b,
                                          GkOut* out) {
    const int lane = threadIdx.x & 31;
    double c[2], h[2];
    for (int t = 0; t < 2; t++) {
        c[t] = __dmul_rn(0.5, __dadd_rn(a[t], b[t]));
        h[t] = __dmul_rn(0.5, __dsub_rn(b[t], a[t]));
    }
    double fv[4];
    double rk[2] = {0, 0}, rg[2] = {0, 0}, ra[2] = {0, 0};
    const int nslots = 61 * nint;
#pragma unroll
    for (int m = 0; m < 4; m++) {
        const int s = lane + 32 * m;
        fv[m] = 0.0;
        if (s < nslots) {
            const int t = s >= 61 ? 1 : 0;
            const int j = s - 61 * t;
            const double x = __dadd_rn(c[t], __dmul_rn(h[t], N.x[j]));
            const double v = f(x);
            fv[m] = v;
            if (t == 0) { rk[0] += N.wk[j] * v; rg[0] += N.wg[j] * v; ra[0] += N.wk[j] * fabs(v); }
            else { rk[1] += N.wk[j] * v; rg[1] += N.wg[j] * v; ra[1] += N.wk[j] * fabs(v); }
        }
    }
    double mean[2];
    for (int t = 0; t < nint; t++) {
        rk[t] = bcast0(warp_sum_to0(rk[t]));
        rg[t] = bcast0(warp_sum_to0(rg[t]));
        ra[t] = bcast0(warp_sum_to0(ra[t]));
        mean[t] = 0.5 * rk[t];
    }
    double rs[2] = {0, 0};
#pragma unroll
    for (int m = 0; m < 4; m++) {
        const int s = lane + 32 * m;
        if (s < nslots) {
            const int t = s >= 61 ? 1 : 0;
            const int j = s - 61 * t;
            const double d = N.wk[j] * fabs(fv[m] - mean[t]);
            if (t == 0) rs[0] += d; else rs[1] += d;
        }
    }
    for (int t = 0; t < nint; t++) {
        rs[t] = bcast0(warp_sum_to0(rs[t]));
        const double err = (rk[t] - rg[t]) * h[t];
        out[t].result = rk[t] * h[t];
        out[t].resabs = ra[t] * fabs(h[t]);
        out[t].resasc = rs[t] * fabs(h[t]);
        out[t].abserr = rescale_error(err, out[t].resabs, out[t].resasc);
    }
}

struct QagList {  // per-warp interval list in shared memory
    double a[kQagLimit], b[kQagLimit], r[kQagLimit], e[kQagLimit];
    int slot[kQagLimit];  // node-cache slot of the interval (-1: not cached)
};

struct QagResult { double result, abserr; int ok; int nint; };

// QUADPACK QAG (Piessens et al. 1983) with the 61-point rule, run by one warp:
// bisect the interval with the largest error estimate until the summed error is
// below max(epsabs, epsrel |area|); QUADPACK's round-off and tiny-interval checks.
// Same decisions as the GSL-based reference path (delta_tot_table.c:404,597).
template <class F>
__device__ QagResult qag_warp(const F& f, const Gk61Nodes& N, QagList& L, double a, double b, double epsabs,
                              double epsrel, int limit) {
    const int lane = threadIdx.x & 31;
    QagResult R;
    GkOut g[2];
    double aa[2] = {a, a}, bb[2] = {b, b};
    gk61_warp(f, N, 1, aa, bb, g);
    if (lane == 0) { L.a[0] = a; L.b[0] = b; L.r[0] = g[0].result; L.e[0] = g[0].abserr; }
    __syncwarp();
    double tol = fmax(epsabs, epsrel * fabs(g[0].result));
    const double round_off = 50 * DBL_EPSILON * g[0].resabs;
    R.nint = 1;
    R.result = g[0].result;
    R.abserr = g[0].abserr;
    if (g[0].abserr <= round_off && g[0].abserr > tol) { R.ok = 0; return R; }
    if ((g[0].abserr <= tol && g[0].abserr != g[0].resasc) || g[0].abserr == 0.0) { R.ok = 1; return R; }
    if (limit == 1) { R.ok = 0; return R; }
    double area = g[0].result, errsum = g[0].abserr;
    int n = 1, roundoff1 = 0, roundoff2 = 0, error_type = 0;
    do {
        // argmax of the error list (lowest index on ties)
        const int bk = warp_argmax_err(L.e, n);
        const int k = bk;
        const double a_i = L.a[k], b_i = L.b[k], r_i = L.r[k], e_i = L.e[k];
        const double a1 = a_i, b1 = 0.5 * (a_i + b_i), a2 = b1, b2 = b_i;
        aa[0] = a1; bb[0] = b1; aa[1] = a2; bb[1] = b2;
        gk61_warp(f, N, 2, aa, bb, g);
        const double area12 = g[0].result + g[1].result, error12 = g[0].abserr + g[1].abserr;
        errsum += error12 - e_i;
        area += area12 - r_i;
        if (g[0].resasc != g[0].abserr && g[1].resasc != g[1].abserr) {
            if (fabs(r_i - area12) <= 1.0e-5 * fabs(area12) && error12 >= 0.99 * e_i) roundoff1++;
            if (n >= 10 && error12 > e_i) roundoff2++;
        }
        tol = fmax(epsabs, epsrel * fabs(area));
        if (errsum > tol) {
            if (roundoff1 >= 6 || roundoff2 >= 20) error_type = 2;
            const double tiny = (1 + 100 * DBL_EPSILON) * (fabs(a2) + 1000 * DBL_MIN);
            if (fabs(a1) <= tiny && fabs(b2) <= tiny) error_type = 3;
        }
        __syncwarp();
        if (lane == 0) {
            L.b[k] = b1; L.r[k] = g[0].result; L.e[k] = g[0].abserr;
            L.a[n] = a2; L.b[n] = b2; L.r[n] = g[1].result; L.e[n] = g[1].abserr;
        }
        __syncwarp();
        n++;
    } while (n < limit && !error_type && errsum > tol);
    double sum = 0;
    if (lane == 0)
        for (int i = 0; i < n; i++) sum += L.r[i];
    R.result = bcast0(sum);
    R.abserr = errsum;
    R.nint = n;
    R.ok = errsum <= tol;
    __syncwarp();
    return R;
}
// ------------------------------------------------------------------ cached QAG
// QAG only ever bisects, so its intervals are dyadic subintervals of [a, b].  For the
// delta_nu integral it refines toward the upper end (log a, where J -> 1 and the newest
// history rows are): at every depth the intervals it evaluates are the two children of
// the rightmost interval of the depth above.  Those are numbered: slot 0 = [a, b]; at
// depth d >= 1, slot 2d-1 the left and slot 2d the right child of the depth-(d-1)
// rightmost interval.  A functor with node(slot, j, x) may serve the 61 nodes of such an
// interval from a table built once; the others pass slot -1.
constexpr int kNcMaxLevels = 12;
constexpr int kNcMaxSlots = 1 + 2 * kNcMaxLevels;  // 25 intervals
constexpr int kNcNodes = kNcMaxSlots * 61;         // capacity of a node table

// child slot of s (right = 0, 1) in a table of nslots = 1 + 2 levels slots
__device__ __forceinline__ int nc_child(int s, int right, int nslots) {
    if (s < 0 || (s > 0 && (s & 1))) return -1;  // only the rightmost intervals have cached children
    const int d = s / 2 + 1;                      // depth of the children
    const int c = 2 * d - 1 + right;
    return c < nslots ? c : -1;
}

// The GK61 sums of one or two intervals from the node values of a warp (lane holds the
// values of slots lane, lane+32, lane+64, lane+96; slot s is node s%61 of interval s/61),
// and the rule's outputs, identical on every lane.  The six sums (Kronrod, Gauss and
// |f| sums of both intervals) are reduced together by a butterfly that halves the set of
// values each lane carries at every step (9 additions per lane instead of 30), then
// resasc's two sums likewise (5 instead of 10); the results are broadcast.
__device__ __forceinline__ void gk61_lane_sums(const Gk61Nodes& N, const double* fv, int nslots, int nint,
                                               const double* h, GkOut* out) {
    const int lane = threadIdx.x & 31;
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // rk0 rg0 ra0 - rk1 rg1 ra1 -
#pragma unroll
    for (int m = 0; m < 4; m++) {
        const int s = lane + 32 * m;
        if (s < nslots) {
            const int t = s >= 61 ? 1 : 0;
            const int j = s - 61 * t;
            const double x = fv[m];
            if (t == 0) { v[0] += N.wk[j] * x; v[1] += N.wg[j] * x; v[2] += N.wk[j] * fabs(x); }
            else { v[4] += N.wk[j] * x; v[5] += N.wg[j] * x; v[6] += N.wk[j] * fabs(x); }
        }
    }
    // value q ends in lanes with bits (4, 3, 2) = (q >> 2, (q >> 1) & 1, q & 1)
    const int b4 = (lane >> 4) & 1, b3 = (lane >> 3) & 1, b2 = (lane >> 2) & 1;
    double w[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const double keep = b4 ? v[4 + k] : v[k], give = b4 ? v[k] : v[4 + k];
        w[k] = keep + __shfl_xor_sync(0xffffffffu, give, 16);
    }
    double x2[2];
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const double keep = b3 ? w[2 + k] : w[k], give = b3 ? w[k] : w[2 + k];
        x2[k] = keep + __shfl_xor_sync(0xffffffffu, give, 8);
    }
    double y;
    {
        const double keep = b2 ? x2[1] : x2[0], give = b2 ? x2[0] : x2[1];
        y = keep + __shfl_xor_sync(0xffffffffu, give, 4);
    }
    y += __shfl_xor_sync(0xffffffffu, y, 2);
    y += __shfl_xor_sync(0xffffffffu, y, 1);
    const double rk0 = __shfl_sync(0xffffffffu, y, 0), rk1 = __shfl_sync(0xffffffffu, y, 16);
    const double mean[2] = {0.5 * rk0, 0.5 * rk1};
    double rs[2] = {0, 0};
#pragma unroll
    for (int m = 0; m < 4; m++) {
        const int s = lane + 32 * m;
        if (s < nslots) {
            const int t = s >= 61 ? 1 : 0;
            const int j = s - 61 * t;
            const double d = N.wk[j] * fabs(fv[m] - mean[t]);
            if (t == 0) rs[0] += d; else rs[1] += d;
        }
    }
    double z = (b4 ? rs[1] : rs[0]) + __shfl_xor_sync(0xffffffffu, b4 ? rs[0] : rs[1], 16);
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) z += __shfl_xor_sync(0xffffffffu, z, o);
    // the outputs of interval t on lane t only (FP64 is issued per active lane), then
    // broadcast
    const int t = lane & 1;
    const double rgt = __shfl_sync(0xffffffffu, y, t ? 20 : 4);
    const double rat = __shfl_sync(0xffffffffu, y, t ? 24 : 8);
    const double rst = __shfl_sync(0xffffffffu, z, t ? 16 : 0);
    GkOut o = {0.0, 0.0, 0.0, 0.0};
    if (lane < nint) {
        const double ht = t ? h[1] : h[0];
        const double rkt = t ? rk1 : rk0;
        o.result = rkt * ht;
        o.resabs = rat * fabs(ht);
        o.resasc = rst * fabs(ht);
        o.abserr = rescale_error((rkt - rgt) * ht, o.resabs, o.resasc);
    }
    for (int u = 0; u < nint; u++) {
        out[u].result = __shfl_sync(0xffffffffu, o.result, u);
        out[u].resabs = __shfl_sync(0xffffffffu, o.resabs, u);
        out[u].resasc = __shfl_sync(0xffffffffu, o.resasc, u);
        out[u].abserr = __shfl_sync(0xffffffffu, o.abserr, u);
    }
}

// gk61_warp with interval slots (same arithmetic)
template <class F>
__device__ __forceinline__ void gk61_warp_c(const F& f, const Gk61Nodes& N, int nint, const double* a,
                                            const double* b, const int* slot, GkOut* out) {
    const int lane = threadIdx.x & 31;
    // the intervals' geometry on lane 0, broadcast (FP64 is issued per active lane)
    double c[2] = {0.0, 0.0}, h[2] = {0.0, 0.0};
    if (lane == 0) {
        for (int t = 0; t < 2; t++) {
            c[t] = __dmul_rn(0.5, __dadd_rn(a[t], b[t]));
            h[t] = __dmul_rn(0.5, __dsub_rn(b[t], a[t]));
        }
    }
#pragma unroll
    for (int t = 0; t < 2; t++) {
        c[t] = __shfl_sync(0xffffffffu, c[t], 0);
        h[t] = __shfl_sync(0xffffffffu, h[t], 0);
    }
    double fv[4];
    const int nslots = 61 * nint;
#pragma unroll
    for (int m = 0; m < 4; m++) {
        const int s = lane + 32 * m;
        fv[m] = 0.0;
        if (s < nslots) {
            const int t = s >= 61 ? 1 : 0;
            const int j = s - 61 * t;
            fv[m] = f.node_at(slot[t], j, c[t], h[t], N.x[j]);
        }
    }
    gk61_lane_sums(N, fv, nslots, nint, h, out);
}

// qag_warp with interval slots (same decisions)
template <class F>
__device__ QagResult qag_warp_c(const F& f, const Gk61Nodes& N, QagList& L, double a, double b, double epsabs,
                                double epsrel, int limit) {
    const int lane = threadIdx.x & 31;
    QagResult R;
    GkOut g[2];
    double aa[2] = {a, a}, bb[2] = {b, b};
    int ss[2] = {f.nc.nslots > 0 ? 0 : -1, -1};
    gk61_warp_c(f, N, 1, aa, bb, ss, g);
    if (lane == 0) { L.a[0] = a; L.b[0] = b; L.r[0] = g[0].result; L.e[0] = g[0].abserr; L.slot[0] = ss[0]; }
    __syncwarp();
    double tol = fmax(epsabs, epsrel * fabs(g[0].result));
    const double round_off = 50 * DBL_EPSILON * g[0].resabs;
    R.nint = 1;
    R.result = g[0].result;
    R.abserr = g[0].abserr;
    if (g[0].abserr <= round_off && g[0].abserr > tol) { R.ok = 0; return R; }
    if ((g[0].abserr <= tol && g[0].abserr != g[0].resasc) || g[0].abserr == 0.0) { R.ok = 1; return R; }
    if (limit == 1) { R.ok = 0; return R; }
    double area = g[0].result, errsum = g[0].abserr;
    int n = 1, roundoff1 = 0, roundoff2 = 0, error_type = 0, cont = 0;
    do {
        const int bk = warp_argmax_err(L.e, n);
        const int k = bk;
        const double a_i = L.a[k], b_i = L.b[k], r_i = L.r[k], e_i = L.e[k];
        const int s_i = L.slot[k];
        const double a1 = a_i, b1 = 0.5 * (a_i + b_i), a2 = b1, b2 = b_i;
        aa[0] = a1; bb[0] = b1; aa[1] = a2; bb[1] = b2;
        ss[0] = nc_child(s_i, 0, f.nc.nslots);
        ss[1] = nc_child(s_i, 1, f.nc.nslots);
        gk61_warp_c(f, N, 2, aa, bb, ss, g);
        // QUADPACK's bookkeeping on lane 0 (its FP64 is not repeated on 32 lanes)
        cont = 0;
        __syncwarp();
        if (lane == 0) {
            const double area12 = g[0].result + g[1].result, error12 = g[0].abserr + g[1].abserr;
            errsum += error12 - e_i;
            area += area12 - r_i;
            if (g[0].resasc != g[0].abserr && g[1].resasc != g[1].abserr) {
                if (fabs(r_i - area12) <= 1.0e-5 * fabs(area12) && error12 >= 0.99 * e_i) roundoff1++;
                if (n >= 10 && error12 > e_i) roundoff2++;
            }
            tol = fmax(epsabs, epsrel * fabs(area));
            if (errsum > tol) {
                if (roundoff1 >= 6 || roundoff2 >= 20) error_type = 2;
                const double tiny = (1 + 100 * DBL_EPSILON) * (fabs(a2) + 1000 * DBL_MIN);
                if (fabs(a1) <= tiny && fabs(b2) <= tiny) error_type = 3;
            }
            L.b[k] = b1; L.r[k] = g[0].result; L.e[k] = g[0].abserr; L.slot[k] = ss[0];
            L.a[n] = a2; L.b[n] = b2; L.r[n] = g[1].result; L.e[n] = g[1].abserr; L.slot[n] = ss[1];
            cont = n + 1 < limit && !error_type && errsum > tol;
        }
        cont = __shfl_sync(0xffffffffu, cont, 0);
        __syncwarp();
        n++;
    } while (cont);
    double sum = 0;
    if (lane == 0)
        for (int i = 0; i < n; i++) sum += L.r[i];
    R.result = bcast0(sum);
    R.abserr = bcast0(errsum);
    R.nint = n;
    R.ok = __shfl_sync(0xffffffffu, (int)(errsum <= tol), 0);
    __syncwarp();
    return R;
}

// ------------------------------------------------------------------ block-cooperative QAG
// The same rule and decisions with the node evaluations spread over the warps of a block
// (blockDim.x = 32 * W, W = 2 or 4): thread t evaluates slot t, t + 32W, ...; warp 0
// then forms every lane's partial sums over the slots lane + 32m in the order m = 0..3
// and reduces them with the butterfly of gk61_warp_c: the arithmetic of qag_warp_c in
// the same order (the compiler may contract multiply-adds differently per kernel, so the
// results agree to the last bits).  Shared scratch: QagBlockSmem.
struct QagBlockSmem {
    double fv[128];
    GkOut out[2];
    double a[2], b[2];
    int slot[2];
    int k, cont, ok;   // the interval to bisect, whether to go on, errsum <= tol
    double errsum;
};

template <class F>
__device__ __forceinline__ void gk61_block_c(const F& f, const Gk61Nodes& N, int nint, const double* a,
                                             const double* b, const int* slot, GkOut* out, QagBlockSmem& sh) {
    const int tid = threadIdx.x, lane = tid & 31;
    double c[2], h[2];
    for (int t = 0; t < 2; t++) {
        c[t] = __dmul_rn(0.5, __dadd_rn(a[t], b[t]));
        h[t] = __dmul_rn(0.5, __dsub_rn(b[t], a[t]));
    }
    const int nslots = 61 * nint;
    for (int s = tid; s < nslots; s += blockDim.x) {
        const int t = s >= 61 ? 1 : 0;
        const int j = s - 61 * t;
        sh.fv[s] = f.node_at(slot[t], j, c[t], h[t], N.x[j]);
    }
    __syncthreads();
    if (tid < 32) {  // warp 0: the sums exactly as gk61_warp_c forms them
        double fv[4];
#pragma unroll
        for (int m = 0; m < 4; m++) {
            const int s = lane + 32 * m;
            fv[m] = s < nslots ? sh.fv[s] : 0.0;
        }
        GkOut o[2];
        gk61_lane_sums(N, fv, nslots, nint, h, o);
        if (lane < nint) sh.out[lane] = o[lane];
    }
    __syncthreads();
    for (int t = 0; t < nint; t++) out[t] = sh.out[t];
}

// qag_warp_c run by a whole block: every thread follows the same decisions (they read the
// same shared list); thread 0 writes the list.
template <class F>
__device__ QagResult qag_block_c(const F& f, const Gk61Nodes& N, QagList& L, double a, double b, double epsabs,
                                 double epsrel, int limit, QagBlockSmem& sh) {
    const int tid = threadIdx.x, lane = tid & 31;
    QagResult R;
    GkOut g[2];
    double aa[2] = {a, a}, bb[2] = {b, b};
    int ss[2] = {f.nc.nslots > 0 ? 0 : -1, -1};
    gk61_block_c(f, N, 1, aa, bb, ss, g, sh);
    if (tid == 0) { L.a[0] = a; L.b[0] = b; L.r[0] = g[0].result; L.e[0] = g[0].abserr; L.slot[0] = ss[0]; }
    __syncthreads();
    double tol = fmax(epsabs, epsrel * fabs(g[0].result));
    const double round_off = 50 * DBL_EPSILON * g[0].resabs;
    R.nint = 1;
    R.result = g[0].result;
    R.abserr = g[0].abserr;
    if (g[0].abserr <= round_off && g[0].abserr > tol) { R.ok = 0; return R; }
    if ((g[0].abserr <= tol && g[0].abserr != g[0].resasc) || g[0].abserr == 0.0) { R.ok = 1; return R; }
    if (limit == 1) { R.ok = 0; return R; }
    double area = g[0].result, errsum = g[0].abserr;
    int n = 1, roundoff1 = 0, roundoff2 = 0, error_type = 0;
    do {
        // warp 0 finds the interval of largest error (lowest index on ties)
        if (tid < 32) {
            const int bk = warp_argmax_err(L.e, n);
            if (lane == 0) sh.k = bk;
        }
        __syncthreads();
        const int k = sh.k;
        const double a_i = L.a[k], b_i = L.b[k], r_i = L.r[k], e_i = L.e[k];
        const int s_i = L.slot[k];
        const double a1 = a_i, b1 = 0.5 * (a_i + b_i), a2 = b1, b2 = b_i;
        aa[0] = a1; bb[0] = b1; aa[1] = a2; bb[1] = b2;
        ss[0] = nc_child(s_i, 0, f.nc.nslots);
        ss[1] = nc_child(s_i, 1, f.nc.nslots);
        gk61_block_c(f, N, 2, aa, bb, ss, g, sh);
        // QUADPACK's bookkeeping on thread 0
        if (tid == 0) {
            const double area12 = g[0].result + g[1].result, error12 = g[0].abserr + g[1].abserr;
            errsum += error12 - e_i;
            area += area12 - r_i;
            if (g[0].resasc != g[0].abserr && g[1].resasc != g[1].abserr) {
                if (fabs(r_i - area12) <= 1.0e-5 * fabs(area12) && error12 >= 0.99 * e_i) roundoff1++;
                if (n >= 10 && error12 > e_i) roundoff2++;
            }
            tol = fmax(epsabs, epsrel * fabs(area));
            if (errsum > tol) {
                if (roundoff1 >= 6 || roundoff2 >= 20) error_type = 2;
                const double tiny = (1 + 100 * DBL_EPSILON) * (fabs(a2) + 1000 * DBL_MIN);
                if (fabs(a1) <= tiny && fabs(b2) <= tiny) error_type = 3;
            }
            L.b[k] = b1; L.r[k] = g[0].result; L.e[k] = g[0].abserr; L.slot[k] = ss[0];
            L.a[n] = a2; L.b[n] = b2; L.r[n] = g[1].result; L.e[n] = g[1].abserr; L.slot[n] = ss[1];
            sh.cont = n + 1 < limit && !error_type && errsum > tol;
            sh.errsum = errsum;
            sh.ok = errsum <= tol;
        }
        __syncthreads();
        n++;
    } while (sh.cont);
    double sum = 0;
    if (lane == 0)
        for (int i = 0; i < n; i++) sum += L.r[i];
    R.result = bcast0(sum);
    R.abserr = sh.errsum;
    R.nint = n;
    R.ok = sh.ok;
    __syncthreads();
    return R;
}

// ------------------------------------------------------------------ block QAG with look-ahead
// qag_block_c with one level of look-ahead.  On these integrands QAG nearly always
// bisects next the right half it has just made (the late-time end, where delta_tot and
// the free-streaming kernel change fastest).  A round that evaluates the halves of
// interval k therefore also evaluates the halves of k's right half; when the next round
// picks that half, its rule results are already there and the round is bookkeeping only,
// so the sequential evaluation rounds are halved.  Node values come from the same
// node_at, and each interval's sums are formed by one warp in the lane layout of a
// two-interval gk61_block_c call, so every rule result is that of qag_block_c (to the
// last bits, which the compiler's multiply-add contraction may change from kernel to
// kernel) and so is every decision.  blockDim.x = 256: the 244 node slots of a round in
// one pass.  Shared scratch: QagSpecSmem.
struct QagSpecSmem {
    double fv[244];  // group A: slots [0, 122), group B: [122, 244)
    GkOut out[4];    // group A intervals 0, 1 | group B intervals 0, 1
    GkOut pg[2];     // rule results of the halves of list entry pre_k
    double ic[4], ih[4];  // centre and half-width of the intervals of the next evaluation
    int isl[4];           // and their node-table slots
    int k, hit, cont, ok, pre_k;
    double errsum;
};

// The geometry of interval q of the next evaluation, formed once (one thread) as every
// GK61 call forms it: c = (a + b) / 2, h = (b - a) / 2.
__device__ __forceinline__ void spec_set_interval(QagSpecSmem& sh, int q, double a, double b, int slot) {
    sh.ic[q] = __dmul_rn(0.5, __dadd_rn(a, b));
    sh.ih[q] = __dmul_rn(0.5, __dsub_rn(b, a));
    sh.isl[q] = slot;
}

// Rule results of two groups of intervals, nA in {1, 2} (intervals 0, 1) and nB in
// {0, 1, 2} (intervals 2, 3), whose geometry is in sh.ic / sh.ih / sh.isl.  Warp 0 sums
// group A, warp 1 group B, each as gk61_block_c sums a call of that many intervals.
template <class F>
__device__ __forceinline__ void gk61_block_groups(const F& f, const Gk61Nodes& N, int nA, int nB, QagSpecSmem& sh) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int s = tid; s < 244; s += blockDim.x) {
        const int g = s >= 122 ? 1 : 0;
        const int u = s - 122 * g;
        const int t = u >= 61 ? 1 : 0;
        const int j = u - 61 * t;
        if (t < (g ? nB : nA)) {
            const int q = 2 * g + t;
            sh.fv[s] = f.node_at(sh.isl[q], j, sh.ic[q], sh.ih[q], N.x[j]);
        }
    }
    __syncthreads();
    const int ng = warp == 0 ? nA : (warp == 1 ? nB : 0);
    if (ng > 0) {  // warp-uniform
        const double* fvg = sh.fv + 122 * warp;
        double fv[4];
#pragma unroll
        for (int m = 0; m < 4; m++) {
            const int sl = lane + 32 * m;
            fv[m] = sl < 61 * ng ? fvg[sl] : 0.0;
        }
        const double hh[2] = {sh.ih[2 * warp], sh.ih[2 * warp + 1]};
        GkOut o[2];
        gk61_lane_sums(N, fv, 61 * ng, ng, hh, o);
        if (lane == 0) {
            sh.out[2 * warp] = o[0];
            if (ng > 1) sh.out[2 * warp + 1] = o[1];
        }
    }
    __syncthreads();
}

template <class F>
__device__ QagResult qag_block_spec_c(const F& f, const Gk61Nodes& N, QagList& L, double a, double b, double epsabs,
                                      double epsrel, int limit, QagSpecSmem& sh) {
    const int tid = threadIdx.x, lane = tid & 31;
    const int ns = f.nc.nslots;
    QagResult R;
    const int s0 = ns > 0 ? 0 : -1;
    if (tid == 0) {  // the root, and its halves ahead
        const double m = 0.5 * (a + b);
        spec_set_interval(sh, 0, a, b, s0);
        spec_set_interval(sh, 2, a, m, nc_child(s0, 0, ns));
        spec_set_interval(sh, 3, m, b, nc_child(s0, 1, ns));
    }
    __syncthreads();
    gk61_block_groups(f, N, 1, 2, sh);
    const GkOut g0 = sh.out[0];
    if (tid == 0) {
        L.a[0] = a; L.b[0] = b; L.r[0] = g0.result; L.e[0] = g0.abserr; L.slot[0] = s0;
        sh.pre_k = 0; sh.pg[0] = sh.out[2]; sh.pg[1] = sh.out[3];
    }
    __syncthreads();
    double tol = fmax(epsabs, epsrel * fabs(g0.result));
    const double round_off = 50 * DBL_EPSILON * g0.resabs;
    R.nint = 1;
    R.result = g0.result;
    R.abserr = g0.abserr;
    if (g0.abserr <= round_off && g0.abserr > tol) { R.ok = 0; return R; }
    if ((g0.abserr <= tol && g0.abserr != g0.resasc) || g0.abserr == 0.0) { R.ok = 1; return R; }
    if (limit == 1) { R.ok = 0; return R; }
    double area = g0.result, errsum = g0.abserr;
    int n = 1, roundoff1 = 0, roundoff2 = 0, error_type = 0;
    do {
        // warp 0 finds the interval of largest error (lowest index on ties); its lane 0
        // notes whether the halves are already evaluated and, if not, lays out the halves
        // of k and of k's right half
        if (tid < 32) {
            const int bk = warp_argmax_err(L.e, n);
            if (lane == 0) {
                const bool hit = bk == sh.pre_k;
                sh.k = bk;
                sh.hit = hit;
                if (!hit) {
                    const double a_i = L.a[bk], b_i = L.b[bk];
                    const int s_i = L.slot[bk];
                    const double b1 = 0.5 * (a_i + b_i);
                    const double m2 = 0.5 * (b1 + b_i);
                    const int c1 = nc_child(s_i, 1, ns);
                    spec_set_interval(sh, 0, a_i, b1, nc_child(s_i, 0, ns));
                    spec_set_interval(sh, 1, b1, b_i, c1);
                    spec_set_interval(sh, 2, b1, m2, nc_child(c1, 0, ns));
                    spec_set_interval(sh, 3, m2, b_i, nc_child(c1, 1, ns));
                }
            }
        }
        __syncthreads();
        const int k = sh.k;
        if (!sh.hit) gk61_block_groups(f, N, 2, 2, sh);  // block-uniform
        // QUADPACK's bookkeeping on thread 0
        if (tid == 0) {
            const bool hit = sh.hit;
            const double a_i = L.a[k], b_i = L.b[k], r_i = L.r[k], e_i = L.e[k];
            const int s_i = L.slot[k];
            const double a1 = a_i, b1 = 0.5 * (a_i + b_i), a2 = b1, b2 = b_i;
            const GkOut g[2] = {hit ? sh.pg[0] : sh.out[0], hit ? sh.pg[1] : sh.out[1]};
            const double area12 = g[0].result + g[1].result, error12 = g[0].abserr + g[1].abserr;
            errsum += error12 - e_i;
            area += area12 - r_i;
            if (g[0].resasc != g[0].abserr && g[1].resasc != g[1].abserr) {
                if (fabs(r_i - area12) <= 1.0e-5 * fabs(area12) && error12 >= 0.99 * e_i) roundoff1++;
                if (n >= 10 && error12 > e_i) roundoff2++;
            }
            tol = fmax(epsabs, epsrel * fabs(area));
            if (errsum > tol) {
                if (roundoff1 >= 6 || roundoff2 >= 20) error_type = 2;
                const double tiny = (1 + 100 * DBL_EPSILON) * (fabs(a2) + 1000 * DBL_MIN);
                if (fabs(a1) <= tiny && fabs(b2) <= tiny) error_type = 3;
            }
            L.b[k] = b1; L.r[k] = g[0].result; L.e[k] = g[0].abserr; L.slot[k] = nc_child(s_i, 0, ns);
            L.a[n] = a2; L.b[n] = b2; L.r[n] = g[1].result; L.e[n] = g[1].abserr; L.slot[n] = nc_child(s_i, 1, ns);
            if (hit) {
                sh.pre_k = -1;
            } else {
                sh.pre_k = n;
                sh.pg[0] = sh.out[2];
                sh.pg[1] = sh.out[3];
            }
            sh.cont = n + 1 < limit && !error_type && errsum > tol;
            sh.errsum = errsum;
            sh.ok = errsum <= tol;
        }
        __syncthreads();
        n++;
    } while (sh.cont);
    double sum = 0;
    if (lane == 0)
        for (int i = 0; i < n; i++) sum += L.r[i];
    R.result = bcast0(sum);
    R.abserr = sh.errsum;
    R.nint = n;
    R.ok = sh.ok;
    __syncthreads();
    return R;
}

}  // namespace ksp
#include "ksp_jfit.cuh"
namespace ksp {

// ------------------------------------------------------------------ delta_nu integrand
// delta_tot_table.c:492-500: fslength(x, log a) / (a H(a)) J(k fslength / (m/kT))
// delta_tot(k, x) at x = log a_i.  Split into the part that depends only on x (and the
// instance), NodeTerms, and the per-bin rest.
struct NodeTerms {
    double g;    // fslength / (a H(a))
    double fsl;  // fslength(x, log a)
    double dx;   // x - knot[j]
    int j;       // history segment: knot[j] <= x < knot[j+1]
};

// Not inlined: the table builder and the uncached path run the same compiled code and
// produce the same numbers bit for bit.
static __device__ __noinline__ NodeTerms dnu_node_terms(const Background* B, const double* fs_x, const double* fs_y,
                                                 const double* fs_c, int nfs, double fs_x0, double fs_inv,
                                                 const double* kx, int na, double x) {
    NodeTerms t;
    int i = (int)((x - fs_x0) * fs_inv);
    i = i < 0 ? 0 : (i > nfs - 2 ? nfs - 2 : i);
    while (i > 0 && x < fs_x[i]) i--;
    while (i < nfs - 2 && x >= fs_x[i + 1]) i++;
    {
        const double x0 = fs_x[i], x1 = fs_x[i + 1];
        const double y0 = fs_y[i], y1 = fs_y[i + 1];
        const double c0 = fs_c[i], c1 = fs_c[i + 1];
        const double h = x1 - x0, dx = x - x0;
        const double bq = (y1 - y0) / h - h * (c1 + 2.0 * c0) / 3.0;
        const double d = (c1 - c0) / (3.0 * h);
        t.fsl = y0 + dx * (bq + dx * (c0 + dx * d));
    }
    t.j = seg_bsearch(kx, na, x);
    t.dx = x - kx[t.j];
    const double ai = exp(x);
    t.g = t.fsl / (ai * hubble(*B, ai));
    return t;
}

// Per-segment constants of the history knots: 1/h, h/3, 1/(3h).
struct KnotSeg {
    const double* ih;
    const double* h3;
    const double* ih3;
};

// The history row's natural spline (or linear for 2 knots) at a node.
__device__ __forceinline__ double dnu_S(const NodeTerms& t, const double* ky, const double* kc, int na,
                                        const KnotSeg& ks) {
    const int j = t.j;
    const double y0 = ky[j], y1 = ky[j + 1];
    if (na > 2) {
        const double c0 = kc[j], c1 = kc[j + 1];
        const double bq = (y1 - y0) * __ldg(ks.ih + j) - (c1 + 2.0 * c0) * __ldg(ks.h3 + j);
        const double d = (c1 - c0) * __ldg(ks.ih3 + j);
        return y0 + t.dx * (bq + t.dx * (c0 + t.dx * d));
    }
    return y0 + t.dx * ((y1 - y0) * __ldg(ks.ih + j));
}

// The node-independent part of dnu_S per segment of a history row, computed once per
// (row, call) into sb / sd by threads t, t+nt, ...: the same expressions as dnu_S, so
// that dnu_S_poly returns the same values with three FMAs per node.
__device__ __forceinline__ void seg_poly(const double* ky, const double* kc, int na, const KnotSeg& ks, double* sb,
                                         double* sd, int t, int nt) {
    for (int j = t; j < na - 1; j += nt) {
        const double y0 = ky[j], y1 = ky[j + 1], c0 = kc[j], c1 = kc[j + 1];
        sb[j] = (y1 - y0) * __ldg(ks.ih + j) - (c1 + 2.0 * c0) * __ldg(ks.h3 + j);
        sd[j] = (c1 - c0) * __ldg(ks.ih3 + j);
    }
}
__device__ __forceinline__ double dnu_S_poly(const NodeTerms& t, const double* ky, const double* kc,
                                             const double* sb, const double* sd, int na, const KnotSeg& ks) {
    const int j = t.j;
    if (na > 2) return ky[j] + t.dx * (sb[j] + t.dx * (kc[j] + t.dx * sd[j]));
    return ky[j] + t.dx * ((ky[j + 1] - ky[j]) * __ldg(ks.ih + j));
}

// The per-bin rest: J and the history row's natural spline (or linear for 2 knots) at
// the node.  Same for the cached and uncached paths.
// k_over_m = k / (m / kT): J's argument is fslength * k_over_m (one division per bin
// instead of one per node).
__device__ __forceinline__ double dnu_combine(const NodeTerms& t, double k_over_m, double qc, double nfl,
                                              const double* ky, const double* kc, const double* sb,
                                              const double* sd, int na, const KnotSeg& ks) {
    const double S = dnu_S_poly(t, ky, kc, sb, sd, na, ks);
    const double J = specialJ_tab(t.fsl * k_over_m, qc, nfl);
    return t.g * J * S;
}

// Node table of one instance for one call: nslots * 61 entries, slot-major.
struct NodeCache {
    double* g;
    double* fsl;
    double* dx;
    int* j;
    int nslots;
};

// The full integrand with the node table.
struct DnuIntegrandC {
    const Background* B;
    double k_over_m, qc, nfl;
    const double* fs_x; const double* fs_y; const double* fs_c; int nfs; double fs_x0, fs_inv;
    const double* kx; const double* ky; const double* kc; int na;
    const double* sb; const double* sd;  // seg_poly of (ky, kc)
    KnotSeg ks;
    NodeCache nc;
    __device__ double node(int slot, int jn, double x) const {
        NodeTerms t;
        if (slot >= 0) {
            const int q = slot * 61 + jn;
            t.g = __ldg(nc.g + q);
            t.fsl = __ldg(nc.fsl + q);
            t.dx = __ldg(nc.dx + q);
            t.j = __ldg(nc.j + q);
        } else {
            t = dnu_node_terms(B, fs_x, fs_y, fs_c, nfs, fs_x0, fs_inv, kx, na, x);
        }
        return dnu_combine(t, k_over_m, qc, nfl, ky, kc, sb, sd, na, ks);
    }
    // node jn of the interval with centre c and half-length h: x = c + h x_jn is needed
    // only where the node table has no entry
    __device__ double node_at(int slot, int jn, double c, double h, double xj) const {
        NodeTerms t;
        if (slot >= 0) {
            const int q = slot * 61 + jn;
            t.g = __ldg(nc.g + q);
            t.fsl = __ldg(nc.fsl + q);
            t.dx = __ldg(nc.dx + q);
            t.j = __ldg(nc.j + q);
        } else {
            t = dnu_node_terms(B, fs_x, fs_y, fs_c, nfs, fs_x0, fs_inv, kx, na, __dadd_rn(c, __dmul_rn(h, xj)));
        }
        return dnu_combine(t, k_over_m, qc, nfl, ky, kc, sb, sd, na, ks);
    }
    __device__ NodeTerms terms(int slot, int jn, double x) const {
        if (slot >= 0) {
            const int q = slot * 61 + jn;
            NodeTerms t;
            t.g = __ldg(nc.g + q);
            t.fsl = __ldg(nc.fsl + q);
            t.dx = __ldg(nc.dx + q);
            t.j = __ldg(nc.j + q);
            return t;
        }
        return dnu_node_terms(B, fs_x, fs_y, fs_c, nfs, fs_x0, fs_inv, kx, na, x);
    }
};

// Slot of the dyadic interval [a, b] of [lo, hi] in a node table of nslots slots (-1: not
// one of them), by the bisections QAG performs.
__device__ __forceinline__ int nc_slot_of(double a, double b, double lo, double hi, int nslots) {
    if (nslots <= 0) return -1;
    if (a == lo && b == hi) return 0;
    for (int d = 1; 2 * d < nslots + 1; d++) {
        const double m = 0.5 * (lo + hi);
        if (a == lo && b == m) return 2 * d - 1;
        if (a == m && b == hi) return 2 * d;
        lo = m;
    }
    return -1;
}

// Segmented sums over the lanes of a warp: runs of equal key (in lane order) are summed
// onto the run's last lane, for four values at once.
__device__ __forceinline__ void warp_seg_sum4(int key, double& a, double& b, double& c, double& d, bool& tail) {
    const int lane = threadIdx.x & 31;
    const int up = __shfl_up_sync(0xffffffffu, key, 1);
    const bool head = lane == 0 || up != key;
    const unsigned heads = __ballot_sync(0xffffffffu, head);
    const int my_head = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
#pragma unroll
    for (int dd = 1; dd < 32; dd <<= 1) {
        const double oa = __shfl_up_sync(0xffffffffu, a, dd), ob = __shfl_up_sync(0xffffffffu, b, dd);
        const double oc = __shfl_up_sync(0xffffffffu, c, dd), od = __shfl_up_sync(0xffffffffu, d, dd);
        if (lane - dd >= my_head) { a += oa; b += ob; c += oc; d += od; }
    }
    tail = lane == 31 || ((heads >> (lane + 1)) & 1u);
}

// End points of cache slot s of [a, b], by the bisections QAG performs (b1 = (a+b)/2).
__device__ __forceinline__ void nc_interval(int s, double a, double b, double* lo, double* hi) {
    if (s == 0) { *lo = a; *hi = b; return; }
    const int d = (s + 1) / 2;
    for (int k = 1; k < d; k++) a = 0.5 * (a + b);  // the rightmost interval of depth k
    const double m = 0.5 * (a + b);
    if (s & 1) { *lo = a; *hi = m; } else { *lo = m; *hi = b; }
}
#endif  // __CUDACC__

}  // namespace ksp
