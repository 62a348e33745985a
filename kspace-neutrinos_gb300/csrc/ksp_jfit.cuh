// ksp_jfit.cuh -- J(x) of the delta_nu integrand (delta_tot_table.c:417-428) evaluated
// from the piecewise polynomials of jfit_table.h (generated by gen_jtable.py): the
// octave and the top mantissa bits of x select a piece, a subtraction and seven FMAs
// evaluate it (the polynomial is stored in t = x - centre).  This
// replaces the FP64 log and exp of x^4.1811 (the FP64 rate of the GPU is 1/64 of
// FP32) at ~2e-16 relative accuracy.
#pragma once
#include <cuda_runtime.h>
#include "jfit_table.h"

namespace ksp {

static __device__ const double g_jfit[KSP_JFIT_PIECES * KSP_JFIT_STRIDE] = KSP_JFIT_TABLE_INIT;

__device__ __forceinline__ double specialJ_fit_tab(double x) {
    // x <= 0 tested on the bit pattern (+0 and the negatives are the non-positive
    // integers; a NaN, whatever its sign, goes on as the FP64 compare would let it), on
    // the integer pipe: an FP64 compare costs a warp the FP64 pipe's full time
    const long long bits = __double_as_longlong(x);
    if (bits <= 0 && (bits & 0x7fffffffffffffffLL) <= 0x7ff0000000000000LL) return 1.;
    const int e = (int)((bits >> 52) & 0x7ff) - 1023;
    if (e < KSP_JFIT_E0) {  // x < 2^-20: the x^4.1811 term is below 1e-25 relative
        const double x2 = x * x, x4 = x2 * x2, x8 = x4 * x4;
        return (1. + 0.0168 * x2 + 0.0407 * x4) / (1. + 2.1734 * x2 + 0.1467 * x8);
    }
    if (e >= KSP_JFIT_E1) return specialJ_fit(x);
    const int sub = (int)((bits >> (52 - KSP_JFIT_SUB_BITS)) & ((1 << KSP_JFIT_SUB_BITS) - 1));
    const double* p = g_jfit + (((e - KSP_JFIT_E0) << KSP_JFIT_SUB_BITS) | sub) * KSP_JFIT_STRIDE;
    const double t = x - __ldg(p);
    double v = __ldg(p + 1 + KSP_JFIT_DEG);
#pragma unroll
    for (int j = KSP_JFIT_DEG - 1; j >= 0; j--) v = fma(v, t, __ldg(p + 1 + j));
    return v;
}

// J and dJ/dx together (the adjoint): the derivative of the piece's polynomial, times
// du/dx; outside the table the formula and its derivative.
__device__ __forceinline__ void specialJ_fit_tab_d(double x, double& J, double& Jd) {
    const long long bits = __double_as_longlong(x);
    if (bits <= 0 && (bits & 0x7fffffffffffffffLL) <= 0x7ff0000000000000LL) { J = 1.; Jd = 0.; return; }
    const int e = (int)((bits >> 52) & 0x7ff) - 1023;
    if (e < KSP_JFIT_E0 || e >= KSP_JFIT_E1) {
        const double x2 = x * x, x4 = x2 * x2, x8 = x4 * x4;
        const double p = e < KSP_JFIT_E0 ? 0.0 : exp(4.1811 * log(x));
        const double N = 1. + 0.0168 * x2 + 0.0407 * x4;
        const double D = 1. + 2.1734 * x2 + 1.6787 * p + 0.1467 * x8;
        const double dN = 0.0336 * x + 0.1628 * x2 * x;
        const double dD = 4.3468 * x + 1.6787 * 4.1811 * p / x + 1.1736 * x4 * x2 * x;
        J = N / D;
        Jd = (dN * D - N * dD) / (D * D);
        return;
    }
    const int sub = (int)((bits >> (52 - KSP_JFIT_SUB_BITS)) & ((1 << KSP_JFIT_SUB_BITS) - 1));
    const double* p = g_jfit + (((e - KSP_JFIT_E0) << KSP_JFIT_SUB_BITS) | sub) * KSP_JFIT_STRIDE;
    const double t = x - __ldg(p);
    double v = __ldg(p + 1 + KSP_JFIT_DEG), dv = 0.0;
#pragma unroll
    for (int j = KSP_JFIT_DEG - 1; j >= 0; j--) {
        dv = fma(dv, t, v);
        v = fma(v, t, __ldg(p + 1 + j));
    }
    J = v;
    Jd = dv;
}

// specialJ (delta_tot_table.c:442-463) with the tabulated fit
__device__ __forceinline__ double specialJ_tab(double x, double qc, double nufrac_low) {
    return qc > 0 ? specialJ(x, qc, nufrac_low) : specialJ_fit_tab(x);
}

}  // namespace ksp
