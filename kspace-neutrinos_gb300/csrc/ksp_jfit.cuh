// ksp_jfit.cuh -- J(x) of the delta_nu integrand (delta_tot_table.c:417-428) evaluated
// from the piecewise polynomials of jfit_table.h (generated by gen_jtable.py): the
// octave and the top mantissa bits of x select a piece, nine FMAs evaluate it.  This
// replaces the FP64 log and exp of x^4.1811 (the FP64 rate of the GPU is 1/64 of
// FP32) at ~2e-16 relative accuracy.
#pragma once
#include <cuda_runtime.h>
#include "jfit_table.h"

namespace ksp {

static __device__ const double g_jfit[KSP_JFIT_PIECES * KSP_JFIT_STRIDE] = KSP_JFIT_TABLE_INIT;

__device__ __forceinline__ double specialJ_fit_tab(double x) {
    if (x <= 0.) return 1.;
    const long long bits = __double_as_longlong(x);
    const int e = (int)((bits >> 52) & 0x7ff) - 1023;
    if (e < KSP_JFIT_E0) {  // x < 2^-20: the x^4.1811 term is below 1e-25 relative
        const double x2 = x * x, x4 = x2 * x2, x8 = x4 * x4;
        return (1. + 0.0168 * x2 + 0.0407 * x4) / (1. + 2.1734 * x2 + 0.1467 * x8);
    }
    if (e >= KSP_JFIT_E1) return specialJ_fit(x);
    const int sub = (int)((bits >> (52 - KSP_JFIT_SUB_BITS)) & ((1 << KSP_JFIT_SUB_BITS) - 1));
    const double* p = g_jfit + (((e - KSP_JFIT_E0) << KSP_JFIT_SUB_BITS) | sub) * KSP_JFIT_STRIDE;
    const double u = (x - __ldg(p)) * __ldg(p + 1);
    double v = __ldg(p + 2 + KSP_JFIT_DEG);
#pragma unroll
    for (int j = KSP_JFIT_DEG - 1; j >= 0; j--) v = fma(v, u, __ldg(p + 2 + j));
    return v;
}

// specialJ (delta_tot_table.c:442-463) with the tabulated fit
__device__ __forceinline__ double specialJ_tab(double x, double qc, double nufrac_low) {
    return qc > 0 ? specialJ(x, qc, nufrac_low) : specialJ_fit_tab(x);
}

}  // namespace ksp
