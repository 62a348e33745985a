/* kspace_hubble_match.h -- shared by the drop-in layers (kspace_dropin.c,
 * kspace_delta_tot_table.c): identify the host's hubble_function with the GPU's
 * background model.
 *
 * The reference calls the host's hubble_function(a) (gadget_defines.h:11) inside its
 * integrals; the GPU evaluates H(a) itself.  First choice: the form H0 sqrt(Omega_nonu/a^3
 * + Omega_K/a^2 + Omega_L + Omega_nu(a) [+ Omega_g/a^4]) of the reference's test host and
 * of the Gadget-2 patch, with H0 = HUBBLE * UnitTime_in_s and Omega0 from the caller and
 * Omega_L, the curvature and the radiation term identified from the host function,
 * verified at 64 points from a_lo/2 to 2 to 1e-12 (then the GPU reproduces the host's
 * arithmetic).  Otherwise (another dark-energy model, other units or another neutrino
 * background in the host's H): the host function sampled at 4097 points uniform in log a
 * over [a_lo/2, max(2, 2 a_hi)], interpolated on the GPU as a cubic spline of log H,
 * verified between the samples of [a_lo, max(a_hi, 1)] to 1e-10.
 */
#ifndef KSPACE_HUBBLE_MATCH_H
#define KSPACE_HUBBLE_MATCH_H
#include <math.h>
#include "kspace_gpu.h"

#define KSP_HUBBLE_CGS 3.24077929e-18

double hubble_function(double a);

#define KSP_HTAB_N 4097

/* Returns KSPACE_OK, or KSPACE_ERR_HUBBLE with the best relative difference in *err. */
static int kspace_match_hubble(kspace_ctx *ctx, double Omega0, double UnitTime_in_s, double a_lo, double a_hi,
                               double *err)
{
    const double H0 = KSP_HUBBLE_CGS * UnitTime_in_s;
    double best_err = 1e300;
    int st;
    /* candidates: flat (Omega_L = 1 - Omega0) or curved with Omega_L from H(0.5);
     * radiation on or off */
    for (int rad = 1; rad >= 0; rad--) {
        for (int flat = 1; flat >= 0; flat--) {
            double OL = 1 - Omega0;
            if (!flat) {
                /* with Omega_K = 1 - Omega0 - OL: h^2 = flat_h^2 + (1 - Omega0 - OL)(1/a^2 - 1) at a = 0.5 */
                const double h1 = hubble_function(0.5) / H0;
                if ((st = kspace_gpu_set_hubble(ctx, Omega0, 1 - Omega0, UnitTime_in_s, rad)))
                    return st;
                double hm = 0;
                kspace_gpu_hubble(ctx, 0.5, &hm);
                hm /= H0;
                OL = 1 - Omega0 - (h1 * h1 - hm * hm) / 3.0;
            }
            if ((st = kspace_gpu_set_hubble(ctx, Omega0, OL, UnitTime_in_s, rad)))
                return st;
            double a[64], H[64], e = 0;
            for (int i = 0; i < 64; i++) {
                a[i] = exp(log(a_lo / 2) + i * (log(2.0) - log(a_lo / 2)) / 63);
                H[i] = hubble_function(a[i]);
            }
            kspace_gpu_check_hubble(ctx, a, H, 64, 1e-12, &e);
            if (e < best_err)
                best_err = e;
            if (e < 1e-12) {
                if (err)
                    *err = e;
                return KSPACE_OK;
            }
        }
    }
    /* the tabulated form */
    {
        static double H[KSP_HTAB_N];
        const double lo = log(a_lo / 2), hi = log(a_hi > 1.0 ? 2 * a_hi : 2.0);
        const double dx = (hi - lo) / (KSP_HTAB_N - 1);
        for (int i = 0; i < KSP_HTAB_N; i++)
            H[i] = hubble_function(exp(lo + i * dx));
        if ((st = kspace_gpu_set_hubble_table(ctx, lo, dx, KSP_HTAB_N, H)))
            return st;
        /* between samples over [a_lo, max(a_hi, 1)], where the integrals evaluate H (the
         * natural end conditions are least accurate in the margins beyond) */
        const int i0 = (int)((log(a_lo) - lo) / dx), i1 = (int)((log(a_hi > 1.0 ? a_hi : 1.0) - lo) / dx);
        double a[64], Hm[64], e = 0;
        for (int i = 0; i < 64; i++) {
            a[i] = exp(lo + (i0 + i * (i1 - i0 - 1) / 63 + 0.5) * dx);
            Hm[i] = hubble_function(a[i]);
        }
        kspace_gpu_check_hubble(ctx, a, Hm, 64, 1e-10, &e);
        if (e < best_err)
            best_err = e;
        if (e < 1e-10) {
            if (err)
                *err = e;
            return KSPACE_OK;
        }
    }
    if (err)
        *err = best_err;
    return KSPACE_ERR_HUBBLE;
}
#endif
