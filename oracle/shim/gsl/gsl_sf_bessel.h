/* Project-written stand-in: spherical Bessel j0(x) = sin(x)/x (delta_tot_table.c:433). */
#ifndef KSP_SHIM_GSL_SF_BESSEL_H
#define KSP_SHIM_GSL_SF_BESSEL_H
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_bessel_j0(double x);
#ifdef __cplusplus
}
#endif
#endif
