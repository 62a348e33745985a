/* Project-written stand-in for the GSL 1-D interpolation API used by kspace-neutrinos
 * (delta_tot_table.c:104-116,553-602; delta_pow.c:14-16,35,41-42;
 * omega_nu_single.c:135-136,151,199).  Linear and natural cubic spline only.
 * Test infrastructure: not shipped. */
#ifndef KSP_SHIM_GSL_INTERP_H
#define KSP_SHIM_GSL_INTERP_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { const char *name; unsigned int min_size; int kind; } gsl_interp_type;
extern const gsl_interp_type *gsl_interp_linear;
extern const gsl_interp_type *gsl_interp_cspline;
typedef struct {
    const gsl_interp_type *type;
    double xmin, xmax;
    size_t size;
    double *c;      /* natural spline: half the second derivative at each knot */
} gsl_interp;
typedef struct { size_t cache, miss_count, hit_count; } gsl_interp_accel;
gsl_interp_accel *gsl_interp_accel_alloc(void);
void gsl_interp_accel_free(gsl_interp_accel *a);
gsl_interp *gsl_interp_alloc(const gsl_interp_type *T, size_t n);
int gsl_interp_init(gsl_interp *interp, const double xa[], const double ya[], size_t size);
double gsl_interp_eval(const gsl_interp *interp, const double xa[], const double ya[], double x,
                       gsl_interp_accel *a);
void gsl_interp_free(gsl_interp *interp);
#ifdef __cplusplus
}
#endif
#endif
