/* Project-written stand-in for the GSL integration API used by kspace-neutrinos
 * (delta_tot_table.c:397-406,588-605; omega_nu_single.c:140-150,217-227):
 * QAG with the 61-point Gauss-Kronrod rule only.  Test infrastructure: not shipped. */
#ifndef KSP_SHIM_GSL_INTEGRATION_H
#define KSP_SHIM_GSL_INTEGRATION_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { double (*function)(double x, void *params); void *params; } gsl_function;
#define GSL_FN_EVAL(F, x) (*((F)->function))(x, (F)->params)
enum { GSL_INTEG_GAUSS15 = 1, GSL_INTEG_GAUSS21 = 2, GSL_INTEG_GAUSS31 = 3,
       GSL_INTEG_GAUSS41 = 4, GSL_INTEG_GAUSS51 = 5, GSL_INTEG_GAUSS61 = 6 };
typedef struct {
    size_t limit, size;
    double *alist, *blist, *rlist, *elist;
} gsl_integration_workspace;
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace *w);
int gsl_integration_qag(const gsl_function *f, double a, double b, double epsabs, double epsrel,
                        size_t limit, int key, gsl_integration_workspace *workspace,
                        double *result, double *abserr);
#ifdef __cplusplus
}
#endif
#endif
