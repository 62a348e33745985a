/* Project-written stand-in for the part of GSL's error API that kspace-neutrinos
 * uses (delta_tot_table.c:70-73,101).  Test infrastructure: not shipped. */
#ifndef KSP_SHIM_GSL_ERRNO_H
#define KSP_SHIM_GSL_ERRNO_H
#ifdef __cplusplus
extern "C" {
#endif
enum { GSL_SUCCESS = 0, GSL_EDOM = 1, GSL_EINVAL = 4, GSL_ENOMEM = 8, GSL_EMAXITER = 11,
       GSL_EBADTOL = 13, GSL_EROUND = 18, GSL_ESING = 21 };
typedef void gsl_error_handler_t(const char *reason, const char *file, int line, int gsl_errno);
gsl_error_handler_t *gsl_set_error_handler(gsl_error_handler_t *new_handler);
/* Invoke the installed handler (or the shim's default one). */
void gslsub_error(const char *reason, const char *file, int line, int gsl_errno);
#ifdef __cplusplus
}
#endif
#endif
