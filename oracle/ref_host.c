/* oracle/ref_host.c -- host services the reference C expects from its N-body host
 * (gadget_defines.h:11,24-32), written for the oracle harness.  TEST INFRASTRUCTURE
 * ONLY: linked into oracle/_ref together with the unmodified reference sources.
 *
 *  - hubble_function(a): the flat LCDM + neutrino + photon form of the reference's own
 *    test suite (delta_tot_table_test.c:25-45), optionally with curvature as in the
 *    Gadget-2 hook (gadget-2/0003-...patch:38-52);
 *  - terminate(): instead of exiting, unwinds with longjmp to the guard set by the
 *    ref_* entry points below and returns the reference's error code;
 *  - message()/mymalloc/myfree: printing switchable, malloc-backed.
 */
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include "gadget_defines.h"
#include "omega_nu_single.h"

int ThisTask = 0;
static const _omega_nu *h_omnu = NULL;
static double h_Omega_nonu, h_OmegaLambda, h_OmegaK, h_Hubble;
static int h_radiation = 1;
static int g_verbose = 0;
static jmp_buf *g_guard = NULL;
static int g_term_code = 0;
static char g_term_msg[512];

void ref_set_verbose(int v) { g_verbose = v; }
int ref_last_terminate_code(void) { return g_term_code; }
const char *ref_last_terminate_message(void) { return g_term_msg; }

/* delta_tot_table_test.c:25-31 */
void ref_init_hubble(const _omega_nu *omnu, double Omega0, double OmegaLambda, double UnitTime_in_s,
                     int radiation)
{
    h_omnu = omnu;
    h_Omega_nonu = Omega0 - get_omega_nu(omnu, 1);
    h_OmegaLambda = OmegaLambda;
    h_OmegaK = 1.0 - Omega0 - OmegaLambda;
    h_Hubble = HUBBLE * UnitTime_in_s;
    h_radiation = radiation;
}

/* delta_tot_table_test.c:33-45 (test form); curvature term as gadget-2/0003 patch:38. */
int ref_hubble_uses_global(void);
double ref_hubble_global(double a);
double hubble_function(double a)
{
    if (ref_hubble_uses_global())
        return ref_hubble_global(a);
    if (!h_omnu) {
        fprintf(stderr, "ref_host: hubble_function called before ref_init_hubble\n");
        abort();
    }
    double omega_tot = h_Omega_nonu / pow(a, 3) + h_OmegaLambda;
    if (h_OmegaK != 0.0)
        omega_tot += h_OmegaK / (a * a);
    omega_tot += get_omega_nu(h_omnu, a);
    if (h_radiation)
        omega_tot += get_omegag(h_omnu, a);
    return h_Hubble * sqrt(omega_tot);
}

void terminate(int ierr, const char *fmt, ...)
{
    va_list va;
    va_start(va, fmt);
    vsnprintf(g_term_msg, sizeof(g_term_msg), fmt, va);
    va_end(va);
    g_term_code = ierr ? ierr : -1;
    if (g_verbose)
        fprintf(stderr, "reference terminate(%d): %s", ierr, g_term_msg);
    if (g_guard)
        longjmp(*g_guard, 1);
    fprintf(stderr, "reference terminate(%d) outside a guard: %s", ierr, g_term_msg);
    exit(ierr);
}

void message(int ierr, const char *fmt, ...)
{
    (void)ierr;
    if (!g_verbose)
        return;
    va_list va;
    va_start(va, fmt);
    vfprintf(stdout, fmt, va);
    va_end(va);
}

void *mymalloc_fullinfo(const char *string, size_t size, const char *func, const char *file, int line)
{
    (void)string; (void)func; (void)file; (void)line;
    return malloc(size);
}

void myfree_fullinfo(void *ptr, const char *func, const char *file, int line)
{
    (void)func; (void)file; (void)line;
    free(ptr);
}

/* GSL default error handler of the subset: route to terminate so it unwinds too. */
extern void (*gslsub_default_error_hook)(const char *reason, int gsl_errno);
static void ref_gsl_default(const char *reason, int gsl_errno)
{
    terminate(9000 + gsl_errno, "GSL error before a handler was installed: %s\n", reason);
}

/* Guard helpers used by ref_entry.c */
jmp_buf *ref_guard_push(jmp_buf *env)
{
    jmp_buf *old = g_guard;
    g_guard = env;
    g_term_code = 0;
    gslsub_default_error_hook = ref_gsl_default;
    return old;
}
void ref_guard_pop(jmp_buf *old) { g_guard = old; }

/* Allreduce hook of the single-rank mpi.h stand-in (NULL = one rank). */
#include "mpi.h"
int (*kspace_shim_allreduce_hook)(void *buf, int count, MPI_Datatype dt) = NULL;
