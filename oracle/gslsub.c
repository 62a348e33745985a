/* oracle/gslsub.c -- project-written restatement of the GSL subset that the
 * kspace-neutrinos hot path calls.  TEST INFRASTRUCTURE ONLY: it is linked into the
 * CPU oracle and into the reference C built here (oracle/_ref); the GPU product never
 * links it.
 *
 * GSL itself is not present in this environment and the reference pins no version
 * (Makefile:1 links -lgsl -lgslcblas).  What is restated here, from the published
 * mathematics:
 *   - natural cubic spline interpolation (second-derivative formulation, tridiagonal
 *     solve) and linear interpolation, with the usual "x_i <= x < x_{i+1}" segment
 *     choice (x == x_max uses the last segment);
 *   - QUADPACK's QAG adaptive integrator (Piessens, de Doncker-Kapenga, Ueberhuber &
 *     Kahaner 1983): 61-point Gauss-Kronrod rule on each interval, QUADPACK's error
 *     estimate err = resasc * min(1, (200 |K-G| / resasc)^1.5) floored at
 *     50 eps resabs, repeated bisection of the interval with the largest error
 *     estimate, and QUADPACK's round-off and interval-size checks;
 *   - the spherical Bessel function j0(x) = sin(x)/x (Taylor series near 0).
 * Interval selection picks the interval with the largest error estimate (lowest
 * index on ties).  QUADPACK's partially sorted error list only differs from that
 * once more than limit/2+2 intervals exist, which never happens on the workloads
 * this project checks (the interval count is exposed for that check).
 */
#include <math.h>
#include <float.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "gsl/gsl_errno.h"
#include "gsl/gsl_interp.h"
#include "gsl/gsl_integration.h"
#include "gsl/gsl_sf_bessel.h"
#include "kronrod61.h"

/* ------------------------------------------------------------------ errors */
static gsl_error_handler_t *g_handler = NULL;
/* Called when no handler is installed; the reference-side test harness replaces it
 * so that an error unwinds to the caller instead of aborting the process. */
void (*gslsub_default_error_hook)(const char *reason, int gsl_errno) = NULL;

gsl_error_handler_t *gsl_set_error_handler(gsl_error_handler_t *new_handler)
{
    gsl_error_handler_t *old = g_handler;
    g_handler = new_handler;
    return old;
}

void gslsub_error(const char *reason, const char *file, int line, int gsl_errno)
{
    if (g_handler) {
        g_handler(reason, file, line, gsl_errno);
        return;
    }
    if (gslsub_default_error_hook) {
        gslsub_default_error_hook(reason, gsl_errno);
        return;
    }
    fprintf(stderr, "gsl subset: %s:%d: ERROR: %s\n", file, line, reason);
    abort();
}

/* ------------------------------------------------------------------ interpolation */
static const gsl_interp_type linear_type = {"linear", 2, 0};
static const gsl_interp_type cspline_type = {"cspline", 3, 1};
const gsl_interp_type *gsl_interp_linear = &linear_type;
const gsl_interp_type *gsl_interp_cspline = &cspline_type;

gsl_interp_accel *gsl_interp_accel_alloc(void)
{
    return (gsl_interp_accel *)calloc(1, sizeof(gsl_interp_accel));
}

void gsl_interp_accel_free(gsl_interp_accel *a) { free(a); }

gsl_interp *gsl_interp_alloc(const gsl_interp_type *T, size_t n)
{
    if (n < T->min_size) {
        gslsub_error("too few knots for this interpolant", __FILE__, __LINE__, GSL_EINVAL);
        return NULL;
    }
    gsl_interp *p = (gsl_interp *)calloc(1, sizeof(gsl_interp));
    p->type = T;
    p->size = n;
    if (T->kind == 1)
        p->c = (double *)calloc(n, sizeof(double));
    return p;
}

void gsl_interp_free(gsl_interp *interp)
{
    if (!interp)
        return;
    free(interp->c);
    free(interp);
}

/* Natural cubic spline: with c_i = S''(x_i)/2, c_0 = c_{n-1} = 0 and for i=1..n-2
 *   h_{i-1} c_{i-1} + 2 (h_{i-1}+h_i) c_i + h_i c_{i+1} = 3 (s_i - s_{i-1}),
 * s_i = (y_{i+1}-y_i)/h_i.  Solved by Gaussian elimination without pivoting
 * (the system is symmetric, strictly diagonally dominant). */
static void natural_spline_coeffs(const double *x, const double *y, size_t n, double *c)
{
    size_t m = n - 2, i;
    c[0] = 0.0;
    c[n - 1] = 0.0;
    if (m == 0)
        return;
    double *diag = (double *)malloc(m * sizeof(double));
    double *rhs = (double *)malloc(m * sizeof(double));
    for (i = 0; i < m; i++) {
        const double h0 = x[i + 1] - x[i], h1 = x[i + 2] - x[i + 1];
        diag[i] = 2.0 * (h0 + h1);
        rhs[i] = 3.0 * ((y[i + 2] - y[i + 1]) / h1 - (y[i + 1] - y[i]) / h0);
    }
    /* forward elimination; off-diagonal between unknowns i and i+1 is h_{i+1} */
    for (i = 1; i < m; i++) {
        const double off = x[i + 1] - x[i];
        const double f = off / diag[i - 1];
        diag[i] -= f * off;
        rhs[i] -= f * rhs[i - 1];
    }
    c[m] = rhs[m - 1] / diag[m - 1];
    for (i = m - 1; i-- > 0;) {
        const double off = x[i + 2] - x[i + 1];
        c[i + 1] = (rhs[i] - off * c[i + 2]) / diag[i];
    }
    free(diag);
    free(rhs);
}

int gsl_interp_init(gsl_interp *interp, const double xa[], const double ya[], size_t size)
{
    size_t i;
    if (size != interp->size) {
        gslsub_error("knot count differs from the allocated interpolant", __FILE__, __LINE__, GSL_EINVAL);
        return GSL_EINVAL;
    }
    for (i = 1; i < size; i++) {
        if (!(xa[i - 1] < xa[i])) {
            gslsub_error("knots are not in strictly ascending order", __FILE__, __LINE__, GSL_EINVAL);
            return GSL_EINVAL;
        }
    }
    interp->xmin = xa[0];
    interp->xmax = xa[size - 1];
    if (interp->type->kind == 1)
        natural_spline_coeffs(xa, ya, size, interp->c);
    return GSL_SUCCESS;
}

/* Segment index i with xa[i] <= x < xa[i+1]; x == xa[n-1] gives n-2. */
static size_t find_segment(const double *xa, size_t n, double x)
{
    size_t lo = 0, hi = n - 1;
    while (hi > lo + 1) {
        const size_t mid = (lo + hi) / 2;
        if (xa[mid] > x)
            hi = mid;
        else
            lo = mid;
    }
    return lo;
}

double gsl_interp_eval(const gsl_interp *interp, const double xa[], const double ya[], double x,
                       gsl_interp_accel *a)
{
    if (x < interp->xmin || x > interp->xmax) {
        gslsub_error("query outside the knot range", __FILE__, __LINE__, GSL_EDOM);
        return NAN;
    }
    const size_t i = find_segment(xa, interp->size, x);
    if (a)
        a->cache = i;
    const double h = xa[i + 1] - xa[i];
    const double dx = x - xa[i];
    if (interp->type->kind == 0)
        return ya[i] + dx * ((ya[i + 1] - ya[i]) / h);
    const double *c = interp->c;
    const double b = (ya[i + 1] - ya[i]) / h - h * (c[i + 1] + 2.0 * c[i]) / 3.0;
    const double d = (c[i + 1] - c[i]) / (3.0 * h);
    return ya[i] + dx * (b + dx * (c[i] + dx * d));
}

/* ------------------------------------------------------------------ QAG / GK61 */
static const double XK[31] = KSP_GK61_XK_INIT;
static const double WK[31] = KSP_GK61_WK_INIT;
static const double WG[31] = KSP_GK61_WG_INIT;

static double rescale_error(double err, double resabs, double resasc)
{
    err = fabs(err);
    if (resasc != 0.0 && err != 0.0) {
        const double s = pow(200.0 * err / resasc, 1.5);
        err = s < 1.0 ? resasc * s : resasc;
    }
    if (resabs > DBL_MIN / (50.0 * DBL_EPSILON)) {
        const double floor_err = 50.0 * DBL_EPSILON * resabs;
        if (floor_err > err)
            err = floor_err;
    }
    return err;
}

/* One 61-point Gauss-Kronrod application on [a,b]. */
static void gk61(const gsl_function *f, double a, double b, double *result, double *abserr,
                 double *resabs, double *resasc)
{
    const double center = 0.5 * (a + b);
    const double half = 0.5 * (b - a);
    const double fc = GSL_FN_EVAL(f, center);
    double f1[30], f2[30];
    double resk = WK[30] * fc, resg = 0.0, rabs = fabs(resk);
    int j;
    for (j = 0; j < 30; j++) {
        const double dx = half * XK[j];
        f1[j] = GSL_FN_EVAL(f, center - dx);
        f2[j] = GSL_FN_EVAL(f, center + dx);
        const double s = f1[j] + f2[j];
        resk += WK[j] * s;
        resg += WG[j] * s;
        rabs += WK[j] * (fabs(f1[j]) + fabs(f2[j]));
    }
    const double mean = 0.5 * resk;
    double rasc = WK[30] * fabs(fc - mean);
    for (j = 0; j < 30; j++)
        rasc += WK[j] * (fabs(f1[j] - mean) + fabs(f2[j] - mean));
    const double err = (resk - resg) * half;
    *result = resk * half;
    *resabs = rabs * fabs(half);
    *resasc = rasc * fabs(half);
    *abserr = rescale_error(err, *resabs, *resasc);
}

gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n)
{
    if (n == 0) {
        gslsub_error("integration workspace needs at least one interval", __FILE__, __LINE__, GSL_EDOM);
        return NULL;
    }
    gsl_integration_workspace *w = (gsl_integration_workspace *)calloc(1, sizeof(*w));
    w->limit = n;
    w->alist = (double *)calloc(4 * n, sizeof(double));
    w->blist = w->alist + n;
    w->rlist = w->blist + n;
    w->elist = w->rlist + n;
    return w;
}

void gsl_integration_workspace_free(gsl_integration_workspace *w)
{
    if (!w)
        return;
    free(w->alist);
    free(w);
}

/* Diagnostics for the checker: interval count and status of the most recent QAG. */
static int g_last_intervals = 0;
int gslsub_last_qag_intervals(void) { return g_last_intervals; }
static long long g_total_qag_calls = 0, g_total_qag_intervals = 0;
void gslsub_qag_counters(long long *calls, long long *intervals)
{
    *calls = g_total_qag_calls;
    *intervals = g_total_qag_intervals;
}
/* rule applications by depth in the bisection tree of [a, b] (diagnostics) */
static long long g_depth_rules[32];
static double g_depth_a, g_depth_w;
static long long g_slot_rules[255];
static void count_rule(double lo, double hi)
{
    const double r = g_depth_w / (hi - lo);
    int d = 0;
    while (d < 31 && r > 1.5 * (double)(1LL << d)) d++;
    g_depth_rules[d]++;
    if (d < 8) {
        const int p = (int)floor((lo - g_depth_a) / (hi - lo) + 0.5);
        const int s = (1 << d) - 1 + p;
        if (s >= 0 && s < 255) g_slot_rules[s]++;
    }
}
void gslsub_depth_rules(long long *out32, int reset)
{
    for (int i = 0; i < 32; i++) {
        out32[i] = g_depth_rules[i];
        if (reset) g_depth_rules[i] = 0;
    }
}
void gslsub_slot_rules(long long *out255, int reset)
{
    for (int i = 0; i < 255; i++) {
        out255[i] = g_slot_rules[i];
        if (reset) g_slot_rules[i] = 0;
    }
}
void gslsub_reset_counters(void) { g_total_qag_calls = 0; g_total_qag_intervals = 0; }

int gsl_integration_qag(const gsl_function *f, double a, double b, double epsabs, double epsrel,
                        size_t limit, int key, gsl_integration_workspace *w, double *result,
                        double *abserr)
{
    double area, errsum, res0, err0, rabs0, rasc0, tol;
    size_t n, i;
    int roundoff1 = 0, roundoff2 = 0, error_type = 0;
    *result = 0;
    *abserr = 0;
    if (key != GSL_INTEG_GAUSS61) {
        gslsub_error("this subset has the 61-point rule only", __FILE__, __LINE__, GSL_EINVAL);
        return GSL_EINVAL;
    }
    if (limit > w->limit) {
        gslsub_error("subdivision limit larger than the workspace", __FILE__, __LINE__, GSL_EINVAL);
        return GSL_EINVAL;
    }
    if (epsabs <= 0 && (epsrel < 50 * DBL_EPSILON || epsrel < 0.5e-28)) {
        gslsub_error("requested tolerances are unreachable (epsabs <= 0 and epsrel too small)", __FILE__, __LINE__, GSL_EBADTOL);
        return GSL_EBADTOL;
    }
    g_total_qag_calls++;
    g_depth_a = a;
    g_depth_w = b - a;
    count_rule(a, b);
    gk61(f, a, b, &res0, &err0, &rabs0, &rasc0);
    w->size = 1;
    w->alist[0] = a;
    w->blist[0] = b;
    w->rlist[0] = res0;
    w->elist[0] = err0;
    tol = fmax(epsabs, epsrel * fabs(res0));
    const double round_off = 50 * DBL_EPSILON * rabs0;
    g_last_intervals = 1;
    g_total_qag_intervals += 1;
    if (err0 <= round_off && err0 > tol) {
        *result = res0;
        *abserr = err0;
        gslsub_error("first rule evaluation already dominated by rounding: tolerance unreachable", __FILE__, __LINE__, GSL_EROUND);
        return GSL_EROUND;
    } else if ((err0 <= tol && err0 != rasc0) || err0 == 0.0) {
        *result = res0;
        *abserr = err0;
        return GSL_SUCCESS;
    } else if (limit == 1) {
        *result = res0;
        *abserr = err0;
        gslsub_error("tolerance not met and the subdivision limit is one", __FILE__, __LINE__, GSL_EMAXITER);
        return GSL_EMAXITER;
    }
    area = res0;
    errsum = err0;
    n = 1;
    do {
        /* interval with the largest error estimate (lowest index on ties) */
        size_t k = 0;
        for (i = 1; i < n; i++)
            if (w->elist[i] > w->elist[k])
                k = i;
        const double a_i = w->alist[k], b_i = w->blist[k], r_i = w->rlist[k], e_i = w->elist[k];
        const double a1 = a_i, b1 = 0.5 * (a_i + b_i), a2 = b1, b2 = b_i;
        double area1, error1, rabs1, rasc1, area2, error2, rabs2, rasc2;
        count_rule(a1, b1);
        count_rule(a2, b2);
        gk61(f, a1, b1, &area1, &error1, &rabs1, &rasc1);
        gk61(f, a2, b2, &area2, &error2, &rabs2, &rasc2);
        const double area12 = area1 + area2, error12 = error1 + error2;
        errsum += error12 - e_i;
        area += area12 - r_i;
        if (rasc1 != error1 && rasc2 != error2) {
            if (fabs(r_i - area12) <= 1.0e-5 * fabs(area12) && error12 >= 0.99 * e_i)
                roundoff1++;
            if (n >= 10 && error12 > e_i)
                roundoff2++;
        }
        tol = fmax(epsabs, epsrel * fabs(area));
        if (errsum > tol) {
            if (roundoff1 >= 6 || roundoff2 >= 20)
                error_type = 2;
            const double tiny = (1 + 100 * DBL_EPSILON) * (fabs(a2) + 1000 * DBL_MIN);
            if (fabs(a1) <= tiny && fabs(b2) <= tiny)
                error_type = 3;
        }
        /* left half replaces the bisected interval, right half is appended */
        w->blist[k] = b1;
        w->rlist[k] = area1;
        w->elist[k] = error1;
        w->alist[n] = a2;
        w->blist[n] = b2;
        w->rlist[n] = area2;
        w->elist[n] = error2;
        n++;
    } while (n < limit && !error_type && errsum > tol);
    w->size = n;
    double sum = 0;
    for (i = 0; i < n; i++)
        sum += w->rlist[i];
    *result = sum;
    *abserr = errsum;
    g_last_intervals = (int)n;
    g_total_qag_intervals += (long long)n - 1;
    if (errsum <= tol)
        return GSL_SUCCESS;
    if (error_type == 2) {
        gslsub_error("rounding errors grew too large to meet the tolerance", __FILE__, __LINE__, GSL_EROUND);
        return GSL_EROUND;
    }
    if (error_type == 3) {
        gslsub_error("integrand too irregular: an interval became too narrow to split", __FILE__, __LINE__, GSL_ESING);
        return GSL_ESING;
    }
    gslsub_error("subdivision limit reached before the tolerance was met", __FILE__, __LINE__, GSL_EMAXITER);
    return GSL_EMAXITER;
}

/* ------------------------------------------------------------------ j0 */
double gsl_sf_bessel_j0(double x)
{
    const double ax = fabs(x);
    if (ax < 0.05) {
        /* sin(x)/x = 1 - y/6 + y^2/120 - y^3/5040 + y^4/362880, y = x^2 */
        const double y = x * x;
        return 1.0 - y / 6.0 * (1.0 - y / 20.0 * (1.0 - y / 42.0 * (1.0 - y / 72.0)));
    }
    return sin(x) / x;
}
