/* oracle/kspace_oracle.c -- CPU restatement of the kspace-neutrinos hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the CPU "port" baseline).  The GPU product
 * never links this file.  The arithmetic follows the reference step by step; each
 * function cites the reference file:line it restates.  Error returns use the
 * reference's terminate() codes.  Parity: pinned against the reference C compiled
 * here (oracle/_ref) and the reference test suite's known answers.
 */
#include <math.h>
#include <float.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "gsl/gsl_errno.h"
#include "gsl/gsl_interp.h"
#include "gsl/gsl_integration.h"
#include "gsl/gsl_sf_bessel.h"
#include "kspace_oracle.h"
#include "kronrod61.h"

/* kspace_neutrino_const.h:9-19, gadget_defines.h:8, omega_nu_single.c:10-14 */
#define NUSPECIES 3
#define LIGHTCGS 2.99792458e10
#define BOLEVK 8.61734e-5
#define FLOAT_ACC 1e-6
#define GSL_VAL 200
#define HUBBLE 3.24077929e-18
#define HBAR 6.582119e-16
#define STEFAN_BOLTZMANN 5.670373e-5
#define GRAVITY 6.67408e-8
#define NRHOTAB 200
#define NU_SW 100
#define TNUCMB (pow(4 / 11., 1 / 3.) * 1.00328) /* omega_nu_single.h:17 */

int gslsub_last_qag_intervals(void);

/* The GSL subset reports errors through a handler; the oracle records the first one
 * so the calling function can return code 2001 as the reference's handler would
 * (delta_tot_table.c:70-73). */
static __thread int g_gsl_err = 0;
static void oracle_gsl_handler(const char *reason, const char *file, int line, int err)
{
    (void)reason; (void)file; (void)line;
    if (!g_gsl_err)
        g_gsl_err = err ? err : -1;
}
static void ensure_handler(void) { gsl_set_error_handler(oracle_gsl_handler); }

/* ================================================================== background */
typedef struct {
    int has_table;
    double mnu;
    double loga[NRHOTAB], rhonu[NRHOTAB];
    gsl_interp *interp;
} rho_tab;

struct ko_bg {
    rho_tab tab[NUSPECIES];
    int deg[NUSPECIES];
    double rhocrit, kBtnu, tcmb0;
    int hyb_enabled;
    double nufrac_low[NUSPECIES], nu_crit_time, vcrit;
    double Omega0, OmegaLambda, OmegaK, hubble, Omega_nonu_H;
    int radiation;
};

/* omega_nu_single.c:89-96 */
static double rho_nu_int(double q, void *params)
{
    const double amnu = ((double *)params)[0];
    const double kT = ((double *)params)[1];
    const double epsilon = sqrt(q * q + amnu * amnu);
    const double f0 = 1. / (exp(q / kT) + 1);
    return q * q * epsilon * f0;
}

/* omega_nu_single.c:100-114 */
static double rho_nu_conversion(void)
{
    double convert = 4 * M_PI * 2;
    const double chbar = 1. / (2 * M_PI * LIGHTCGS * HBAR);
    convert *= (chbar * chbar * chbar);
    convert *= (1.60217646e-12 / LIGHTCGS / LIGHTCGS);
    return convert;
}

/* omega_nu_single.c:117-153 */
static void rho_nu_init(rho_tab *t, double a0, double mnu, double kBtnu)
{
    const double logA0 = log(a0) - log(1.2);
    const double logaf = log(NU_SW * kBtnu / mnu) + log(1.2);
    t->mnu = mnu;
    t->has_table = 0;
    if (mnu < 1e-6 * kBtnu || logaf < logA0)
        return;
    gsl_integration_workspace *w = gsl_integration_workspace_alloc(GSL_VAL);
    gsl_function F;
    F.function = &rho_nu_int;
    for (int i = 0; i < NRHOTAB; i++) {
        double param[2], abserr;
        t->loga[i] = logA0 + i * (logaf - logA0) / (NRHOTAB - 1);
        param[0] = mnu * exp(t->loga[i]);
        param[1] = kBtnu;
        F.params = param;
        gsl_integration_qag(&F, 0, 500 * kBtnu, 0, 1e-9, GSL_VAL, 6, w, &t->rhonu[i], &abserr);
        t->rhonu[i] = t->rhonu[i] / pow(exp(t->loga[i]), 4) * rho_nu_conversion();
    }
    gsl_integration_workspace_free(w);
    t->interp = gsl_interp_alloc(gsl_interp_cspline, NRHOTAB);
    gsl_interp_init(t->interp, t->loga, t->rhonu, NRHOTAB);
    t->has_table = 1;
}

/* omega_nu_single.c:156-160 */
static double non_rel_rho_nu(double a, double kT, double amnu, double kTamnu2)
{
    return amnu * (kT * kT * kT) / (a * a * a * a) *
           (1.5 * 1.202056903159594 + kTamnu2 * 45. / 4. * 1.0369277551433704 +
            2835. / 32. * kTamnu2 * kTamnu2 * 1.0083492773819229 +
            80325 / 32. * kTamnu2 * kTamnu2 * kTamnu2 * 1.0020083928260826) *
           rho_nu_conversion();
}

/* omega_nu_single.c:164-167 */
static double rel_rho_nu(double a, double kT) { return 7 * pow(M_PI * kT / a, 4) / 120. * rho_nu_conversion(); }

/* omega_nu_single.c:171-202 */
static double rho_nu(const rho_tab *t, double a, double kT)
{
    const double amnu = a * t->mnu;
    const double kTamnu2 = (kT * kT / amnu / amnu);
    if (NU_SW * NU_SW * kTamnu2 < 1)
        return non_rel_rho_nu(a, kT, amnu, kTamnu2);
    if (amnu < 1e-6 * kT)
        return rel_rho_nu(a, kT);
    const double loga = log(a);
    if (!t->has_table || loga < t->loga[0]) {
        if (amnu < 1e-4 * kT)
            return rel_rho_nu(a, kT);
        return non_rel_rho_nu(a, kT, amnu, kTamnu2);
    }
    return gsl_interp_eval(t->interp, t->loga, t->rhonu, loga, NULL);
}

/* omega_nu_single.c:246-257 */
double ko_particle_nu_fraction(const ko_bg *bg, double a, int i)
{
    if (!bg->hyb_enabled)
        return 0;
    if (a > bg->nu_crit_time)
        return bg->nufrac_low[i];
    return 0;
}

/* omega_nu_single.c:55-65 */
double ko_omega_nu(const ko_bg *bg, double a)
{
    double rhonu = 0;
    for (int mi = 0; mi < NUSPECIES; mi++)
        if (bg->deg[mi] > 0)
            rhonu += bg->deg[mi] * rho_nu(&bg->tab[mi], a, bg->kBtnu);
    return rhonu / bg->rhocrit;
}

/* omega_nu_single.c:69-74 */
double ko_omega_nu_nopart(const ko_bg *bg, double a)
{
    const double omega_nu = ko_omega_nu(bg, a);
    const double part_nu = ko_omega_nu(bg, 1) * ko_particle_nu_fraction(bg, a, 0) / (a * a * a);
    return omega_nu - part_nu;
}

/* omega_nu_single.c:77-81 */
double ko_omegag(const ko_bg *bg, double a)
{
    const double omegag = 4 * STEFAN_BOLTZMANN / (LIGHTCGS * LIGHTCGS * LIGHTCGS) * pow(bg->tcmb0, 4) / bg->rhocrit;
    return omegag / pow(a, 4);
}

/* omega_nu_single.c:262-279 */
double ko_omega_nu_single(const ko_bg *bg, double a, int i)
{
    if (bg->deg[i] == 0) {
        for (int j = i; j >= 0; j--)
            if (bg->deg[j]) {
                i = j;
                break;
            }
    }
    double omega_nu = rho_nu(&bg->tab[i], a, bg->kBtnu) / bg->rhocrit;
    double omega_part = rho_nu(&bg->tab[i], 1, bg->kBtnu) / bg->rhocrit;
    omega_part *= ko_particle_nu_fraction(bg, a, i) / (a * a * a);
    return omega_nu - omega_part;
}

/* omega_nu_single.c:207-228 */
static double fermi_dirac_kernel(double x, void *params)
{
    (void)params;
    return x * x / (exp(x) + 1);
}
double ko_nufrac_low(double qc)
{
    ensure_handler();
    gsl_integration_workspace *w = gsl_integration_workspace_alloc(100);
    double abserr, total_fd;
    gsl_function F;
    F.function = &fermi_dirac_kernel;
    F.params = NULL;
    gsl_integration_qag(&F, 0, qc, 0, 1e-6, 100, 6, w, &total_fd, &abserr);
    total_fd /= 1.5 * 1.202056903159594;
    gsl_integration_workspace_free(w);
    return total_fd;
}

/* omega_nu_single.c:16-51 plus the test hubble function state
 * (delta_tot_table_test.c:25-31). */
ko_bg *ko_bg_new(const double MNu[3], double a0, double HubbleParam, double tcmb0, double Omega0,
                 double OmegaLambda, double UnitTime_in_s, int radiation)
{
    ensure_handler();
    ko_bg *bg = (ko_bg *)calloc(1, sizeof(ko_bg));
    bg->tcmb0 = tcmb0;
    bg->kBtnu = BOLEVK * TNUCMB * tcmb0;
    bg->rhocrit = (3 * HUBBLE * HubbleParam * HUBBLE * HubbleParam) / (8 * M_PI * GRAVITY);
    for (int mi = 0; mi < NUSPECIES; mi++) {
        int mmi;
        bg->deg[mi] = 0;
        for (mmi = 0; mmi < mi; mmi++) {
            if (fabs(MNu[mi] - MNu[mmi]) < FLOAT_ACC) {
                bg->deg[mmi] += 1;
                break;
            }
        }
        if (mmi == mi)
            bg->deg[mi] = 1;
    }
    for (int mi = 0; mi < NUSPECIES; mi++) {
        if (bg->deg[mi])
            rho_nu_init(&bg->tab[mi], a0, MNu[mi], bg->kBtnu);
        else
            bg->tab[mi].mnu = MNu[mi];
    }
    bg->Omega0 = Omega0;
    bg->OmegaLambda = OmegaLambda;
    bg->OmegaK = 1.0 - Omega0 - OmegaLambda;
    bg->hubble = HUBBLE * UnitTime_in_s;
    bg->radiation = radiation;
    bg->Omega_nonu_H = Omega0 - ko_omega_nu(bg, 1);
    return bg;
}

void ko_bg_free(ko_bg *bg)
{
    if (!bg)
        return;
    for (int i = 0; i < NUSPECIES; i++)
        gsl_interp_free(bg->tab[i].interp);
    free(bg);
}

/* omega_nu_single.c:230-240 */
int ko_bg_hybrid(ko_bg *bg, double vcrit, double light, double nu_crit_time)
{
    bg->hyb_enabled = 1;
    bg->nu_crit_time = nu_crit_time;
    bg->vcrit = vcrit / light;
    for (int i = 0; i < NUSPECIES; i++) {
        const double qc = bg->tab[i].mnu * vcrit / light / bg->kBtnu;
        bg->nufrac_low[i] = ko_nufrac_low(qc);
    }
    return 0;
}

void ko_bg_info(const ko_bg *bg, double *rhocrit, double *kBtnu, int *deg, double *mnu)
{
    *rhocrit = bg->rhocrit;
    *kBtnu = bg->kBtnu;
    for (int i = 0; i < NUSPECIES; i++) {
        deg[i] = bg->deg[i];
        mnu[i] = bg->tab[i].mnu;
    }
}

int ko_bg_table(const ko_bg *bg, int i, double *loga, double *rhonu)
{
    if (!bg->tab[i].has_table)
        return 0;
    memcpy(loga, bg->tab[i].loga, sizeof(bg->tab[i].loga));
    memcpy(rhonu, bg->tab[i].rhonu, sizeof(bg->tab[i].rhonu));
    return NRHOTAB;
}

/* delta_tot_table_test.c:33-45 (curvature term: gadget-2/0003 patch:38) */
double ko_hubble(const ko_bg *bg, double a)
{
    double omega_tot = bg->Omega_nonu_H / pow(a, 3) + bg->OmegaLambda;
    if (bg->OmegaK != 0.0)
        omega_tot += bg->OmegaK / (a * a);
    omega_tot += ko_omega_nu(bg, a);
    if (bg->radiation)
        omega_tot += ko_omegag(bg, a);
    return bg->hubble * sqrt(omega_tot);
}

/* ================================================================== J, fslength */
/* delta_tot_table.c:417-428 */
static double specialJ_fit(double x)
{
    if (x <= 0.)
        return 1.;
    const double x2 = x * x, x4 = x2 * x2, x8 = x4 * x4;
    return (1. + 0.0168 * x2 + 0.0407 * x4) / (1. + 2.1734 * x2 + 1.6787 * exp(4.1811 * log(x)) + 0.1467 * x8);
}
/* delta_tot_table.c:431-434 */
static double II(double x, double qc, int n)
{
    return (n * n + n * n * n * qc + n * qc * x * x - x * x) * qc * gsl_sf_bessel_j0(qc * x) +
           (2 * n + n * n * qc + qc * x * x) * cos(qc * x);
}
/* delta_tot_table.c:442-454 */
static double Jfrac_high(double x, double qc, double nufrac_low)
{
    double integ = 0;
    for (int n = 1; n < 20; n++)
        integ += -1 * pow((-1), n) * exp(-n * qc) / (n * n + x * x) / (n * n + x * x) * II(x, qc, n);
    integ /= 1.5 * 1.202056903159594 * (1 - nufrac_low);
    return integ;
}
/* delta_tot_table.c:457-463 */
double ko_specialJ(double x, double qc, double nufrac_low)
{
    if (qc > 0)
        return Jfrac_high(x, qc, nufrac_low);
    return specialJ_fit(x);
}

/* delta_tot_table.c:378-383 */
static double fslength_int(double loga, void *params)
{
    const ko_bg *bg = (const ko_bg *)params;
    const double a = exp(loga);
    return 1. / a / (a * ko_hubble(bg, a));
}

static double qag_run_keep(gsl_function *F, double a, double b, double epsrel, int *status,
                           gsl_integration_workspace **keep)
{
    gsl_integration_workspace *w = gsl_integration_workspace_alloc(GSL_VAL);
    double r = 0, e;
    g_gsl_err = 0;
    gsl_integration_qag(F, a, b, 0, epsrel, GSL_VAL, 6, w, &r, &e);
    if (g_gsl_err && status && !*status)
        *status = 2001;
    if (keep)
        *keep = w;
    else
        gsl_integration_workspace_free(w);
    return r;
}
static double qag_run(gsl_function *F, double a, double b, double epsrel, int *status)
{
    return qag_run_keep(F, a, b, epsrel, status, NULL);
}

/* delta_tot_table.c:394-407 */
double ko_fslength(const ko_bg *bg, double logai, double logaf, double light, int *status)
{
    ensure_handler();
    if (logai >= logaf)
        return 0;
    gsl_function F;
    F.function = &fslength_int;
    F.params = (void *)bg;
    return light * qag_run(&F, logai, logaf, 1e-6, status);
}

/* One non-adaptive 61-point Gauss-Kronrod application (the Kronrod sum only), used by
 * the all-FP64 oracle on short segments where the integrand is smooth. */
static double gk61_plain(gsl_function *F, double a, double b)
{
    static const double XK[31] = KSP_GK61_XK_INIT;
    static const double WK[31] = KSP_GK61_WK_INIT;
    const double c = 0.5 * (a + b), h = 0.5 * (b - a);
    double s = WK[30] * GSL_FN_EVAL(F, c);
    for (int j = 0; j < 30; j++)
        s += WK[j] * (GSL_FN_EVAL(F, c - h * XK[j]) + GSL_FN_EVAL(F, c + h * XK[j]));
    return s * h;
}

/* exact fslength for the FP64 oracle: GK61 on 64 equal pieces (integrand analytic
 * apart from the 200-knot Omega_nu spline; pieces are short) */
static double fslength_exact(const ko_bg *bg, double logai, double logaf, double light, int *status)
{
    (void)status;
    if (logai >= logaf)
        return 0;
    gsl_function F;
    F.function = &fslength_int;
    F.params = (void *)bg;
    double acc = 0;
    const int n = 64;
    for (int i = 0; i < n; i++)
        acc += gk61_plain(&F, logai + (logaf - logai) * i / n, logai + (logaf - logai) * (i + 1) / n);
    return light * acc;
}

/* ================================================================== state */
struct ko_state {
    ko_bg *bg;
    int nk, nk_alloc, namax, ia, init_done;
    double prefac, Omeganonu, light, TimeTransfer;
    double *scalefact, *delta_tot; /* delta_tot[ik*namax + ia] */
    double *nu_init, *nu_last, *wavenum;
    int ntrans;
    double *t_logk, *t_Tnu;
    int fs_mode, exact;
    int last_max_intervals;
    long long last_total_intervals;
    int last_nfs;
    double *last_fs_scales, *last_fs_lengths;
    /* differentiation support (test infrastructure): mass used inside J per species,
     * and the adjoint accumulators filled when adj_dnu_bar is set */
    int mJ_set;
    double mJ[NUSPECIES];
    const double *adj_dnu_bar;
    double *adj_Dbar;       /* [nk][Na] */
    double adj_mbar[NUSPECIES];
    double adj_weight;      /* omega_s / Omega_nu_tot of the species being integrated */
    int adj_species;
};

/* delta_tot_table.c:25-60 */
ko_state *ko_state_new(ko_bg *bg, int nk_in, double TimeTransfer, double TimeMax, double Omega0,
                       double UnitTime_in_s, double UnitLength_in_cm)
{
    ko_state *s = (ko_state *)calloc(1, sizeof(ko_state));
    s->bg = bg;
    s->nk_alloc = nk_in;
    s->nk = nk_in;
    s->TimeTransfer = TimeTransfer;
    s->namax = (int)ceil(100 * (TimeMax - TimeTransfer)) + 2;
    s->ia = 0;
    s->scalefact = (double *)calloc((size_t)s->namax * (nk_in + 1), sizeof(double));
    s->delta_tot = s->scalefact + s->namax;
    s->nu_init = (double *)calloc(3 * (size_t)nk_in, sizeof(double));
    s->nu_last = s->nu_init + nk_in;
    s->wavenum = s->nu_init + 2 * nk_in;
    s->light = LIGHTCGS * UnitTime_in_s / UnitLength_in_cm;
    s->prefac = 1.5 * Omega0 * HUBBLE * HUBBLE * pow(UnitTime_in_s, 2) / s->light;
    s->Omeganonu = Omega0 - ko_omega_nu(bg, 1);
    return s;
}

void ko_state_free(ko_state *s)
{
    if (!s)
        return;
    free(s->scalefact);
    free(s->nu_init);
    free(s->t_logk);
    free(s->last_fs_scales);
    free(s);
}

int ko_state_set_transfer(ko_state *s, const double *logk, const double *T_nu, int n)
{
    free(s->t_logk);
    s->t_logk = (double *)malloc(2 * (size_t)n * sizeof(double));
    s->t_Tnu = s->t_logk + n;
    memcpy(s->t_logk, logk, n * sizeof(double));
    memcpy(s->t_Tnu, T_nu, n * sizeof(double));
    s->ntrans = n;
    return 0;
}

/* interface_common.c:166-180 */
int ko_state_set_nu_state(ko_state *s, const double *scalefact, const double *delta_tot, int nk, int ia)
{
    if (ia > s->namax || nk > s->nk_alloc)
        return 2011;
    s->nk = nk;
    s->ia = ia;
    for (int i = 0; i < ia; i++)
        s->scalefact[i] = scalefact[i];
    for (int ik = 0; ik < nk; ik++)
        for (int i = 0; i < ia; i++)
            s->delta_tot[(size_t)ik * s->namax + i] = delta_tot[(size_t)ik * ia + i];
    return 0;
}

void ko_state_get(const ko_state *s, int *ints, double *scalefact, double *delta_tot, double *vec3)
{
    if (ints) {
        ints[0] = s->nk; ints[1] = s->nk_alloc; ints[2] = s->namax; ints[3] = s->ia; ints[4] = s->init_done;
    }
    if (scalefact)
        memcpy(scalefact, s->scalefact, s->namax * sizeof(double));
    if (delta_tot)
        memcpy(delta_tot, s->delta_tot, (size_t)s->namax * s->nk_alloc * sizeof(double));
    if (vec3)
        memcpy(vec3, s->nu_init, 3 * (size_t)s->nk_alloc * sizeof(double));
}

void ko_state_scalars(const ko_state *s, double *out)
{
    out[0] = s->prefac; out[1] = s->Omeganonu; out[2] = s->light; out[3] = s->TimeTransfer;
}

void ko_state_set_ia(ko_state *s, int ia) { s->ia = ia; }
void ko_state_options(ko_state *s, int fs_mode, int exact) { s->fs_mode = fs_mode; s->exact = exact; }

void ko_last_qag_stats(const ko_state *s, int *max_intervals, long long *total_intervals)
{
    *max_intervals = s->last_max_intervals;
    *total_intervals = s->last_total_intervals;
}

int ko_last_fs_table(const ko_state *s, double *scales, double *lengths)
{
    if (scales && s->last_fs_scales) {
        memcpy(scales, s->last_fs_scales, s->last_nfs * sizeof(double));
        memcpy(lengths, s->last_fs_lengths, s->last_nfs * sizeof(double));
    }
    return s->last_nfs;
}

/* delta_tot_table.c:613-617 */
double ko_get_delta_tot(double dnu, double dcdm, double OmegaNua3, double Omeganonu, double Omeganu1, double partnu)
{
    const double fcdm = 1 - OmegaNua3 / (Omeganonu + Omeganu1);
    return fcdm * (dcdm + dnu * OmegaNua3 / (Omeganonu + Omeganu1 * partnu));
}

/* ------------------------------------------------------------------ get_delta_nu */
typedef struct {
    double k, mnubykT, qc, nufrac_low;
    gsl_interp *spline, *fs_spline;
    const double *scale, *delta_tot, *fsscales, *fslengths;
    const ko_bg *bg;
} dnu_params;

/* delta_tot_table.c:492-500 */
static double get_delta_nu_int(double logai, void *params)
{
    const dnu_params *p = (const dnu_params *)params;
    const double fsl_aia = gsl_interp_eval(p->fs_spline, p->fsscales, p->fslengths, logai, NULL);
    const double delta_tot_at_a = gsl_interp_eval(p->spline, p->scale, p->delta_tot, logai, NULL);
    const double specJ = ko_specialJ(p->k * fsl_aia / p->mnubykT, p->qc, p->nufrac_low);
    const double ai = exp(logai);
    return fsl_aia / (ai * ko_hubble(p->bg, ai)) * specJ * delta_tot_at_a;
}

/* Gauss-Legendre n-point nodes/weights on [-1,1] (positive half), computed by Newton
 * iteration on P_n so no table is transcribed. */
static void gl_nodes(int n, double *X, double *Wt)
{
    for (int i = 0; i < n / 2; i++) {
        double x = cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0;
        for (int it = 0; it < 100; it++) {
            double p0 = 1, p1 = x;
            for (int k = 2; k <= n; k++) {
                const double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (x * p1 - p0) / (x * x - 1);
            const double dx = p1 / dp;
            x -= dx;
            if (fabs(dx) < 1e-16)
                break;
        }
        X[i] = x;
        Wt[i] = 2 / ((1 - x * x) * dp * dp);
    }
}
static double GL8_X[4], GL8_W[4], GL4_X[2], GL4_W[2];
static int gl_ready = 0;
static void gl8_init(void)
{
    if (gl_ready)
        return;
    gl_nodes(8, GL8_X, GL8_W);
    gl_nodes(4, GL4_X, GL4_W);
    gl_ready = 1;
}

/* fslength table: mode 0 = one QAG per node (delta_tot_table.c:574-584);
 * mode 1 = cumulative 8-point Gauss-Legendre over the uniform node segments;
 * exact = QAG at 1e-13 per node. */
static void fs_table(ko_state *s, double a, int Nfs, double *fsscales, double *fslengths, int *status)
{
    const double la = log(a), l0 = log(s->TimeTransfer);
    for (int ik = 0; ik < Nfs; ik++)
        fsscales[ik] = l0 + ik * (la - l0) / (Nfs - 1.);
    if (s->exact) {
        gsl_function F;
        F.function = &fslength_int;
        F.params = (void *)s->bg;
        double acc = fsscales[Nfs - 1] < la ? gk61_plain(&F, fsscales[Nfs - 1], la) : 0;
        fslengths[Nfs - 1] = s->light * acc;
        for (int ik = Nfs - 2; ik >= 0; ik--) {
            acc += gk61_plain(&F, fsscales[ik], fsscales[ik + 1]);
            fslengths[ik] = s->light * acc;
        }
        return;
    }
    if (s->fs_mode == 0) {
        for (int ik = 0; ik < Nfs; ik++)
            fslengths[ik] = ko_fslength(s->bg, fsscales[ik], la, s->light, status);
        return;
    }
    gl8_init();
    /* fs_mode 1: 8-point rule per segment; fs_mode 2: 4-point rule; fs_mode 3: the GPU's
     * rule, 2-point where the knots are closer than 1.5e-3 in log a, else 4-point */
    static const double GL2_X[1] = {0.57735026918962576451}, GL2_W[1] = {1.0};
    const int use2 = s->fs_mode == 3 && (la - l0) / (Nfs - 1.) < 1.5e-3;
    const int np = use2 ? 1 : (s->fs_mode >= 2 ? 2 : 4);
    const double *GX = use2 ? GL2_X : (s->fs_mode >= 2 ? GL4_X : GL8_X);
    const double *GW = use2 ? GL2_W : (s->fs_mode >= 2 ? GL4_W : GL8_W);
    double acc = 0;
    /* tail beyond the last node (non-zero only through rounding of the node formula) */
    if (fsscales[Nfs - 1] < la) {
        const double c = 0.5 * (fsscales[Nfs - 1] + la), h = 0.5 * (la - fsscales[Nfs - 1]);
        for (int j = 0; j < np; j++)
            acc += GW[j] * h * (fslength_int(c - h * GX[j], s->bg) + fslength_int(c + h * GX[j], s->bg));
    }
    fslengths[Nfs - 1] = fsscales[Nfs - 1] >= la ? 0 : s->light * acc;
    for (int ik = Nfs - 2; ik >= 0; ik--) {
        const double c = 0.5 * (fsscales[ik] + fsscales[ik + 1]), h = 0.5 * (fsscales[ik + 1] - fsscales[ik]);
        double seg = 0;
        for (int j = 0; j < np; j++)
            seg += GW[j] * (fslength_int(c - h * GX[j], s->bg) + fslength_int(c + h * GX[j], s->bg));
        acc += h * seg;
        fslengths[ik] = s->light * acc;
    }
}

/* d specialJ_fit / dx (derivative of the rational fit of delta_tot_table.c:417-428) */
static double specialJ_fit_deriv(double x)
{
    if (x <= 0.)
        return 0.;
    const double x2 = x * x, x4 = x2 * x2, x8 = x4 * x4;
    const double p = exp(4.1811 * log(x));
    const double N = 1. + 0.0168 * x2 + 0.0407 * x4;
    const double D = 1. + 2.1734 * x2 + 1.6787 * p + 0.1467 * x8;
    const double dN = 0.0336 * x + 0.1628 * x2 * x;
    const double dD = 4.3468 * x + 1.6787 * 4.1811 * p / x + 1.1736 * x4 * x2 * x;
    return (dN * D - N * dD) / (D * D);
}

/* Adjoint of one bin's time integral over the final QAG subdivision in w: the
 * derivative of the computed Kronrod sums with the subdivision held fixed.  Adds
 * prefac*sbar*d(integral)/d(row values) to Dbar_row[Na] and returns
 * d(integral)/d(mass) (J argument only). */
static double adj_bin(const ko_state *s, const dnu_params *p, const gsl_integration_workspace *w, int Na,
                      double *Dbar_row, double sbar)
{
    static const double XK[31] = KSP_GK61_XK_INIT;
    static const double WK[31] = KSP_GK61_WK_INIT;
    double *ybar = (double *)calloc(2 * (size_t)Na, sizeof(double));
    double *cbar = ybar + Na;
    const double *x = p->scale, *y = p->delta_tot;
    const double *cc = Na > 2 ? p->spline->c : NULL;
    double mder = 0;
    for (size_t iv = 0; iv < w->size; iv++) {
        const double c = 0.5 * (w->alist[iv] + w->blist[iv]), h = 0.5 * (w->blist[iv] - w->alist[iv]);
        for (int jn = 0; jn < 61; jn++) {
            const double xn = jn < 30 ? c - h * XK[jn] : (jn < 60 ? c + h * XK[jn - 30] : c);
            const double wt = (jn < 60 ? WK[jn % 30] : WK[30]) * h;
            const double fsl = gsl_interp_eval(p->fs_spline, p->fsscales, p->fslengths, xn, NULL);
            size_t lo = 0, hi = (size_t)Na - 1;
            while (hi > lo + 1) {
                const size_t mid = (lo + hi) / 2;
                if (x[mid] > xn) hi = mid; else lo = mid;
            }
            const size_t i = lo;
            const double hh = x[i + 1] - x[i], dx = xn - x[i];
            const double S = gsl_interp_eval(p->spline, p->scale, p->delta_tot, xn, NULL);
            const double xj = p->k * fsl / p->mnubykT;
            const double J = ko_specialJ(xj, p->qc, p->nufrac_low);
            const double ai = exp(xn);
            const double g = fsl / (ai * ko_hubble(p->bg, ai));
            const double u = wt * g * J;
            ybar[i] += u * (1 - dx / hh);
            ybar[i + 1] += u * (dx / hh);
            if (cc) {
                cbar[i] += u * (dx * (-2 * hh / 3) + dx * dx - dx * dx * dx / (3 * hh));
                cbar[i + 1] += u * (dx * (-hh / 3) + dx * dx * dx / (3 * hh));
            }
            if (p->qc <= 0)
                mder += wt * g * specialJ_fit_deriv(xj) * (-xj / (p->mnubykT * s->bg->kBtnu)) * S;
        }
    }
    if (cc && Na > 2) {
        /* c (interior) = A^-1 rhs(y); z = A^-1 cbar (A symmetric), ybar += rhs^T z */
        const int m = Na - 2;
        double *diag = (double *)malloc(2 * (size_t)m * sizeof(double));
        double *z = diag + m;
        for (int u = 0; u < m; u++) {
            diag[u] = 2.0 * ((x[u + 1] - x[u]) + (x[u + 2] - x[u + 1]));
            z[u] = cbar[u + 1];
        }
        for (int u = 1; u < m; u++) {
            const double off = x[u + 1] - x[u];
            const double f = off / diag[u - 1];
            diag[u] -= f * off;
            z[u] -= f * z[u - 1];
        }
        z[m - 1] /= diag[m - 1];
        for (int u = m - 1; u-- > 0;)
            z[u] = (z[u] - (x[u + 2] - x[u + 1]) * z[u + 1]) / diag[u];
        for (int u = 0; u < m; u++) {
            const double ih0 = 1.0 / (x[u + 1] - x[u]), ih1 = 1.0 / (x[u + 2] - x[u + 1]);
            ybar[u] += 3 * z[u] * ih0;
            ybar[u + 1] -= 3 * z[u] * (ih0 + ih1);
            ybar[u + 2] += 3 * z[u] * ih1;
        }
        free(diag);
    }
    for (int j = 0; j < Na; j++)
        Dbar_row[j] += s->prefac * sbar * ybar[j];
    free(ybar);
    return mder;
}

/* delta_tot_table.c:507-611 */
int ko_get_delta_nu(ko_state *s, double a, const double *wavenum, double *dnu, double mnu)
{
    const ko_bg *bg = s->bg;
    int status = 0;
    double qc = 0;
    const int Na = s->ia;
    const double mnubykT = mnu / bg->kBtnu;
    double relerr = 1e-6;
    ensure_handler();
    s->last_max_intervals = 0;
    s->last_total_intervals = 0;
    const double fsl_A0a = s->exact ? fslength_exact(bg, log(s->TimeTransfer), log(a), s->light, &status)
                                    : ko_fslength(bg, log(s->TimeTransfer), log(a), s->light, &status);
    const double deriv_prefac = s->TimeTransfer * (ko_hubble(bg, s->TimeTransfer) / s->light) * s->TimeTransfer;
    for (int ik = 0; ik < s->nk; ik++) {
        const double specJ = ko_specialJ(wavenum[ik] * fsl_A0a / (mnubykT > 0 ? mnubykT : 1), qc, bg->nufrac_low[0]);
        dnu[ik] = specJ * s->nu_init[ik] * (1. + deriv_prefac * fsl_A0a);
        if (s->adj_dnu_bar && mnubykT > 0) {
            const double x0 = wavenum[ik] * fsl_A0a / mnubykT;
            s->adj_mbar[s->adj_species] += s->adj_dnu_bar[ik] * s->adj_weight * specialJ_fit_deriv(x0) * (-x0 / mnu) *
                                           s->nu_init[ik] * (1. + deriv_prefac * fsl_A0a);
        }
    }
    const double partnu = ko_particle_nu_fraction(bg, a, 0);
    if (partnu > 0) {
        if (1 - partnu < 1e-3)
            return status;
        qc = bg->vcrit * mnubykT;
        relerr /= (1. + 1e-5 - ko_particle_nu_fraction(bg, a, 0));
    }
    if (Na > 1 && mnubykT > 0) {
        const int Nfs = Na * 16;
        double *fsscales = (double *)malloc(Nfs * sizeof(double));
        double *fslengths = (double *)malloc(Nfs * sizeof(double));
        fs_table(s, a, Nfs, fsscales, fslengths, &status);
        free(s->last_fs_scales);
        s->last_fs_scales = (double *)malloc(2 * (size_t)Nfs * sizeof(double));
        s->last_fs_lengths = s->last_fs_scales + Nfs;
        memcpy(s->last_fs_scales, fsscales, Nfs * sizeof(double));
        memcpy(s->last_fs_lengths, fslengths, Nfs * sizeof(double));
        s->last_nfs = Nfs;
        dnu_params p;
        p.spline = gsl_interp_alloc(Na > 2 ? gsl_interp_cspline : gsl_interp_linear, Na);
        p.fs_spline = gsl_interp_alloc(gsl_interp_cspline, Nfs);
        p.scale = s->scalefact;
        p.mnubykT = mnubykT;
        p.qc = qc;
        p.nufrac_low = bg->nufrac_low[0];
        p.fsscales = fsscales;
        p.fslengths = fslengths;
        p.bg = bg;
        gsl_interp_init(p.fs_spline, fsscales, fslengths, Nfs);
        gsl_function F;
        F.function = &get_delta_nu_int;
        F.params = &p;
        for (int ik = 0; ik < s->nk; ik++) {
            p.k = wavenum[ik];
            p.delta_tot = s->delta_tot + (size_t)ik * s->namax;
            gsl_interp_init(p.spline, p.scale, p.delta_tot, Na);
            double d_nu_tmp = 0;
            if (!s->exact) {
                gsl_integration_workspace *wk = NULL;
                d_nu_tmp = qag_run_keep(&F, log(s->TimeTransfer), log(a), relerr, &status, &wk);
                if (s->adj_dnu_bar) {
                    const double sbar = s->adj_dnu_bar[ik] * s->adj_weight;
                    s->adj_mbar[s->adj_species] +=
                        s->prefac * sbar * adj_bin(s, &p, wk, Na, s->adj_Dbar + (size_t)ik * Na, sbar);
                }
                gsl_integration_workspace_free(wk);
                const int ni = gslsub_last_qag_intervals();
                if (ni > s->last_max_intervals)
                    s->last_max_intervals = ni;
                s->last_total_intervals += ni;
            } else {
                /* all-FP64 reference: integrate exactly knot segment by knot segment
                 * (breakpoints: the delta_tot knots and the fslength knots). */
                /* stop at the last knot of either spline (they can differ from log a by
                 * rounding); the sliver beyond has zero width in exact arithmetic */
                const double lo = log(s->TimeTransfer);
                double hi = log(a);
                if (fsscales[Nfs - 1] < hi)
                    hi = fsscales[Nfs - 1];
                if (s->scalefact[Na - 1] < hi)
                    hi = s->scalefact[Na - 1];
                int i_fs = 0, i_dt = 0;
                double x = lo;
                while (x < hi) {
                    double nx = hi;
                    while (i_fs < Nfs && fsscales[i_fs] <= x)
                        i_fs++;
                    while (i_dt < Na && s->scalefact[i_dt] <= x)
                        i_dt++;
                    if (i_fs < Nfs && fsscales[i_fs] < nx)
                        nx = fsscales[i_fs];
                    if (i_dt < Na && s->scalefact[i_dt] < nx)
                        nx = s->scalefact[i_dt];
                    d_nu_tmp += gk61_plain(&F, x, nx);
                    x = nx;
                }
            }
            dnu[ik] += s->prefac * d_nu_tmp;
        }
        gsl_interp_free(p.spline);
        gsl_interp_free(p.fs_spline);
        free(fsscales);
        free(fslengths);
    }
    return status;
}

/* delta_tot_table.c:153-172 */
int ko_get_delta_nu_combined(ko_state *s, double a, const double *wavenum, double *dnu)
{
    const ko_bg *bg = s->bg;
    const double Omega_nu_tot = ko_omega_nu_nopart(bg, a);
    int status = 0;
    memset(dnu, 0, s->nk * sizeof(double));
    double *single = (double *)malloc((s->nk > 0 ? s->nk : 1) * sizeof(double));
    for (int mi = 0; mi < NUSPECIES; mi++) {
        if (bg->deg[mi] > 0) {
            const double omeganu = bg->deg[mi] * ko_omega_nu_single(bg, a, mi);
            s->adj_weight = omeganu / Omega_nu_tot;
            s->adj_species = mi;
            int st = ko_get_delta_nu(s, a, wavenum, single, s->mJ_set ? s->mJ[mi] : bg->tab[mi].mnu);
            if (st && !status)
                status = st;
            for (int ik = 0; ik < s->nk; ik++)
                dnu[ik] += single[ik] * omeganu / Omega_nu_tot;
        }
    }
    free(single);
    return status;
}

/* delta_tot_table.c:177-191 */
static int update_delta_tot(ko_state *s, double a, const double *dcdm, const double *dnu, int overwrite)
{
    const ko_bg *bg = s->bg;
    const double OmegaNua3 = ko_omega_nu_nopart(bg, a) * pow(a, 3);
    const double OmegaNu1 = ko_omega_nu(bg, 1);
    const double partnu = ko_particle_nu_fraction(bg, a, 0);
    if (!overwrite) {
        if (s->ia >= s->namax)
            return 2025; /* the reference has no check here: it would write past the table */
        s->ia++;
    }
    s->scalefact[s->ia - 1] = log(a);
    for (int ik = 0; ik < s->nk; ik++)
        s->delta_tot[(size_t)ik * s->namax + s->ia - 1] =
            ko_get_delta_tot(dnu[ik], dcdm[ik], OmegaNua3, s->Omeganonu, OmegaNu1, partnu);
    return 0;
}

/* delta_tot_table.c:79-149 */
int ko_delta_tot_init(ko_state *s, int nk_in, const double *wavenum, const double *dcdm, double Time)
{
    const ko_bg *bg = s->bg;
    for (int ik = 0; ik < s->ia; ik++) {
        if (log(Time) <= s->scalefact[ik]) {
            s->ia = ik;
            break;
        }
    }
    if (Time > s->TimeTransfer + 0.01 && s->ia == 0)
        return 2023;
    if (Time < s->TimeTransfer - 1e-5)
        return 2024;
    if (nk_in > s->nk_alloc)
        return 2011;
    if (!s->t_logk)
        return 2019;
    ensure_handler();
    s->nk = nk_in;
    const double OmegaNua3 = ko_omega_nu_nopart(bg, s->TimeTransfer) * pow(s->TimeTransfer, 3);
    const double OmegaNu1 = ko_omega_nu(bg, 1);
    gsl_interp *spline = gsl_interp_alloc(gsl_interp_cspline, s->ntrans);
    gsl_interp_init(spline, s->t_logk, s->t_Tnu, s->ntrans);
    if (log(wavenum[s->nk - 1]) > s->t_logk[s->ntrans - 1]) {
        gsl_interp_free(spline);
        return 2;
    }
    g_gsl_err = 0;
    for (int ik = 0; ik < s->nk; ik++) {
        const double T = gsl_interp_eval(spline, s->t_logk, s->t_Tnu, log(wavenum[ik]), NULL);
        const double OmegaMa = (s->Omeganonu + OmegaNua3);
        if (s->ia == 0) {
            const double partnu = ko_particle_nu_fraction(bg, s->TimeTransfer, 0);
            s->delta_tot[(size_t)ik * s->namax] = ko_get_delta_tot(dcdm[ik] * T, dcdm[ik], OmegaNua3, s->Omeganonu, OmegaNu1, partnu);
        }
        s->nu_init[ik] = s->delta_tot[(size_t)ik * s->namax] * OmegaMa / (OmegaMa - OmegaNua3 + T * OmegaNua3) * fabs(T);
        s->wavenum[ik] = wavenum[ik];
    }
    gsl_interp_free(spline);
    if (g_gsl_err)
        return 2001;
    if (s->ia == 0) {
        s->scalefact[0] = log(s->TimeTransfer);
        s->ia = 1;
    }
    int st = ko_get_delta_nu_combined(s, exp(s->scalefact[s->ia - 1]), wavenum, s->nu_last);
    s->init_done = 1;
    return st;
}

/* delta_tot_table.c:193-250 */
int ko_get_delta_nu_update(ko_state *s, double a, int nk_in, const double *keff, const double *dcdm, double *dnu)
{
    int st;
    if (!s->init_done) {
        st = ko_delta_tot_init(s, nk_in, keff, dcdm, a);
        if (st)
            return st;
    }
    if (nk_in != s->nk)
        return 2002;
    if (s->nk < 2)
        return 2003;
    if (log(a) - s->scalefact[s->ia - 1] < FLOAT_ACC) {
        for (int ik = 0; ik < s->nk; ik++)
            dnu[ik] = s->nu_last[ik];
        return 0;
    }
    st = update_delta_tot(s, a, dcdm, s->nu_last, 0);
    if (st)
        return st;
    st = ko_get_delta_nu_combined(s, a, keff, dnu);
    for (int ik = 0; ik < s->nk; ik++)
        s->nu_last[ik] = dnu[ik];
    if (a >= exp(s->scalefact[s->ia - 2]) + 0.009)
        update_delta_tot(s, a, dcdm, dnu, 1);
    else
        s->ia--;
    for (int ik = 0; ik < s->nk; ik++) {
        if (isnan(dnu[ik]))
            return 2004;
        if (dnu[ik] < 0)
            dnu[ik] = 0;
    }
    return st;
}

/* ================================================================== binning */
/* powerspectrum.c:8-12 (fftw_real = float) */
static float onedinvwindow(int kx, int n) { return kx ? M_PI * kx / (n * sin(M_PI * kx / (float)n)) : 1.0; }
/* powerspectrum.c:16-24 */
static float invwindow(int kx, int ky, int kz, int n)
{
    if (n == 0)
        return 0;
    const float iwx = onedinvwindow(kx, n), iwy = onedinvwindow(ky, n), iwz = onedinvwindow(kz, n);
    return pow(iwx * iwy * iwz, 2);
}
static double onedinvwindow_d(int kx, int n) { return kx ? M_PI * kx / (n * sin(M_PI * kx / (double)n)) : 1.0; }
static double invwindow_d(int kx, int ky, int kz, int n)
{
    const double w = onedinvwindow_d(kx, n) * onedinvwindow_d(ky, n) * onedinvwindow_d(kz, n);
    return w * w;
}

typedef struct {
    int dims, nrbins, i0, i1, startslab, mode;
    const float *grid;
    double binsperunit;
    double *power, *keffs;
    long long *count;
    double F0sq;
} ps_job;

#define KVAL(n, dims) ((n) <= (dims) / 2 ? (n) : ((n) - (dims)))

/* powerspectrum.c:56-89 for slabs [i0, i1) */
static void *ps_worker(void *arg)
{
    ps_job *j = (ps_job *)arg;
    const int dims = j->dims, nz = dims / 2 + 1;
    for (int i = j->i0; i < j->i1; i++) {
        const size_t indx = (size_t)(i - j->startslab) * dims * nz;
        const int ki = KVAL(i, dims);
        for (int jj = 0; jj < dims; jj++) {
            const int kj = KVAL(jj, dims);
            const size_t indy = indx + (size_t)jj * nz;
            for (int k = 0; k <= dims / 2; k++) {
                const float re = j->grid[2 * (indy + k)], im = j->grid[2 * (indy + k) + 1];
                const long long k2 = (long long)ki * ki + (long long)kj * kj + (long long)k * k;
                if (k2 == 0)
                    continue;
                const double kk = sqrt((double)k2);
                const int psindex = (int)floor(j->binsperunit * log(kk));
                const int w = (k == 0 || k == dims / 2) ? 1 : 2;
                double p;
                if (j->mode == 0) {
                    const float F2 = re * re + im * im;
                    const float iw = invwindow(ki, kj, k, dims);
                    p = F2 * pow(iw, 2);
                } else {
                    const double F2 = (double)re * re + (double)im * im;
                    const double iw = invwindow_d(ki, kj, k, dims);
                    p = F2 * iw * iw;
                }
                j->power[psindex] += w * p;
                j->count[psindex] += w;
                j->keffs[psindex] += w * kk;
            }
        }
    }
    return NULL;
}

/* powerspectrum.c:33-117 */
int ko_total_powerspectrum(int dims, const float *grid, int nrbins, int startslab, int nslab, double *power,
                           long long *count, double *keffs, int mode, int partial, double *F0sq, int nthreads)
{
    if (nthreads < 1)
        nthreads = 1;
    if (nthreads > nslab)
        nthreads = nslab > 0 ? nslab : 1;
    const double binsperunit = (nrbins - 1) / log(sqrt(3) * dims / 2.0);
    double total_mass2 = 0;
    if (startslab == 0 && nslab > 0) {
        if (mode == 0)
            total_mass2 = grid[0] * grid[0] + grid[1] * grid[1];
        else
            total_mass2 = (double)grid[0] * grid[0] + (double)grid[1] * grid[1];
    }
    ps_job *jobs = (ps_job *)calloc(nthreads, sizeof(ps_job));
    pthread_t *th = (pthread_t *)calloc(nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; t++) {
        ps_job *j = &jobs[t];
        j->dims = dims;
        j->nrbins = nrbins;
        j->startslab = startslab;
        j->i0 = startslab + (int)((long long)nslab * t / nthreads);
        j->i1 = startslab + (int)((long long)nslab * (t + 1) / nthreads);
        j->mode = mode;
        j->grid = grid;
        j->binsperunit = binsperunit;
        j->power = (double *)calloc(nrbins, sizeof(double));
        j->keffs = (double *)calloc(nrbins, sizeof(double));
        j->count = (long long *)calloc(nrbins, sizeof(long long));
        if (nthreads > 1)
            pthread_create(&th[t], NULL, ps_worker, j);
        else
            ps_worker(j);
    }
    memset(power, 0, nrbins * sizeof(double));
    memset(keffs, 0, nrbins * sizeof(double));
    memset(count, 0, nrbins * sizeof(long long));
    for (int t = 0; t < nthreads; t++) {
        if (nthreads > 1)
            pthread_join(th[t], NULL);
        for (int b = 0; b < nrbins; b++) {
            power[b] += jobs[t].power[b];
            keffs[b] += jobs[t].keffs[b];
            count[b] += jobs[t].count[b];
        }
        free(jobs[t].power);
        free(jobs[t].keffs);
        free(jobs[t].count);
    }
    free(jobs);
    free(th);
    if (F0sq)
        *F0sq = total_mass2;
    if (partial)
        return nrbins;
    int nonzero = 0;
    for (int i = 0; i < nrbins; i++) {
        power[i] /= total_mass2;
        if (count[i]) {
            keffs[i] /= count[i];
            power[i] /= count[i];
        }
    }
    for (int i = 0; i < nrbins; i++) {
        if (count[i]) {
            if (nonzero < i) {
                power[nonzero] = power[i];
                keffs[nonzero] = keffs[i];
                count[nonzero] = count[i];
            }
            nonzero++;
        }
    }
    return nonzero;
}

/* ================================================================== interpolation + multiply */
/* delta_pow.c:19-37 */
double ko_dnudcdm(const double *logk, const double *ratio, int n, double norm, double kk, int *warn)
{
    if (kk < logk[0] && kk > logk[0] - log(2))
        kk = logk[0];
    if (kk < logk[0] - log(2)) {
        if (warn)
            *warn = 1;
        kk = logk[0];
    }
    if (kk > logk[n - 1])
        kk = logk[n - 1];
    size_t lo = 0, hi = (size_t)n - 1;
    while (hi > lo + 1) {
        const size_t mid = (lo + hi) / 2;
        if (logk[mid] > kk)
            hi = mid;
        else
            lo = mid;
    }
    const double dx = kk - logk[lo];
    const double y = ratio[lo] + dx * ((ratio[lo + 1] - ratio[lo]) / (logk[lo + 1] - logk[lo]));
    return norm * y;
}

typedef struct {
    void *grid;
    int pmgrid, slab0, y0, y1, nk, mode, nan;
    double BoxSize, norm;
    const double *logk, *ratio;
} mul_job;

/* interface_gadget.c:163-188 for slabs [y0, y1) */
static void *mul_worker(void *arg)
{
    mul_job *j = (mul_job *)arg;
    const int pm = j->pmgrid;
    for (int y = j->y0; y < j->y1; y++)
        for (int x = 0; x < pm; x++)
            for (int z = 0; z < pm / 2 + 1; z++) {
                const double kx = x > pm / 2 ? x - pm : x;
                const double ky = y > pm / 2 ? y - pm : y;
                const double kz = z > pm / 2 ? z - pm : z;
                double k2 = kx * kx + ky * ky + kz * kz;
                if (k2 <= 0)
                    continue;
                k2 = log(sqrt(k2) * 2 * M_PI / j->BoxSize);
                const double smth = 1 + ko_dnudcdm(j->logk, j->ratio, j->nk, j->norm, k2, NULL);
                if (isnan(smth))
                    j->nan = 1;
                const size_t ip = (size_t)pm * (pm / 2 + 1) * (y - j->slab0) + (size_t)(pm / 2 + 1) * x + z;
                if (j->mode == 0) {
                    float *g = (float *)j->grid;
                    g[2 * ip] *= smth;
                    g[2 * ip + 1] *= smth;
                } else {
                    double *g = (double *)j->grid;
                    g[2 * ip] *= smth;
                    g[2 * ip + 1] *= smth;
                }
            }
    return NULL;
}

int ko_apply_correction(void *grid, int pmgrid, int slab0, int nslab, double BoxSize, const double *logk,
                        const double *ratio, int nk, double norm, int mode, int nthreads)
{
    if (nthreads < 1)
        nthreads = 1;
    if (nthreads > nslab)
        nthreads = nslab > 0 ? nslab : 1;
    mul_job *jobs = (mul_job *)calloc(nthreads, sizeof(mul_job));
    pthread_t *th = (pthread_t *)calloc(nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; t++) {
        mul_job *j = &jobs[t];
        j->grid = grid;
        j->pmgrid = pmgrid;
        j->slab0 = slab0;
        j->y0 = slab0 + (int)((long long)nslab * t / nthreads);
        j->y1 = slab0 + (int)((long long)nslab * (t + 1) / nthreads);
        j->nk = nk;
        j->mode = mode;
        j->BoxSize = BoxSize;
        j->norm = norm;
        j->logk = logk;
        j->ratio = ratio;
        if (nthreads > 1)
            pthread_create(&th[t], NULL, mul_worker, j);
        else
            mul_worker(j);
    }
    int nan = 0;
    for (int t = 0; t < nthreads; t++) {
        if (nthreads > 1)
            pthread_join(th[t], NULL);
        nan |= jobs[t].nan;
    }
    free(jobs);
    free(th);
    return nan ? 5 : 0;
}

/* interface_common.c:125-148 */
int ko_neutrino_power_internal(ko_state *s, double Time, double *keff, double *dcdm, double *dnu, int nk,
                               double *norm)
{
    int st = ko_get_delta_nu_update(s, Time, nk, keff, dcdm, dnu);
    if (st)
        return st;
    for (int i = 0; i < nk; i++) {
        keff[i] = log(keff[i]);
        dcdm[i] = dnu[i] / dcdm[i];
    }
    const double OmegaNu_nop = ko_omega_nu_nopart(s->bg, Time);
    const double omega_hybrid = ko_omega_nu(s->bg, Time) - OmegaNu_nop;
    *norm = OmegaNu_nop / (s->Omeganonu / pow(Time, 3) + omega_hybrid);
    return 0;
}

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* interface_gadget.c:75-102 + 158-194, single rank */
int ko_add_nu_power_to_rhogrid(ko_state *s, double Time, double BoxSize, float *grid, int pmgrid, int slab0,
                               int nslab, int nthreads, int *nk_out, double *keff_o, double *dcdm_o, double *dnu_o,
                               double *logk_o, double *ratio_o, double *norm_o, double *t_stages)
{
    const int nb = s->nk_alloc;
    double *power = (double *)malloc(nb * sizeof(double));
    double *keff = (double *)malloc(nb * sizeof(double));
    double *dnu = (double *)malloc(nb * sizeof(double));
    long long *count = (long long *)malloc(nb * sizeof(long long));
    double t0 = now_s();
    const int nk = ko_total_powerspectrum(pmgrid, grid, nb, slab0, nslab, power, count, keff, 0, 0, NULL, nthreads);
    double t1 = now_s();
    const double scale = pow(BoxSize, -3);
    for (int i = 0; i < nk; i++) {
        power[i] = sqrt(power[i] / scale);
        keff[i] *= (2 * M_PI / BoxSize);
    }
    if (keff_o)
        memcpy(keff_o, keff, nk * sizeof(double));
    if (dcdm_o)
        memcpy(dcdm_o, power, nk * sizeof(double));
    double norm = 0;
    int st = ko_neutrino_power_internal(s, Time, keff, power, dnu, nk, &norm);
    double t2 = now_s();
    if (!st)
        st = ko_apply_correction(grid, pmgrid, slab0, nslab, BoxSize, keff, power, nk, norm, 0, nthreads);
    double t3 = now_s();
    if (nk_out)
        *nk_out = nk;
    if (dnu_o)
        memcpy(dnu_o, dnu, nk * sizeof(double));
    if (logk_o)
        memcpy(logk_o, keff, nk * sizeof(double));
    if (ratio_o)
        memcpy(ratio_o, power, nk * sizeof(double));
    if (norm_o)
        *norm_o = norm;
    if (t_stages) {
        t_stages[0] = t1 - t0;
        t_stages[1] = t2 - t1;
        t_stages[2] = t3 - t2;
    }
    free(power);
    free(keff);
    free(dnu);
    free(count);
    return st;
}

/* The same step in FP64 throughout (test infrastructure: the precision reference):
 * |F|^2 and the window in double (ko_total_powerspectrum mode 1), the delta_nu integral
 * as the state's options say (exact = 1 for ~1e-13), the correction applied to a double
 * copy of the grid.  grid_in: float complex [nslab][N][N/2+1]; grid_out: double complex. */
int ko_add_nu_power_to_rhogrid_fp64(ko_state *s, double Time, double BoxSize, const float *grid_in, double *grid_out,
                                    int pmgrid, int nthreads, int *nk_out, double *keff_o, double *dcdm_o,
                                    double *dnu_o, double *ratio_o, double *norm_o)
{
    const int nb = s->nk_alloc;
    double *power = (double *)malloc(nb * sizeof(double));
    double *keff = (double *)malloc(nb * sizeof(double));
    double *dnu = (double *)malloc(nb * sizeof(double));
    long long *count = (long long *)malloc(nb * sizeof(long long));
    const int nk = ko_total_powerspectrum(pmgrid, grid_in, nb, 0, pmgrid, power, count, keff, 1, 0, NULL, nthreads);
    const double scale = pow(BoxSize, -3);
    for (int i = 0; i < nk; i++) {
        power[i] = sqrt(power[i] / scale);
        keff[i] *= (2 * M_PI / BoxSize);
    }
    if (keff_o)
        memcpy(keff_o, keff, nk * sizeof(double));
    if (dcdm_o)
        memcpy(dcdm_o, power, nk * sizeof(double));
    double norm = 0;
    int st = ko_neutrino_power_internal(s, Time, keff, power, dnu, nk, &norm);
    const size_t n2 = (size_t)2 * pmgrid * pmgrid * (pmgrid / 2 + 1);
    for (size_t i = 0; i < n2; i++)
        grid_out[i] = grid_in[i];
    if (!st)
        st = ko_apply_correction(grid_out, pmgrid, 0, pmgrid, BoxSize, keff, power, nk, norm, 1, nthreads);
    if (nk_out)
        *nk_out = nk;
    if (dnu_o)
        memcpy(dnu_o, dnu, nk * sizeof(double));
    if (ratio_o)
        memcpy(ratio_o, power, nk * sizeof(double));
    if (norm_o)
        *norm_o = norm;
    free(power);
    free(keff);
    free(dnu);
    free(count);
    return st;
}

/* ================================================================== differentiation (test infrastructure) */
int ko_state_set_vectors(ko_state *s, const double *nu_init, const double *nu_last, const double *wavenum, int nk)
{
    if (nk > s->nk_alloc)
        return 2011;
    s->nk = nk;
    memcpy(s->nu_init, nu_init, nk * sizeof(double));
    memcpy(s->nu_last, nu_last, nk * sizeof(double));
    memcpy(s->wavenum, wavenum, nk * sizeof(double));
    s->init_done = 1;
    return 0;
}

void ko_state_set_jmass(ko_state *s, const double *mJ)
{
    if (!mJ) {
        s->mJ_set = 0;
        return;
    }
    s->mJ_set = 1;
    for (int i = 0; i < NUSPECIES; i++)
        s->mJ[i] = mJ[i];
}

/* One integrator call at a that leaves the state unchanged: provisional row from dcdm
 * and delta_nu_last (delta_tot_table.c:222), delta_nu (unclamped), row dropped.  With
 * dnu_bar: D_bar[nk][Na] (Na = ia+1; column Na-1 is the provisional row) and the
 * derivative with respect to the mass inside J, per species. */
int ko_dnu_diff(ko_state *s, double a, const double *wavenum, const double *dcdm, double *dnu, const double *dnu_bar,
                double *D_bar, double *mJ_bar)
{
    if (!s->init_done)
        return 10003;
    int st = update_delta_tot(s, a, dcdm, s->nu_last, 0);
    if (st)
        return st;
    const int Na = s->ia;
    if (dnu_bar) {
        s->adj_dnu_bar = dnu_bar;
        s->adj_Dbar = D_bar;
        memset(D_bar, 0, (size_t)s->nk * Na * sizeof(double));
        memset(s->adj_mbar, 0, sizeof(s->adj_mbar));
    }
    st = ko_get_delta_nu_combined(s, a, wavenum, dnu);
    if (dnu_bar) {
        for (int i = 0; i < NUSPECIES; i++)
            mJ_bar[i] = s->adj_mbar[i];
        s->adj_dnu_bar = NULL;
        s->adj_Dbar = NULL;
    }
    s->ia--;
    return st;
}
