/* oracle/ref_entry.c -- ctypes-friendly entry points into the UNMODIFIED reference C
 * (built from the reference sources by oracle/Makefile into oracle/_ref/).  TEST
 * INFRASTRUCTURE ONLY.  Every call that can reach the reference's terminate() runs
 * under a setjmp guard and returns the reference error code (0 = success).
 * Struct accessors copy reference state into flat caller-owned arrays.
 */
#include <setjmp.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "gadget_defines.h"
#include "omega_nu_single.h"
#include "transfer_init.h"
#include "delta_tot_table.h"
#include "delta_pow.h"
#include "powerspectrum.h"
#include "interface_common.h"
#include "interface_gadget.h"

jmp_buf *ref_guard_push(jmp_buf *env);
void ref_guard_pop(jmp_buf *old);
int ref_last_terminate_code(void);
void ref_init_hubble(const _omega_nu *omnu, double Omega0, double OmegaLambda, double UnitTime_in_s,
                     int radiation);

#define GUARDED(body)                                   \
    do {                                                \
        jmp_buf env;                                    \
        jmp_buf *old = ref_guard_push(&env);            \
        if (setjmp(env)) {                              \
            ref_guard_pop(old);                         \
            return ref_last_terminate_code();           \
        }                                               \
        body;                                           \
        ref_guard_pop(old);                             \
        return 0;                                       \
    } while (0)

/* ---- omega_nu (omega_nu_single.c) ---- */
_omega_nu *ref_omnu_new(void) { return (_omega_nu *)calloc(1, sizeof(_omega_nu)); }
void ref_omnu_free(_omega_nu *p) { free(p); }
int ref_init_omega_nu(_omega_nu *omnu, const double *MNu, double a0, double h, double tcmb0)
{
    GUARDED(init_omega_nu(omnu, MNu, a0, h, tcmb0));
}
int ref_init_hybrid_nu(_omega_nu *omnu, const double *mnu, double vcrit, double light, double nu_crit_time)
{
    GUARDED(init_hybrid_nu(&omnu->hybnu, mnu, vcrit, light, nu_crit_time, omnu->kBtnu));
}
double ref_get_omega_nu(const _omega_nu *o, double a) { return get_omega_nu(o, a); }
double ref_get_omega_nu_nopart(const _omega_nu *o, double a) { return get_omega_nu_nopart(o, a); }
double ref_get_omegag(const _omega_nu *o, double a) { return get_omegag(o, a); }
double ref_omega_nu_single(const _omega_nu *o, double a, int i) { return omega_nu_single(o, a, i); }
double ref_particle_nu_fraction(const _omega_nu *o, double a, int i) { return particle_nu_fraction(&o->hybnu, a, i); }
int ref_nufrac_low(double qc, double *out) { GUARDED(*out = nufrac_low(qc)); }
/* scalar fields: rhocrit, kBtnu, degeneracies, rho table */
void ref_omnu_info(const _omega_nu *o, double *rhocrit, double *kBtnu, int *deg)
{
    *rhocrit = o->rhocrit;
    *kBtnu = o->kBtnu;
    for (int i = 0; i < NUSPECIES; i++)
        deg[i] = o->nu_degeneracies[i];
}
/* 200-entry loga/rhonu table of species i; returns 0 if it has no table */
int ref_omnu_table(const _omega_nu *o, int i, double *loga, double *rhonu)
{
    if (!o->RhoNuTab[i] || !o->RhoNuTab[i]->loga)
        return 0;
    memcpy(loga, o->RhoNuTab[i]->loga, 200 * sizeof(double));
    memcpy(rhonu, o->RhoNuTab[i]->rhonu, 200 * sizeof(double));
    return 200;
}
double ref_rho_nu(const _omega_nu *o, int i, double a) { return rho_nu(o->RhoNuTab[i], a, o->kBtnu); }

/* ---- hubble (test form, delta_tot_table_test.c:25-45) ---- */
static int g_use_global = 0;
void ref_set_hubble(const _omega_nu *omnu, double Omega0, double OmegaLambda, double UnitTime_in_s, int radiation)
{
    g_use_global = 0;
    ref_init_hubble(omnu, Omega0, OmegaLambda, UnitTime_in_s, radiation);
}
double ref_hubble(double a) { return hubble_function(a); }

/* ---- transfer_init.c ---- */
_transfer_init_table *ref_transfer_new(void) { return (_transfer_init_table *)calloc(1, sizeof(_transfer_init_table)); }
int ref_transfer_read(_transfer_init_table *t, double BoxSize, double UnitLength_in_cm, double InputUnit, const char *file)
{
    GUARDED(allocate_transfer_init_table(t, BoxSize, UnitLength_in_cm, InputUnit, file));
}
/* set the table from arrays (the reference reads it from a CAMB file) */
void ref_transfer_set(_transfer_init_table *t, const double *logk, const double *T_nu, int n)
{
    t->NPowerTable = n;
    t->logk = (double *)malloc(2 * n * sizeof(double));
    t->T_nu = t->logk + n;
    memcpy(t->logk, logk, n * sizeof(double));
    memcpy(t->T_nu, T_nu, n * sizeof(double));
}
int ref_transfer_get(const _transfer_init_table *t, double *logk, double *T_nu)
{
    if (logk) {
        memcpy(logk, t->logk, t->NPowerTable * sizeof(double));
        memcpy(T_nu, t->T_nu, t->NPowerTable * sizeof(double));
    }
    return t->NPowerTable;
}
void ref_transfer_free(_transfer_init_table *t)
{
    if (t && t->logk)
        free(t->logk);
    free(t);
}

/* ---- delta_tot_table.c ---- */
_delta_tot_table *ref_dtot_new(void) { return (_delta_tot_table *)calloc(1, sizeof(_delta_tot_table)); }
int ref_allocate_delta_tot_table(_delta_tot_table *d, int nk, double TimeTransfer, double TimeMax, double Omega0,
                                 const _omega_nu *omnu, double UnitTime_in_s, double UnitLength_in_cm)
{
    GUARDED(allocate_delta_tot_table(d, nk, TimeTransfer, TimeMax, Omega0, omnu, UnitTime_in_s, UnitLength_in_cm, 0));
}
void ref_dtot_free(_delta_tot_table *d)
{
    if (d && d->scalefact)
        free_delta_tot_table(d);
    free(d);
}
int ref_delta_tot_init(_delta_tot_table *d, int nk, const double *wavenum, const double *dcdm,
                       const _transfer_init_table *t, double Time)
{
    GUARDED(delta_tot_init(d, nk, wavenum, dcdm, t, Time));
}
int ref_get_delta_nu_update(_delta_tot_table *d, double a, int nk, const double *keff, const double *dcdm,
                            double *dnu, _transfer_init_table *t)
{
    GUARDED(get_delta_nu_update(d, a, nk, keff, dcdm, dnu, t));
}
int ref_get_delta_nu_combined(const _delta_tot_table *d, double a, const double *wavenum, double *dnu)
{
    GUARDED(get_delta_nu_combined(d, a, wavenum, dnu));
}
int ref_get_delta_nu(const _delta_tot_table *d, double a, const double *wavenum, double *dnu, double mnu)
{
    GUARDED(get_delta_nu(d, a, wavenum, dnu, mnu));
}
int ref_update_delta_tot(_delta_tot_table *d, double a, const double *dcdm, const double *dnu, int overwrite)
{
    GUARDED(update_delta_tot(d, a, dcdm, dnu, overwrite));
}
int ref_read_all_nu_state(_delta_tot_table *d, char *file) { GUARDED(read_all_nu_state(d, file)); }
int ref_save_all_nu_state(const _delta_tot_table *d, char *file) { GUARDED(save_all_nu_state(d, file)); }
int ref_save_nu_power(const _delta_tot_table *d, double Time, int snapnum, const char *dir, int *ret)
{
    GUARDED(*ret = save_nu_power(d, Time, snapnum, dir));
}
double ref_specialJ(double x, double qc, double nufrac) { return specialJ(x, qc, nufrac); }
int ref_fslength(double logai, double logaf, double light, double *out) { GUARDED(*out = fslength(logai, logaf, light)); }
double ref_get_delta_tot(double dnu, double dcdm, double OmegaNua3, double Omeganonu, double Omeganu1, double partnu)
{
    return get_delta_tot(dnu, dcdm, OmegaNua3, Omeganonu, Omeganu1, partnu);
}
/* integer fields: nk, nk_allocated, namax, ia, delta_tot_init_done */
void ref_dtot_ints(const _delta_tot_table *d, int *out)
{
    out[0] = d->nk; out[1] = d->nk_allocated; out[2] = d->namax; out[3] = d->ia; out[4] = d->delta_tot_init_done;
}
/* double fields: delta_nu_prefac, Omeganonu, light, TimeTransfer */
void ref_dtot_scalars(const _delta_tot_table *d, double *out)
{
    out[0] = d->delta_nu_prefac; out[1] = d->Omeganonu; out[2] = d->light; out[3] = d->TimeTransfer;
}
void ref_dtot_set_ia(_delta_tot_table *d, int ia) { d->ia = ia; }
/* flat copies: scalefact[namax], delta_tot[nk_alloc][namax], vectors[3][nk_alloc] */
void ref_dtot_get(const _delta_tot_table *d, double *scalefact, double *delta_tot, double *vec3)
{
    if (scalefact)
        memcpy(scalefact, d->scalefact, d->namax * sizeof(double));
    if (delta_tot)
        memcpy(delta_tot, d->delta_tot[0], (size_t)d->namax * d->nk_allocated * sizeof(double));
    if (vec3)
        memcpy(vec3, d->delta_nu_init, 3 * d->nk_allocated * sizeof(double));
}
void ref_dtot_set(_delta_tot_table *d, const double *scalefact, const double *delta_tot, int ia, int nk)
{
    memcpy(d->scalefact, scalefact, d->namax * sizeof(double));
    memcpy(d->delta_tot[0], delta_tot, (size_t)d->namax * d->nk_allocated * sizeof(double));
    d->ia = ia;
    d->nk = nk;
}

/* ---- powerspectrum.c ---- */
int ref_total_powerspectrum(int dims, fftw_complex *grid, int nrbins, int startslab, int nslab, double *power,
                            long long *count, double *keffs, int *nk_out)
{
    GUARDED(*nk_out = total_powerspectrum(dims, grid, nrbins, startslab, nslab, power, count, keffs, MPI_COMM_WORLD));
}

/* ---- delta_pow.c ---- */
_delta_pow *ref_dpow_new(void) { return (_delta_pow *)calloc(1, sizeof(_delta_pow)); }
int ref_init_delta_pow(_delta_pow *p, double *logkk, double *ratio, int n, double norm)
{
    GUARDED(init_delta_pow(p, logkk, ratio, n, norm));
}
int ref_get_dnudcdm_powerspec(_delta_pow *p, double kk, double *out) { GUARDED(*out = get_dnudcdm_powerspec(p, kk)); }
void ref_dpow_free(_delta_pow *p)
{
    if (p && p->spline)
        free_d_pow(p);
    free(p);
}

/* ---- interface_common.c / interface_gadget.c (global singletons) ---- */
void ref_set_kspace_params(const char *transfer_file, double TimeTransfer, double InputUnit, const double *MNu,
                           int hybrid, double vcrit, double nu_crit_time)
{
    memset(&kspace_params, 0, sizeof(kspace_params));
    strncpy(kspace_params.KspaceTransferFunction, transfer_file ? transfer_file : "", 499);
    kspace_params.TimeTransfer = TimeTransfer;
    kspace_params.InputSpectrum_UnitLength_in_cm = InputUnit;
    for (int i = 0; i < NUSPECIES; i++)
        kspace_params.MNu[i] = MNu[i];
    kspace_params.hybrid_neutrinos_on = hybrid;
    kspace_params.vcrit = vcrit;
    kspace_params.nu_crit_time = nu_crit_time;
}
int ref_InitOmegaNu(double h, double tcmb0) { GUARDED(InitOmegaNu(h, tcmb0, MPI_COMM_WORLD)); }
double ref_OmegaNu(double a) { return OmegaNu(a); }
double ref_OmegaNu_nopart(double a) { return OmegaNu_nopart(a); }
int ref_allocate_kspace_memory(int nk, double BoxSize, double UnitTime_in_s, double UnitLength_in_cm, double Omega0,
                               char *snapdir, double TimeMax)
{
    GUARDED(allocate_kspace_memory(nk, 0, BoxSize, UnitTime_in_s, UnitLength_in_cm, Omega0, snapdir, TimeMax, MPI_COMM_WORLD));
}
int ref_add_nu_power_to_rhogrid(double Time, double BoxSize, fftw_complex *grid, int pmgrid, int slab0, int nslab)
{
    GUARDED(add_nu_power_to_rhogrid(Time, BoxSize, grid, pmgrid, slab0, nslab, MPI_COMM_WORLD));
}
int ref_compute_total_power_spectrum(double Time, double BoxSize, fftw_complex *grid, int pmgrid, int slab0, int nslab)
{
    GUARDED(compute_total_power_spectrum(Time, BoxSize, grid, pmgrid, slab0, nslab, MPI_COMM_WORLD));
}
int ref_compute_neutrino_power_from_cdm(double Time, const double *keff, const double *P, const long *Nmodes, int nk,
                                        double *logk_out, double *ratio_out, double *norm_out, int *nbins_out)
{
    _delta_pow dp;
    GUARDED({
        dp = compute_neutrino_power_from_cdm(Time, keff, P, Nmodes, nk, MPI_COMM_WORLD);
        for (int i = 0; i < dp.nbins; i++) {
            logk_out[i] = dp.logkk[i];
            ratio_out[i] = dp.delta_ratio[i];
        }
        *norm_out = dp.norm;
        *nbins_out = dp.nbins;
        free_d_pow(&dp);
    });
}
int ref_save_nu_state(char *file) { GUARDED(save_nu_state(file)); }
int ref_save_neutrino_power(double Time, int snapnum, const char *dir, int *ret)
{
    GUARDED(*ret = save_neutrino_power(Time, snapnum, dir));
}
int ref_save_total_power(double Time, int snapnum, const char *dir, int *ret)
{
    GUARDED(*ret = save_total_power(Time, snapnum, dir));
}
int ref_particle_nu_active(double a) { return particle_nu_active(a); }
/* get_nu_state mallocs; copy into caller buffers then free */
int ref_get_nu_state(double *scalefact, double *delta_tot, size_t *nk, size_t *ia, size_t cap)
{
    double *s = NULL, *d = NULL;
    get_nu_state(&s, &d, nk, ia);
    if (*ia <= cap && scalefact)
        memcpy(scalefact, s, *ia * sizeof(double));
    if ((*nk) * (*ia) <= cap * cap && delta_tot)
        memcpy(delta_tot, d, (*nk) * (*ia) * sizeof(double));
    free(s);
    free(d);
    return 0;
}
int ref_set_nu_state(double *scalefact, double *delta_tot, size_t nk, size_t ia)
{
    GUARDED(set_nu_state(scalefact, delta_tot, nk, ia, MPI_COMM_WORLD));
}
/* the global integrator table (interface_common.c:21) */
extern _delta_tot_table delta_tot_table;
_delta_tot_table *ref_global_dtot(void) { return &delta_tot_table; }

/* hubble bound to the global omega_nu table (for the interface-level path) */
static double g_O0, g_OL, g_UT, g_h, g_tcmb;
static int g_rad;
void ref_set_hubble_global(double Omega0, double OmegaLambda, double UnitTime_in_s, int radiation, double h, double tcmb0)
{
    g_O0 = Omega0; g_OL = OmegaLambda; g_UT = UnitTime_in_s; g_rad = radiation; g_h = h; g_tcmb = tcmb0;
    g_use_global = 1;
}
int ref_hubble_uses_global(void) { return g_use_global; }
double ref_hubble_global(double a)
{
    /* gadget-2/0003-...patch:38-52 with KSPACE_NEUTRINOS_2 and INCLUDE_RADIATION */
    double omega_tot = g_O0 / pow(a, 3) + g_OL + (1. - g_OL - g_O0) / (a * a);
    omega_tot += OmegaNu(a) - OmegaNu(1) / pow(a, 3);
    if (g_rad) {
        const double rhocrit = (3 * HUBBLE * g_h * HUBBLE * g_h) / (8 * M_PI * 6.67408e-8);
        omega_tot += 4 * 5.670373e-5 / (LIGHTCGS * LIGHTCGS * LIGHTCGS) * pow(g_tcmb, 4) / rhocrit / pow(a, 4);
    }
    return HUBBLE * g_UT * sqrt(omega_tot);
}
