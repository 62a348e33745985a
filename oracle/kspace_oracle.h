/* oracle/kspace_oracle.h -- CPU restatement of the kspace-neutrinos hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU product is compared with
 * (and the "port" CPU baseline where the reference sources are absent).  The product
 * never links it.  Each function names the reference file:line it restates.
 * Parity: pinned against the reference C built here from its own sources
 * (oracle/_ref) and against the reference test suite's known answers.
 */
#ifndef KSPACE_ORACLE_H
#define KSPACE_ORACLE_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct ko_bg ko_bg;       /* background cosmology: Omega_nu(a), H(a) */
typedef struct ko_state ko_state; /* integrator state (delta_tot history)     */

/* omega_nu_single.c:16-51 init_omega_nu + the test hubble_function
 * (delta_tot_table_test.c:25-45; curvature as gadget-2/0003 patch:38). */
ko_bg *ko_bg_new(const double MNu[3], double a0, double HubbleParam, double tcmb0, double Omega0,
                 double OmegaLambda, double UnitTime_in_s, int radiation);
void ko_bg_free(ko_bg *bg);
/* omega_nu_single.c:230-240 */
int ko_bg_hybrid(ko_bg *bg, double vcrit, double light, double nu_crit_time);
double ko_hubble(const ko_bg *bg, double a);
double ko_omega_nu(const ko_bg *bg, double a);            /* :55-65 */
double ko_omega_nu_nopart(const ko_bg *bg, double a);     /* :69-74 */
double ko_omegag(const ko_bg *bg, double a);              /* :77-81 */
double ko_omega_nu_single(const ko_bg *bg, double a, int i); /* :262-279 */
double ko_particle_nu_fraction(const ko_bg *bg, double a, int i); /* :246-257 */
double ko_nufrac_low(double qc);                          /* :214-228 */
void ko_bg_info(const ko_bg *bg, double *rhocrit, double *kBtnu, int *deg, double *mnu);
int ko_bg_table(const ko_bg *bg, int i, double *loga, double *rhonu);

/* delta_tot_table.c:457-463, 394-407 */
double ko_specialJ(double x, double qc, double nufrac_low);
double ko_fslength(const ko_bg *bg, double logai, double logaf, double light, int *status);

/* delta_tot_table.c:25-60 allocate_delta_tot_table */
ko_state *ko_state_new(ko_bg *bg, int nk_alloc, double TimeTransfer, double TimeMax, double Omega0,
                       double UnitTime_in_s, double UnitLength_in_cm);
void ko_state_free(ko_state *s);
/* transfer table (transfer_init.h:10-15): log k and T_nu/T_nonu */
int ko_state_set_transfer(ko_state *s, const double *logk, const double *T_nu, int n);
/* interface_common.c:166-180 set_nu_state (flat [nk][ia]) */
int ko_state_set_nu_state(ko_state *s, const double *scalefact, const double *delta_tot, int nk, int ia);
/* flat copies of the state */
void ko_state_get(const ko_state *s, int *ints /*nk,nk_alloc,namax,ia,init_done*/, double *scalefact,
                  double *delta_tot /*[nk_alloc][namax]*/, double *vec3 /*init,last,wavenum [nk_alloc]*/);
void ko_state_scalars(const ko_state *s, double *out /*prefac,Omeganonu,light,TimeTransfer*/);
void ko_state_set_ia(ko_state *s, int ia);

/* Integration options (not reference behaviour; used to measure the discretisation):
 *  fs_mode 0: fslength table by one QAG per node (the reference, delta_tot_table.c:574-584)
 *  fs_mode 1: fslength table by a cumulative 8-point Gauss-Legendre sum over the
 *             uniform nodes; fs_mode 2: the same with a 4-point rule (what the GPU does)
 *  exact    : if nonzero, the delta_nu time integral and fslength are integrated to
 *             ~1e-13 relative (QAG at epsrel 1e-13 on each knot segment): the all-FP64
 *             reference of the same splines.                                          */
void ko_state_options(ko_state *s, int fs_mode, int exact);

/* delta_tot_table.c:79-149 */
int ko_delta_tot_init(ko_state *s, int nk, const double *wavenum, const double *dcdm, double Time);
/* delta_tot_table.c:193-250 (keff = k, not log k; dcdm = sqrt(P_cdm)) */
int ko_get_delta_nu_update(ko_state *s, double a, int nk, const double *keff, const double *dcdm, double *dnu);
/* delta_tot_table.c:153-172 */
int ko_get_delta_nu_combined(ko_state *s, double a, const double *wavenum, double *dnu);
/* delta_tot_table.c:507-611 */
int ko_get_delta_nu(ko_state *s, double a, const double *wavenum, double *dnu, double mnu);
/* delta_tot_table.c:613-617 */
double ko_get_delta_tot(double dnu, double dcdm, double OmegaNua3, double Omeganonu, double Omeganu1, double partnu);
/* diagnostics of the last ko_get_delta_nu: QAG intervals per bin (max, total) */
void ko_last_qag_stats(const ko_state *s, int *max_intervals, long long *total_intervals);
/* the fslength table (scales, values) of the last ko_get_delta_nu with Na > 1 */
int ko_last_fs_table(const ko_state *s, double *scales, double *lengths);

/* powerspectrum.c:33-117.  mode 0 = reference float semantics (|F|^2 and the window
 * in float, sums in double); mode 1 = everything promoted to double.
 * partial != 0: return the per-rank sums before the allreduce / normalisation
 * (power[nb], count[nb], ksum[nb], *F0sq), no compaction.  nthreads >= 1 splits the
 * slabs across threads as MPI ranks would (merge = the allreduce). */
int ko_total_powerspectrum(int dims, const float *grid, int nrbins, int startslab, int nslab, double *power,
                           long long *count, double *keffs, int mode, int partial, double *F0sq, int nthreads);

/* delta_pow.c:19-37 get_dnudcdm_powerspec (linear interpolation, clamped) */
double ko_dnudcdm(const double *logk, const double *ratio, int n, double norm, double kk, int *warn);

/* interface_gadget.c:163-188: multiply every mode by 1 + dnudcdm(log|k|).  mode 0 =
 * reference semantics (float mode times double factor, rounded to float); mode 1 = the
 * grid is given as double complex and multiplied in double. Returns 5 on NaN. */
int ko_apply_correction(void *grid, int pmgrid, int slab0, int nslab, double BoxSize, const double *logk,
                        const double *ratio, int nk, double norm, int mode, int nthreads);

/* interface_common.c:125-148: logk, ratio and kspace_prefac from keff/dcdm/dnu */
int ko_neutrino_power_internal(ko_state *s, double Time, double *keff, double *dcdm, double *dnu, int nk,
                               double *norm);

/* interface_gadget.c:158-194 add_nu_power_to_rhogrid as one call (single rank).
 * Outputs (optional): nk, keff (k), dcdm, dnu, logk/ratio/norm of the interpolator. */
/* the same step in FP64 throughout (binning mode 1, correction on a double grid) */
int ko_add_nu_power_to_rhogrid_fp64(ko_state *s, double Time, double BoxSize, const float *grid_in, double *grid_out,
                                    int pmgrid, int nthreads, int *nk_out, double *keff_o, double *dcdm_o,
                                    double *dnu_o, double *ratio_o, double *norm_o);
int ko_add_nu_power_to_rhogrid(ko_state *s, double Time, double BoxSize, float *grid, int pmgrid, int slab0,
                               int nslab, int nthreads, int *nk_out, double *keff, double *dcdm, double *dnu,
                               double *logk, double *ratio, double *norm, double *t_stages);

/* ---- differentiation support ---- */
/* set delta_nu_init, delta_nu_last, wavenum and mark the table initialised */
int ko_state_set_vectors(ko_state *s, const double *nu_init, const double *nu_last, const double *wavenum, int nk);
/* mass (eV) used inside J per species (NULL: the background's masses) */
void ko_state_set_jmass(ko_state *s, const double *mJ);
/* integrator call that leaves the state unchanged; optional FP64 adjoint */
int ko_dnu_diff(ko_state *s, double a, const double *wavenum, const double *dcdm, double *dnu, const double *dnu_bar,
                double *D_bar, double *mJ_bar);

#ifdef __cplusplus
}
#endif
#endif
