/* kspace_gpu.h -- C ABI of libkspace_gb300.so, the GB300 implementation of the
 * kspace-neutrinos linear-response neutrino force correction.
 *
 * Plain C types only (pointers, sizes, doubles).  A context replaces the reference's
 * process-global singletons (interface_common.c:17-26, interface_gadget.c:19-21); the
 * reference-named drop-in entry points (add_nu_power_to_rhogrid, ...) are provided on
 * top of this ABI by kspace_neutrinos_dropin.h / dropin/kspace_dropin.c.
 *
 * Every function returns a status: KSPACE_OK (0), or the reference's terminate()
 * code for the same failure (values below 10000), or a KSPACE_ERR_* code of this
 * library (10000 and up).  Grid pointers may be device pointers (used in place) or
 * host pointers (copied to the device and back inside the call).  Calls on one
 * context are not thread-safe; they run on the context's CUDA stream and return after
 * the results are complete.
 */
#ifndef KSPACE_GPU_H
#define KSPACE_GPU_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes: reference terminate() codes ---- */
#define KSPACE_OK 0
#define KSPACE_ERR_NOMEM 1              /* interface_gadget.c:88 */
#define KSPACE_ERR_KMAX 2               /* delta_tot_table.c:113-114: k beyond the transfer table */
#define KSPACE_ERR_GRID_NAN 5           /* interface_gadget.c:183-184: correction factor is NaN */
#define KSPACE_ERR_GSL 2001             /* integration / interpolation failure (delta_tot_table.c:70-73) */
#define KSPACE_ERR_NK_MISMATCH 2002     /* delta_tot_table.c:203-204 */
#define KSPACE_ERR_NK_SMALL 2003        /* delta_tot_table.c:205-206 */
#define KSPACE_ERR_DNU_NAN 2004         /* delta_tot_table.c:239-244 */
#define KSPACE_ERR_STATE_SHORT 2006     /* delta_tot_table.c:281 */
#define KSPACE_ERR_STATE_START 2007     /* delta_tot_table.c:291-292 */
#define KSPACE_ERR_NK_ALLOC 2011        /* delta_tot_table.c:97-98 */
#define KSPACE_ERR_SAVE_OPEN 2012       /* delta_tot_table.c:317-318 */
#define KSPACE_ERR_TRANSFER_OPEN 2019   /* transfer_init.c:19-20 */
#define KSPACE_ERR_TRANSFER_SHORT 2021  /* transfer_init.c:78-79 */
#define KSPACE_ERR_NO_RESUME 2023       /* delta_tot_table.c:91-92 */
#define KSPACE_ERR_TIME_BEFORE 2024     /* delta_tot_table.c:94-95 */
/* ---- status codes of this library ---- */
#define KSPACE_ERR_NAMAX 2025           /* history table full (the reference writes past it) */
#define KSPACE_ERR_CUDA 10001           /* a CUDA call failed */
#define KSPACE_ERR_ARG 10002            /* invalid argument */
#define KSPACE_ERR_ORDER 10003          /* call made before the state it needs exists */
#define KSPACE_ERR_HUBBLE 10004         /* host hubble_function differs from the device model */
#define KSPACE_ERR_TIMEOUT 10005        /* a bounded device wait expired */

typedef struct kspace_ctx kspace_ctx;

/* Sums `count` doubles in place across all ranks (an MPI_Allreduce with MPI_SUM).
 * Used once per call of the grid binning, on the per-bin sums, as the reference does
 * at powerspectrum.c:91-95.  Returns 0 on success. */
typedef int (*kspace_allreduce_fn)(double *buf, int count, void *user);

/* ---- lifecycle ---- */
int kspace_gpu_create(kspace_ctx **ctx, int device);
int kspace_gpu_destroy(kspace_ctx *ctx);
const char *kspace_gpu_error_string(int status);
/* Run on this CUDA stream (a cudaStream_t; NULL = the context's own stream). */
int kspace_gpu_set_stream(kspace_ctx *ctx, void *cuda_stream);
/* Multi-rank slab decomposition: reduction of the per-bin sums (NULL = one rank). */
int kspace_gpu_set_allreduce(kspace_ctx *ctx, kspace_allreduce_fn fn, void *user);
/* Kernel variant selection for the grid passes.  tma: 5 (default) = binning over
 * row-aligned runs of 17 modes (whole grid rows per bulk copy) with the reference's float
 * roundings and float-pair sums, 6 = the same with FP32 run sums; 3 / 4 = warp-pipelined
 * binning over 16-mode TMA rows (exact / FP32 run sums); 1 = CTA-tiled TMA engine with a
 * thread per 16-mode row, 2 = two threads per row; 0 = plain loads.  The correction pass
 * is warp-pipelined for tma >= 3.  rows_per_cta: 32 x warps per CTA for tma >= 3
 * (128/256); stages: per warp (or tile group) for tma >= 3 (2/3/4), per CTA otherwise;
 * qag_warps: warps per block of the integrator (1..4).  Values < 0 (rows, stages,
 * qag_warps: <= 0) keep the current setting. */
int kspace_gpu_set_tuning(kspace_ctx *ctx, int tma, int rows_per_cta, int stages, int qag_warps);

/* ---- background: Omega_nu(a), H(a) ----
 * Replaces InitOmegaNu / init_omega_nu (interface_common.c:183-188, omega_nu_single.c:16-51).
 * The Fermi-Dirac tables are integrated on the device. */
int kspace_gpu_init_omega_nu(kspace_ctx *ctx, const double MNu[3], double TimeTransfer, double HubbleParam,
                             double tcmb0);
/* init_hybrid_nu (omega_nu_single.c:230-240; called from interface_common.c:80-81) */
int kspace_gpu_init_hybrid_nu(kspace_ctx *ctx, double vcrit, double light, double nu_crit_time);
/* The fields of a host's _hybrid_nu (omega_nu_single.h:51-64) as they are: enabled,
 * vcrit as a fraction of light speed, nu_crit_time, nufrac_low[3]. */
int kspace_gpu_set_hybrid(kspace_ctx *ctx, int enabled, double vcrit_frac, double nu_crit_time,
                          const double *nufrac_low);
/* Parameters of the host's hubble_function (gadget_defines.h:11), evaluated on the
 * device as H0 sqrt(Omega_nonu/a^3 + (1-Omega0-OmegaLambda)/a^2 + OmegaLambda +
 * Omega_nu(a) [+ Omega_g/a^4]) (delta_tot_table_test.c:33-45, gadget-2/0003 patch:38). */
int kspace_gpu_set_hubble(kspace_ctx *ctx, double Omega0, double OmegaLambda, double UnitTime_in_s,
                          int include_radiation);
/* A host hubble_function of another form: n >= 4 samples H[i] = H(a_i) at log a_i =
 * loga_lo + i * dloga.  log H is interpolated by a natural cubic spline in log a (the
 * end segments continue past the table); replaces the form set by kspace_gpu_set_hubble. */
int kspace_gpu_set_hubble_table(kspace_ctx *ctx, double loga_lo, double dloga, int n, const double *H);
/* Compare the device H(a) with n samples of the host's hubble_function; returns
 * KSPACE_ERR_HUBBLE if any relative difference exceeds rtol. */
int kspace_gpu_check_hubble(kspace_ctx *ctx, const double *a, const double *H, int n, double rtol,
                            double *max_rel);
/* OmegaNu / OmegaNu_nopart / particle_nu_active (interface_common.c:29-39,190-197) */
int kspace_gpu_omega_nu(kspace_ctx *ctx, double a, double *omega_nu, double *omega_nu_nopart);
int kspace_gpu_particle_nu_active(kspace_ctx *ctx, double a, int *active);
/* hubble_function as evaluated on the device model */
int kspace_gpu_hubble(kspace_ctx *ctx, double a, double *H);

/* ---- integrator state ----
 * allocate_delta_tot_table (delta_tot_table.c:25-60) as called by allocate_kspace_memory
 * (interface_common.c:91). */
int kspace_gpu_alloc_table(kspace_ctx *ctx, int nk_alloc, double TimeTransfer, double TimeMax, double Omega0,
                           double UnitTime_in_s, double UnitLength_in_cm);
/* The transfer table of transfer_init.h:10-15: log k (internal units) and T_nu/T_nonu. */
int kspace_gpu_set_transfer(kspace_ctx *ctx, const double *logk, const double *T_nu, int n);
/* allocate_transfer_init_table (transfer_init.c:9-83): read a CAMB transfer file. */
int kspace_gpu_read_transfer_file(kspace_ctx *ctx, double BoxSize, double UnitLength_in_cm,
                                  double InputSpectrum_UnitLength_in_cm, const char *path, int *nrows);
/* set_nu_state (interface_common.c:166-180): flat delta_tot[nk][ia] (host or device memory) */
int kspace_gpu_set_nu_state(kspace_ctx *ctx, const double *scalefact, const double *delta_tot, size_t nk,
                            size_t ia);
/* get_nu_state (interface_common.c:150-164).  Pass NULL arrays to query nk and ia. */
int kspace_gpu_get_nu_state(kspace_ctx *ctx, double *scalefact, double *delta_tot, size_t *nk, size_t *ia);
/* read_all_nu_state / save_all_nu_state / save_nu_power (delta_tot_table.c:254-374),
 * same text formats. */
int kspace_gpu_read_nu_state(kspace_ctx *ctx, const char *path);
int kspace_gpu_save_nu_state(kspace_ctx *ctx, const char *path);
int kspace_gpu_save_nu_power(kspace_ctx *ctx, double Time, int snapnum, const char *OutputDir);
/* ints[0..4] = nk, nk_allocated, namax, ia, delta_tot_init_done */
int kspace_gpu_table_info(kspace_ctx *ctx, int *ints);
/* delta_nu_init, delta_nu_last, wavenum (each nk_alloc doubles; NULL to skip) */
int kspace_gpu_get_vectors(kspace_ctx *ctx, double *nu_init, double *nu_last, double *wavenum);

/* ---- the hot path ---- */
/* total_powerspectrum (powerspectrum.c:33-117): outputs compacted to the non-empty
 * bins, power normalised by |F(0)|^2 and the mode count. */
int kspace_gpu_total_powerspectrum(kspace_ctx *ctx, int dims, const void *grid, int nrbins, int startslab,
                                   int nslab, double *power, long long *count, double *keffs, int *nk_out);
/* get_delta_nu_update (delta_tot_table.c:193-250): keff = k (not log k), P_cdm_sqrt =
 * sqrt(P_cdm); writes delta_nu[nk]. */
int kspace_gpu_get_delta_nu_update(kspace_ctx *ctx, double a, int nk, const double *keff, const double *P_cdm_sqrt,
                                   double *delta_nu);
/* delta_tot_init (delta_tot_table.c:79-149) on its own: wavenum = k (not log k) and
 * dcdm = sqrt(P_cdm) of nk bins (host or device memory).  Truncates a resumed history
 * after Time, builds delta_nu_init from the transfer table, the first row on a fresh
 * start, and delta_nu_last. */
int kspace_gpu_delta_tot_init(kspace_ctx *ctx, int nk, const double *wavenum, const double *dcdm, double Time);
/* get_delta_nu (delta_tot_table.c:507-611): delta_nu of one mass state of mass mnu (eV)
 * at scale factor a from the stored rows [0, ia), at the bins' k = wavenum[nk] (host or
 * device memory); delta_nu: host memory. */
int kspace_gpu_get_delta_nu(kspace_ctx *ctx, double a, int nk, const double *wavenum, double *delta_nu, double mnu);
/* get_delta_nu_combined (delta_tot_table.c:153-172): the species-weighted sum of
 * get_delta_nu over the non-degenerate mass states, from the stored rows. */
int kspace_gpu_get_delta_nu_combined(kspace_ctx *ctx, double a, int nk, const double *wavenum, double *delta_nu);
/* update_delta_tot (delta_tot_table.c:177-191): the last row (overwrite != 0) or a new
 * row at a, from dcdm = sqrt(P_cdm) and delta_nu of the stored bins. */
int kspace_gpu_update_delta_tot(kspace_ctx *ctx, double a, const double *dcdm, const double *dnu, int overwrite);
/* The integrator state in the layout of _delta_tot_table (delta_tot_table.h:17-57): nk,
 * ia, the init flag, scalefact[ia], rows of the history at stride ld doubles (row ik at
 * delta_tot + ik * ld, columns [0, ia)), delta_nu_init, delta_nu_last, wavenum (nk each;
 * NULL = unchanged).  Host memory. */
int kspace_gpu_set_table(kspace_ctx *ctx, int nk, int ia, int init_done, const double *scalefact,
                         const double *delta_tot, size_t ld, const double *nu_init, const double *nu_last,
                         const double *wavenum);
/* Read it back: columns [col0, ia) of scalefact and of every row, the vectors, nk, ia and
 * the init flag; any output may be NULL. */
int kspace_gpu_get_table(kspace_ctx *ctx, int col0, int *nk, int *ia, int *init_done, double *scalefact,
                         double *delta_tot, size_t ld, double *nu_init, double *nu_last, double *wavenum);
/* specialJ (delta_tot_table.c:457-463; the fit, or the truncated series when qc > 0) and
 * nufrac_low (omega_nu_single.c:214-228) of n values on the device; ctx may be NULL (the
 * current device).  fslength (delta_tot_table.c:394-407) of n intervals with the
 * context's H(a). */
int kspace_gpu_special_j(kspace_ctx *ctx, const double *x, int n, double qc, double nufrac_low, double *out);
int kspace_gpu_nufrac_low(kspace_ctx *ctx, const double *qc, int n, double *out);
int kspace_gpu_fslength(kspace_ctx *ctx, const double *logai, const double *logaf, int n, double light,
                        double *out);
/* omega_nu_single (omega_nu_single.c:262-279), get_omegag (:77-81), and the _omega_nu
 * fields rhocrit, kBtnu, nu_degeneracies[3] and hybnu.nufrac_low[3] (NULL to skip). */
int kspace_gpu_omega_nu_single(kspace_ctx *ctx, double a, int i, double *out);
int kspace_gpu_omega_g(kspace_ctx *ctx, double a, double *out);
int kspace_gpu_background_info(kspace_ctx *ctx, double *rhocrit, double *kBtnu, int *deg, double *nufrac_low);
/* compute_neutrino_power_from_cdm (interface_common.c:106-123): outputs the
 * interpolation table of delta_nu/delta_cdm (log k, ratio, norm = kspace_prefac). */
int kspace_gpu_compute_neutrino_power_from_cdm(kspace_ctx *ctx, double Time, const double *keff_in,
                                               const double *P_cdm, const long *Nmodes, int nk_in, double *logk,
                                               double *ratio, double *norm, int *nbins);
/* add_nu_power_to_rhogrid (interface_gadget.c:158-194): bin, integrate, multiply every
 * mode of the slab by 1 + norm * ratio(log|k|).  grid: fftw_complex[nslab][pmgrid][pmgrid/2+1]. */
int kspace_gpu_add_nu_power_to_rhogrid(kspace_ctx *ctx, double Time, double BoxSize, void *grid, int pmgrid,
                                       int slabstart_y, int nslab_y);
/* The grid multiply alone (interface_gadget.c:163-188 with delta_pow.c:19-37) for a
 * given interpolation table. */
int kspace_gpu_apply_delta_pow(kspace_ctx *ctx, double BoxSize, void *grid, int pmgrid, int slabstart_y, int nslab_y,
                               int nrbins, const double *logk, const double *ratio, int nk, double norm);
/* compute_total_power_spectrum / save_total_power (interface_gadget.c:114-144,196-224) */
int kspace_gpu_compute_total_power_spectrum(kspace_ctx *ctx, double Time, double BoxSize, const void *grid,
                                            int pmgrid, int slabstart_y, int nslab_y);
int kspace_gpu_save_total_power(kspace_ctx *ctx, double Time, int snapnum, const char *OutputDir);

/* ---- differentiation (one step with the integrator state held fixed) ---- */
/* Set delta_nu_init, delta_nu_last and wavenum (nk each) and mark the table initialised:
 * restores a native snapshot (the reference keeps these in _delta_tot_table,
 * delta_tot_table.h:40-46) and fixes the state a differentiable step starts from. */
int kspace_gpu_set_vectors(kspace_ctx *ctx, const double *nu_init, const double *nu_last, const double *wavenum,
                           int nk);
/* The mass (eV) inside the free-streaming argument of J per mass state (the mnu
 * argument of get_delta_nu, delta_tot_table.c:507); NULL restores the background's. */
int kspace_gpu_set_jmass(kspace_ctx *ctx, const double MNu[3]);
/* Forward of one step (interface_gadget.c:158-194 without updating the state):
 * grid_out = grid_in * (1 + correction) and pnu_out[nk] = delta_nu^2.  Device pointers;
 * grid_out may equal grid_in.  store_intervals keeps each QAG subdivision. */
int kspace_gpu_diff_forward(kspace_ctx *ctx, double Time, double BoxSize, const void *grid_in, void *grid_out,
                            int pmgrid, double *pnu_out, int store_intervals);
/* The count of successful diff_forward calls on the context (read it right after a
 * forward and hand it to that forward's diff_backward). */
int kspace_gpu_diff_generation(kspace_ctx *ctx, long long *generation);
/* Adjoint of the last diff_forward: from dL/dgrid_out and dL/dP_nu, produce dL/dgrid_in,
 * dL/d(history)[nk][ia] (device) and dL/dm per mass state (host, 3).  recompute = 1
 * re-runs each QAG instead of reading the stored subdivision.  generation: the
 * forward's (kspace_gpu_diff_generation); KSPACE_ERR_ORDER if another forward ran on
 * the context since, whose state the adjoint would otherwise read. */
int kspace_gpu_diff_backward(kspace_ctx *ctx, const void *gbar_out, const void *grid_in, const double *pnu_bar,
                             void *gbar_in, double *Dbar, double *mbar, int recompute, long long generation);

/* ---- batches of independent instances ----
 * No counterpart in the reference, which holds one integrator per process.  A batch
 * advances many contexts (each a complete integrator: its own cosmology, masses,
 * transfer table, history length and k bins) with one captured sequence of kernels;
 * each instance's delta_nu is the one kspace_gpu_get_delta_nu_update would return.
 * Every context must be on the batch's device with its table, transfer function and
 * H(a) set; while it belongs to a batch it is driven only through the batch.
 * Per-instance bin arrays are concatenated ("pools"): instance i owns entries
 * [offset[i], offset[i+1]). */
typedef struct kspace_batch kspace_batch;
int kspace_gpu_batch_create(kspace_batch **batch, kspace_ctx *const *ctxs, int M);
int kspace_gpu_batch_destroy(kspace_batch *batch);
/* Bind instance `inst` to a device grid (complex64, pmgrid x pmgrid x (pmgrid/2+1),
 * fixed address): every step bins it into the instance's delta_cdm (nrbins = the
 * context's nk_alloc, as add_nu_power_to_rhogrid) and corrects it in place afterwards.
 * Must precede kspace_gpu_batch_init. */
int kspace_gpu_batch_bind_grid(kspace_batch *batch, int inst, void *grid, int pmgrid, double BoxSize);
/* First call of every instance (delta_tot_init, delta_tot_table.c:79-149) at a[i]:
 * nk[i] bins with keff (physical k) and sqrt(P_cdm) in host arrays holding the
 * unbound instances one after another.  Bound instances take nk, keff and delta_cdm
 * from their grid and have no entries there (their nk[i] is ignored).  Fixes the
 * layout of the step pools (kspace_gpu_batch_layout), where bound instances do own
 * entries (their delta_nu). */
int kspace_gpu_batch_init(kspace_batch *batch, const double *a, const int *nk, const double *keff,
                          const double *dcdm);
/* nk[M] and offset[M+1] of the pools */
int kspace_gpu_batch_layout(kspace_batch *batch, int *nk, int *offset);
/* One step of every instance at a[i] (get_delta_nu_update, delta_tot_table.c:193-250):
 * dcdm = sqrt(P_cdm) pool (host or device; NULL when every instance is bound to a
 * grid), dnu = delta_nu pool out (host or device; NULL to keep it on the device).
 * Returns the first instance's non-zero status (kspace_gpu_batch_status has all). */
int kspace_gpu_batch_step(kspace_batch *batch, const double *a, const double *dcdm, double *dnu);
/* per-instance status of the last step */
int kspace_gpu_batch_status(kspace_batch *batch, int *status);
/* warps per block (1..4) and resident blocks per SM of the integral kernel; use_graph
 * = 0 launches the kernels one by one instead of replaying the captured graph */
int kspace_gpu_batch_set_tuning(kspace_batch *batch, int warps_per_block, int blocks_per_sm, int use_graph);
/* Time each (warps per block, blocks per SM) candidate on `reps` dry steps at a[i]
 * (nothing committed, no state changed) and keep the fastest.  best[2] and its time
 * (ms) are returned. */
int kspace_gpu_batch_autotune(kspace_batch *batch, const double *a, const double *dcdm, int reps, int *best,
                              float *best_ms);
/* device time (ms) of the last step's kernels */
int kspace_gpu_batch_last_ms(kspace_batch *batch, float *ms);

/* ---- allocation-free binning ----
 * No counterpart in the reference.  The per-bin sums of total_powerspectrum's binning
 * pass (powerspectrum.c:56-89) without a context and without allocating any memory,
 * for hosts that cannot let a library allocate (a host that owns all device memory in
 * its own pool, a PM code with no device memory to spare).  bin_sums[nrbins + 1] (host
 * or device) receives sum w |F|^2 W^4 per bin, not normalised, and |F(0)|^2 last;
 * divide by |F(0)|^2 and the mode counts for the power.  grid: device memory.  Limits:
 * nrbins <= 4096, dims <= 4096 (KSPACE_ERR_ARG beyond).  Scratch is one fixed device
 * array shared by all calls: overlapping calls race.  The first call on a device looks
 * up the scratch address.  cuda_stream: a
 * cudaStream_t (NULL = the default stream); returns after the sums are in bin_sums. */
int kspace_gpu_bin_power_noalloc(int dims, const void *grid, int nrbins, int startslab, int nslab,
                                 double *bin_sums, void *cuda_stream);

/* ---- diagnostics ---- */
/* last call: nk, log k, ratio and norm of the correction (arrays of nk_alloc) */
int kspace_gpu_last_correction(kspace_ctx *ctx, int *nk, double *logk, double *ratio, double *norm, double *dcdm,
                               double *keff);
/* device times (ms) of the last add_nu_power_to_rhogrid: [0] binning kernel,
 * [1] integrator, [2] correction kernel, [3] whole call; enable with on=1 */
int kspace_gpu_set_profiling(kspace_ctx *ctx, int on);
int kspace_gpu_stage_times(kspace_ctx *ctx, float *ms4);
/* QAG statistics of the last integrator call: max and total intervals */
int kspace_gpu_qag_stats(kspace_ctx *ctx, int *max_intervals, long long *total_intervals);
/* how many kernels this library has launched on the context (monotonic) */
long long kspace_gpu_launch_count(kspace_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
