/* kspace_delta_tot_table.h -- the integrator-level interface of kspace-neutrinos,
 * unchanged, for host codes that drive the delta_tot table directly (MP-Gadget style)
 * instead of through add_nu_power_to_rhogrid.
 *
 * These are the reference's own types and entry points with the reference's signatures:
 *   delta_tot_table.h:17-155  the integrator state and its functions
 *   delta_pow.h:10-42         the delta_nu/delta_cdm interpolation table
 *   omega_nu_single.h:21-131  the neutrino background (_omega_nu, hybrid neutrinos)
 *   transfer_init.h:12-31     the initial transfer table
 * implemented by kspace-neutrinos_gb300/dropin/kspace_delta_tot_table.c on the C ABI
 * of libkspace_gb300.so (compile that file into the host program and link the library).
 *
 * The structures keep the reference's fields, so host code that reads or edits them
 * (d_tot.ia, d_tot.delta_tot[k][i], omnu.hybnu ...) works as before.  Each has one
 * trailing field the reference lacks, `gpu`, that ties it to its GPU context; the host
 * must not touch it.  The host-visible fields are the truth at every call: a call first
 * sends what the host changed to the GPU and, when it returns, the fields hold the
 * GPU's results.  Every number is computed on the GPU; errors go to the host's
 * terminate() with the reference's codes.
 *
 * Not provided: rho_nu_init and rho_nu (omega_nu_single.h:37,45), the internal
 * Fermi-Dirac table builders; _rho_nu_single's loga/rhonu arrays are NULL (the tables
 * live on the GPU).  fslength uses the H(a) of the most recently allocated delta_tot
 * table (the reference calls the host's hubble_function; here that function is matched
 * once against the GPU's model when the table is first used).
 */
#ifndef KSPACE_DELTA_TOT_TABLE_H
#define KSPACE_DELTA_TOT_TABLE_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef NUSPECIES
#define NUSPECIES 3
#endif

struct kspace_ctx;
struct kspace_dtt_priv;

/* ---- omega_nu_single.h ---- */
/* :21-29 */
struct _rho_nu_single {
    double *loga;
    double *rhonu;
    void *interp;
    void *acc;
    double mnu;
};
typedef struct _rho_nu_single _rho_nu_single;

/* :51-64 */
struct _hybrid_nu {
    int enabled;
    double nufrac_low[NUSPECIES];
    double nu_crit_time;
    double vcrit;
};
typedef struct _hybrid_nu _hybrid_nu;

/* :94-108 */
struct _omega_nu {
    _rho_nu_single *RhoNuTab[NUSPECIES];
    int nu_degeneracies[NUSPECIES];
    double rhocrit;
    double kBtnu;
    double tcmb0;
    _hybrid_nu hybnu;
    /* not in the reference: the GPU context holding the Fermi-Dirac tables */
    struct kspace_omnu_priv *gpu;
};
typedef struct _omega_nu _omega_nu;

void init_omega_nu(_omega_nu *const omnu, const double MNu[], const double a0, const double HubbleParam,
                   const double tcmb0);                                               /* :116 */
double get_omega_nu(const _omega_nu *const omnu, const double a);                      /* :119 */
double get_omega_nu_nopart(const _omega_nu *const omnu, const double a);               /* :122 */
double get_omegag(const _omega_nu *const omnu, const double a);                        /* :125 */
double omega_nu_single(const _omega_nu *const rho_nu_tab, const double a, const int i); /* :131 */
void init_hybrid_nu(_hybrid_nu *const hybnu, const double mnu[], const double vcrit, const double light,
                    const double nu_crit_time, const double kBtnu);                    /* :75 */
double particle_nu_fraction(const _hybrid_nu *const hybnu, const double a, int i);     /* :84 */
double nufrac_low(const double qc);                                                    /* :87 */

/* ---- transfer_init.h:12-31 ---- */
struct _transfer_init_table {
    int NPowerTable;
    double *logk;
    double *T_nu;
};
typedef struct _transfer_init_table _transfer_init_table;

void allocate_transfer_init_table(_transfer_init_table *t_init, const double BoxSize, const double UnitLength_in_cm,
                                  const double InputSpectrum_UnitLength_in_cm,
                                  const char *KspaceTransferFunction); /* :28 */
void free_transfer_init_table(_transfer_init_table *t_init);          /* :31 */

/* ---- delta_tot_table.h ---- */
/* :17-57 */
struct _delta_tot_table {
    int nk;
    int nk_allocated;
    int namax;
    int ia;
    int ThisTask;
    double delta_nu_prefac;
    int delta_tot_init_done;
    int debug;
    double **delta_tot;
    double *scalefact;
    double *delta_nu_init;
    double *delta_nu_last;
    double *wavenum;
    const _omega_nu *omnu;
    double Omeganonu;
    double light;
    double TimeTransfer;
    /* not in the reference: the GPU context and the last state exchanged with it */
    struct kspace_dtt_priv *gpu;
};
typedef struct _delta_tot_table _delta_tot_table;

void allocate_delta_tot_table(_delta_tot_table *d_tot, const int nk_in, const double TimeTransfer,
                              const double TimeMax, const double Omega0, const _omega_nu *const omnu,
                              const double UnitTime_in_s, const double UnitLength_in_cm, int debug); /* :70 */
void free_delta_tot_table(_delta_tot_table *d_tot);                                            /* :73 */
void delta_tot_init(_delta_tot_table *const d_tot, const int nk_in, const double wavenum[],
                    const double delta_cdm_curr[], const _transfer_init_table *const t_init,
                    const double Time);                                                        /* :85 */
void update_delta_tot(_delta_tot_table *const d_tot, const double a, const double delta_cdm_curr[],
                      const double delta_nu_curr[], const int overwrite);                      /* :90 */
void get_delta_nu_update(_delta_tot_table *const d_tot, const double a, const int nk_in, const double keff[],
                         const double P_cdm_curr[], double delta_nu_curr[],
                         _transfer_init_table *transfer_init);                                 /* :104 */
void get_delta_nu(const _delta_tot_table *const d_tot, const double a, const double wavenum[],
                  double delta_nu_curr[], const double mnu);                                   /* :113 */
void get_delta_nu_combined(const _delta_tot_table *const d_tot, const double a, const double wavenum[],
                           double delta_nu_curr[]);                                            /* :117 */
void save_delta_tot(const _delta_tot_table *const d_tot, const int iia, char *savedir);        /* :120 */
void save_all_nu_state(const _delta_tot_table *const d_tot, char *savedir);                    /* :123 */
int save_nu_power(const _delta_tot_table *const d_tot, const double Time, const int snapnum,
                  const char *OutputDir);                                                      /* :131 */
void read_all_nu_state(_delta_tot_table *const d_tot, char *savedir);                          /* :135 */
double specialJ(const double x, const double vcmnubylight, const double nufrac_low);           /* :138 */
double fslength(const double logai, const double logaf, const double light);                   /* :149 */
double get_delta_tot(const double delta_nu_curr, const double delta_cdm_curr, const double OmegaNua3,
                     const double Omeganonu, const double Omeganu1, const double partnu);      /* :155 */

/* ---- delta_pow.h:10-42 ----
 * The GSL interpolation objects of the reference are not needed (get_dnudcdm_powerspec
 * interpolates linearly in log k, as the reference does); spline and acc stay NULL. */
struct _delta_pow {
    double *logkk;
    double *delta_ratio;
    void *spline;
    void *acc;
    int nbins;
    double norm;
};
typedef struct _delta_pow _delta_pow;

void init_delta_pow(_delta_pow *d_pow, double logkk[], double delta_ratio[], int nbins, double norm); /* :30 */
double get_dnudcdm_powerspec(_delta_pow *d_pow, double kk);                                         /* :39 */
void free_d_pow(_delta_pow *d_pow);                                                                 /* :41 */

/* Host services, as in gadget_defines.h:11,24-25 (defined by the host). */
double hubble_function(double a);
void terminate(int ierr, const char *fmt, ...);
void message(int ierr, const char *fmt, ...);

#ifdef __cplusplus
}
#endif
#endif
