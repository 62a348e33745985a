/* kspace_neutrinos_dropin.h -- the kspace-neutrinos public interface, unchanged, for
 * host N-body codes (Gadget-style PM loops) that switch to the GB300 library.
 *
 * These are the reference's own entry points with the reference's signatures; they are
 * implemented by kspace-neutrinos_gb300/dropin/kspace_dropin.c (compile that file into
 * the host program with the host's <mpi.h> and FFTW2 headers, together with
 * dropin/kspace_delta_tot_table.c, and link libkspace_gb300.so).  Like the reference,
 * the host supplies hubble_function(), terminate(), message() (gadget_defines.h:11,24-25).
 */
#ifndef KSPACE_NEUTRINOS_DROPIN_H
#define KSPACE_NEUTRINOS_DROPIN_H
#include <stddef.h>
#include <mpi.h>
#ifdef NOTYPEPREFIX_FFTW
#include <fftw.h>
#else
#ifdef DOUBLEPRECISION_FFTW
#include <dfftw.h>
#else
#include <sfftw.h>
#endif
#endif

#include "kspace_delta_tot_table.h" /* _delta_pow, get_dnudcdm_powerspec, free_d_pow and the integrator API */

#ifdef __cplusplus
extern "C" {
#endif

/* interface_common.h:12-30 */
extern struct __kspace_params {
    char KspaceTransferFunction[500];
    double TimeTransfer;
    double InputSpectrum_UnitLength_in_cm;
    double MNu[NUSPECIES];
    int hybrid_neutrinos_on;
    double vcrit;
    double nu_crit_time;
} kspace_params;

/* ---- interface_common.h ---- */
double OmegaNu(double a);                                   /* :36 */
double OmegaNu_nopart(double a);                            /* :43 */
void InitOmegaNu(const double HubbleParam, const double tcmb0, MPI_Comm MYMPI_COMM_WORLD); /* :45 */
void allocate_kspace_memory(const int nk_in, const int ThisTask, const double BoxSize, const double UnitTime_in_s,
                            const double UnitLength_in_cm, const double Omega0, char *snapdir, const double TimeMax,
                            MPI_Comm MYMPI_COMM_WORLD);     /* :65 */
_delta_pow compute_neutrino_power_from_cdm(const double Time, const double keff_in[], const double P_cdm[],
                                           const long int Nmodes[], const int nk_in,
                                           MPI_Comm MYMPI_COMM_WORLD); /* :79 */
void save_nu_state(char *savedir);                          /* :85 */
void get_nu_state(double **scalefact, double **delta_tot, size_t *nk, size_t *ia); /* :96 */
void set_nu_state(double *scalefact, double *delta_tot, const size_t nk, const size_t ia,
                  MPI_Comm MYMPI_COMM_WORLD);               /* :107 */
int save_neutrino_power(const double Time, const int snapnum, const char *OutputDir); /* :116 */
int particle_nu_active(double a);                           /* :120 */

/* ---- interface_gadget.h ---- */
void add_nu_power_to_rhogrid(const double Time, const double BoxSize, fftw_complex *fft_of_rhogrid,
                             const int pmgrid, int slabstart_y, int nslab_y, MPI_Comm MYMPI_COMM_WORLD); /* :38 */
int set_kspace_vars(char tag[][50], void *addr[], int id[], int nt);     /* :46 */
void compute_total_power_spectrum(const double Time, const double BoxSize, fftw_complex *fft_of_rhogrid,
                                  const int pmgrid, int slabstart_y, int nslab_y, MPI_Comm MYMPI_COMM_WORLD); /* :49 */
int save_total_power(const double Time, const int snapnum, const char *OutputDir); /* :57 */

/* ---- powerspectrum.h ---- */
int total_powerspectrum(const int dims, fftw_complex *outfield, const int nrbins, const int startslab,
                        const int nslab, double *power, long long int *count, double *keffs,
                        const MPI_Comm MYMPI_COMM_WORLD);   /* powerspectrum.h:30 */

#ifdef __cplusplus
}
#endif
#endif
