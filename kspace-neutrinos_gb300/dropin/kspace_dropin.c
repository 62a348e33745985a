/* kspace_dropin.c -- the kspace-neutrinos interface (interface_common.h,
 * interface_gadget.h, powerspectrum.h, delta_pow.h) implemented on the C ABI of
 * libkspace_gb300.so.  Compile into the host program with its <mpi.h> and FFTW2 headers:
 *
 *   cc -I<repo>/include -c kspace_dropin.c && link with -L... -lkspace_gb300
 *
 * The library keeps the integrator on the GPU; this file only moves the reference's
 * process-global state (kspace_params, the context) and its MPI collectives
 * (broadcasts at initialisation, the per-bin allreduce of the binning pass).  Errors
 * are passed to the host's terminate() with the reference's codes.  The GPU used is
 * the one named by KSPACE_GPU_DEVICE, else rank % (number of visible GPUs).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "kspace_neutrinos_dropin.h"
#include "kspace_gpu.h"
#include "kspace_hubble_match.h"

#define KSP_LIGHTCGS 2.99792458e10
/* gadget_defines.h:47-49 (parameter types of the P-Gadget3 reader) */
#define KSP_REAL 1
#define KSP_STRING 2
#define KSP_INT 3

struct __kspace_params kspace_params;

static kspace_ctx *g_ctx = NULL;
static MPI_Comm g_comm;
static int g_rank = 0;
static double g_h = 0.7, g_tcmb0 = 2.7255;
static double *g_dpow_buf = NULL; /* logk | ratio of the last compute_neutrino_power_from_cdm */
static int g_dpow_cap = 0;

static void check(int st, const char *where)
{
    if (st != KSPACE_OK)
        terminate(st, "%s: %s\n", where, kspace_gpu_error_string(st));
}

static int allreduce_sum(double *buf, int count, void *user)
{
    MPI_Comm comm = *(MPI_Comm *)user;
    return MPI_Allreduce(MPI_IN_PLACE, buf, count, MPI_DOUBLE, MPI_SUM, comm) == MPI_SUCCESS ? 0 : 1;
}

static int pick_device(void)
{
    const char *e = getenv("KSPACE_GPU_DEVICE");
    if (e)
        return atoi(e);
    const char *n = getenv("KSPACE_GPU_NDEV");
    const int ndev = n ? atoi(n) : 1;
    return ndev > 0 ? g_rank % ndev : 0;
}

/* interface_common.c:29-39 */
double OmegaNu(double a)
{
    double o = 0;
    check(kspace_gpu_omega_nu(g_ctx, a, &o, NULL), "OmegaNu");
    return o;
}

double OmegaNu_nopart(double a)
{
    double o = 0;
    check(kspace_gpu_omega_nu(g_ctx, a, NULL, &o), "OmegaNu_nopart");
    return o;
}

/* interface_common.c:183-188 */
void InitOmegaNu(const double HubbleParam, const double tcmb0, MPI_Comm comm)
{
    MPI_Bcast(&kspace_params, sizeof(kspace_params), MPI_BYTE, 0, comm);
    MPI_Comm_rank(comm, &g_rank);
    g_comm = comm;
    g_h = HubbleParam;
    g_tcmb0 = tcmb0;
    if (!g_ctx)
        check(kspace_gpu_create(&g_ctx, pick_device()), "kspace_gpu_create");
    check(kspace_gpu_init_omega_nu(g_ctx, kspace_params.MNu, kspace_params.TimeTransfer, HubbleParam, tcmb0),
          "InitOmegaNu");
}

/* transfer_init.c:9-83 on rank 0, then broadcast (interface_common.c:54-63) */
static void load_transfer(double BoxSize, double UnitLength_in_cm, MPI_Comm comm)
{
    int n = 0;
    double *buf = NULL;
    if (g_rank == 0) {
        const double scale = kspace_params.InputSpectrum_UnitLength_in_cm / UnitLength_in_cm;
        const double kmin = M_PI / BoxSize * scale;
        FILE *fd = fopen(kspace_params.KspaceTransferFunction, "r");
        if (!fd)
            terminate(2019, "Can't read input transfer function in file '%s'\n", kspace_params.KspaceTransferFunction);
        char line[1000];
        int cap = 1024;
        buf = (double *)malloc(2 * cap * sizeof(double));
        while (fgets(line, sizeof(line), fd)) {
            double k, Tc, Tb, Tg, Tr, Tnu, Ttot, Tnonu;
            if (line[0] == '#')
                continue;
            if (sscanf(line, " %lg %lg %lg %lg %lg %lg %lg %lg", &k, &Tc, &Tb, &Tg, &Tr, &Tnu, &Ttot, &Tnonu) != 8)
                break;
            if (k > kmin) {
                if (n == cap) {
                    cap *= 2;
                    buf = (double *)realloc(buf, 2 * cap * sizeof(double));
                }
                buf[2 * n] = log(k / scale);
                buf[2 * n + 1] = Tnu / Tnonu;
                n++;
            }
        }
        fclose(fd);
    }
    MPI_Bcast(&n, 1, MPI_INT, 0, comm);
    if (g_rank != 0)
        buf = (double *)malloc(2 * (n > 0 ? n : 1) * sizeof(double));
    MPI_Bcast(buf, 2 * n, MPI_DOUBLE, 0, comm);
    double *lk = (double *)malloc((n > 0 ? n : 1) * sizeof(double));
    double *tt = (double *)malloc((n > 0 ? n : 1) * sizeof(double));
    for (int i = 0; i < n; i++) {
        lk[i] = buf[2 * i];
        tt[i] = buf[2 * i + 1];
    }
    check(kspace_gpu_set_transfer(g_ctx, lk, tt, n), "allocate_transfer_init_table");
    free(lk);
    free(tt);
    free(buf);
}

/* The host owns H(a): identify it with the device model (kspace_hubble_match.h). */
static void match_hubble(double Omega0, double UnitTime_in_s, double TimeMax)
{
    double err = 0;
    if (kspace_match_hubble(g_ctx, Omega0, UnitTime_in_s, kspace_params.TimeTransfer, TimeMax, &err) != KSPACE_OK)
        terminate(10004, "hubble_function is not of the form H0 sqrt(Om/a^3 + Ok/a^2 + OL + Onu(a) [+ Og/a^4]) "
                         "(best relative difference %g)\n", err);
}

/* interface_common.c:77-102 */
void allocate_kspace_memory(const int nk_in, const int ThisTask, const double BoxSize, const double UnitTime_in_s,
                            const double UnitLength_in_cm, const double Omega0, char *snapdir, const double TimeMax,
                            MPI_Comm comm)
{
    g_rank = ThisTask;
    g_comm = comm;
    if (kspace_params.hybrid_neutrinos_on)
        check(kspace_gpu_init_hybrid_nu(g_ctx, kspace_params.vcrit, KSP_LIGHTCGS / 1e5, kspace_params.nu_crit_time),
              "init_hybrid_nu");
    match_hubble(Omega0, UnitTime_in_s, TimeMax);
    check(kspace_gpu_alloc_table(g_ctx, nk_in, kspace_params.TimeTransfer, TimeMax, Omega0, UnitTime_in_s,
                                 UnitLength_in_cm), "allocate_delta_tot_table");
    load_transfer(BoxSize, UnitLength_in_cm, comm);
    check(kspace_gpu_set_allreduce(g_ctx, allreduce_sum, &g_comm), "set_allreduce");
    /* read_all_nu_state on rank 0, then broadcast (interface_common.c:93-97) */
    size_t nk = 0, ia = 0;
    if (ThisTask == 0 && snapdir != NULL) {
        check(kspace_gpu_read_nu_state(g_ctx, snapdir), "read_all_nu_state");
        kspace_gpu_get_nu_state(g_ctx, NULL, NULL, &nk, &ia);
    }
    unsigned long long dims[2] = {nk, ia};
    MPI_Bcast(dims, 2 * sizeof(unsigned long long), MPI_BYTE, 0, comm);
    if (dims[1] > 0) {
        double *sf = (double *)malloc(dims[1] * sizeof(double));
        double *dt = (double *)malloc(dims[0] * dims[1] * sizeof(double));
        if (ThisTask == 0)
            kspace_gpu_get_nu_state(g_ctx, sf, dt, &nk, &ia);
        MPI_Bcast(sf, (int)dims[1], MPI_DOUBLE, 0, comm);
        MPI_Bcast(dt, (int)(dims[0] * dims[1]), MPI_DOUBLE, 0, comm);
        if (ThisTask != 0)
            check(kspace_gpu_set_nu_state(g_ctx, sf, dt, dims[0], dims[1]), "set_nu_state");
        free(sf);
        free(dt);
    }
}

/* interface_gadget.c:158-194 */
void add_nu_power_to_rhogrid(const double Time, const double BoxSize, fftw_complex *fft_of_rhogrid, const int pmgrid,
                             int slabstart_y, int nslab_y, MPI_Comm comm)
{
    g_comm = comm;
    int nranks = 1;
    MPI_Comm_size(comm, &nranks);
    check(kspace_gpu_set_allreduce(g_ctx, nranks > 1 ? allreduce_sum : NULL, &g_comm), "set_allreduce");
    check(kspace_gpu_add_nu_power_to_rhogrid(g_ctx, Time, BoxSize, fft_of_rhogrid, pmgrid, slabstart_y, nslab_y),
          "add_nu_power_to_rhogrid");
    MPI_Barrier(comm);
    message(0, "Done adding neutrinos to grid on all processors\n");
}

/* interface_gadget.c:114-144 */
void compute_total_power_spectrum(const double Time, const double BoxSize, fftw_complex *fft_of_rhogrid,
                                  const int pmgrid, int slabstart_y, int nslab_y, MPI_Comm comm)
{
    g_comm = comm;
    int nranks = 1;
    MPI_Comm_size(comm, &nranks);
    MPI_Comm_rank(comm, &g_rank);
    if (!g_ctx) /* a run without the neutrino module (gadget-2 patch 0004) */
        check(kspace_gpu_create(&g_ctx, pick_device()), "kspace_gpu_create");
    check(kspace_gpu_set_allreduce(g_ctx, nranks > 1 ? allreduce_sum : NULL, &g_comm), "set_allreduce");
    check(kspace_gpu_compute_total_power_spectrum(g_ctx, Time, BoxSize, fft_of_rhogrid, pmgrid, slabstart_y,
                                                  nslab_y), "compute_total_power_spectrum");
}

/* interface_gadget.c:196-224 */
int save_total_power(const double Time, const int snapnum, const char *OutputDir)
{
    if (!g_ctx)
        terminate(10003, "save_total_power before any power spectrum was computed\n");
    return kspace_gpu_save_total_power(g_ctx, Time, snapnum, OutputDir);
}

/* powerspectrum.c:33-117 */
int total_powerspectrum(const int dims, fftw_complex *outfield, const int nrbins, const int startslab,
                        const int nslab, double *power, long long int *count, double *keffs, const MPI_Comm comm)
{
    g_comm = comm;
    int nranks = 1, nk = 0;
    MPI_Comm_size(comm, &nranks);
    check(kspace_gpu_set_allreduce(g_ctx, nranks > 1 ? allreduce_sum : NULL, &g_comm), "set_allreduce");
    check(kspace_gpu_total_powerspectrum(g_ctx, dims, outfield, nrbins, startslab, nslab, power, count, keffs, &nk),
          "total_powerspectrum");
    return nk;
}

/* interface_common.c:106-123 */
_delta_pow compute_neutrino_power_from_cdm(const double Time, const double keff_in[], const double P_cdm[],
                                           const long int Nmodes[], const int nk_in, MPI_Comm comm)
{
    (void)comm;
    _delta_pow d;
    memset(&d, 0, sizeof(d));
    if (g_dpow_cap < nk_in) {
        free(g_dpow_buf);
        g_dpow_buf = (double *)malloc(2 * (size_t)nk_in * sizeof(double));
        g_dpow_cap = nk_in;
    }
    d.logkk = g_dpow_buf;
    d.delta_ratio = g_dpow_buf + nk_in;
    check(kspace_gpu_compute_neutrino_power_from_cdm(g_ctx, Time, keff_in, P_cdm, Nmodes, nk_in, d.logkk,
                                                     d.delta_ratio, &d.norm, &d.nbins),
          "compute_neutrino_power_from_cdm");
    return d;
}

/* interface_common.c:41-52,150-197 */
void save_nu_state(char *savedir)
{
    if (g_rank == 0)
        check(kspace_gpu_save_nu_state(g_ctx, savedir), "save_all_nu_state");
}

int save_neutrino_power(const double Time, const int snapnum, const char *OutputDir)
{
    if (g_rank != 0)
        return 0;
    return kspace_gpu_save_nu_power(g_ctx, Time, snapnum, OutputDir);
}

void get_nu_state(double **scalefact, double **delta_tot, size_t *nk, size_t *ia)
{
    check(kspace_gpu_get_nu_state(g_ctx, NULL, NULL, nk, ia), "get_nu_state");
    *scalefact = (double *)malloc((*ia > 0 ? *ia : 1) * sizeof(double));
    *delta_tot = (double *)malloc((*nk * *ia > 0 ? *nk * *ia : 1) * sizeof(double));
    check(kspace_gpu_get_nu_state(g_ctx, *scalefact, *delta_tot, nk, ia), "get_nu_state");
}

void set_nu_state(double *scalefact, double *delta_tot, const size_t nk, const size_t ia, MPI_Comm comm)
{
    (void)comm; /* every rank receives the same table, as the reference's broadcast ensures */
    check(kspace_gpu_set_nu_state(g_ctx, scalefact, delta_tot, nk, ia), "set_nu_state");
}

int particle_nu_active(double a)
{
    int act = 0;
    check(kspace_gpu_particle_nu_active(g_ctx, a, &act), "particle_nu_active");
    return act;
}

/* interface_gadget.c:25-58 (P-Gadget3 parameter reader) */
int set_kspace_vars(char tag[][50], void *addr[], int id[], int nt)
{
    strcpy(tag[nt], "KspaceTransferFunction");
    addr[nt] = kspace_params.KspaceTransferFunction;
    id[nt++] = KSP_STRING;
    strcpy(tag[nt], "TimeTransfer");
    addr[nt] = &kspace_params.TimeTransfer;
    id[nt++] = KSP_REAL;
    strcpy(tag[nt], "InputSpectrum_UnitLength_in_cm");
    addr[nt] = &kspace_params.InputSpectrum_UnitLength_in_cm;
    id[nt++] = KSP_REAL;
    strcpy(tag[nt], "MNue");
    addr[nt] = &(kspace_params.MNu[0]);
    id[nt++] = KSP_REAL;
    strcpy(tag[nt], "MNum");
    addr[nt] = &(kspace_params.MNu[1]);
    id[nt++] = KSP_REAL;
    strcpy(tag[nt], "MNut");
    addr[nt] = &(kspace_params.MNu[2]);
    id[nt++] = KSP_REAL;
    strcpy(tag[nt], "HybridNeutrinosOn");
    addr[nt] = &(kspace_params.hybrid_neutrinos_on);
    id[nt++] = KSP_INT;
    strcpy(tag[nt], "Vcrit");
    addr[nt] = &(kspace_params.vcrit);
    id[nt++] = KSP_REAL;
    strcpy(tag[nt], "NuPartTime");
    addr[nt] = &(kspace_params.nu_crit_time);
    id[nt++] = KSP_REAL;
    return nt;
}
