/* A minimal PM-loop host (C) that drives the kspace-neutrinos interface exactly as the
 * Gadget-2 hooks do (gadget-2/0002-...patch: begrun -> InitOmegaNu,
 * allocate_kspace_memory; pmforce_periodic -> add_nu_power_to_rhogrid; snapshots ->
 * save_nu_state, save_neutrino_power, save_total_power), linked against the drop-in
 * layer and libkspace_gb300.so.  Test infrastructure.
 *
 * usage: pm_harness transfer_file state_file grid_in grid_out outdir N nbins L TimeMax a1 [a2 ...]
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "kspace_neutrinos_dropin.h"

#define HUBBLE 3.24077929e-18
#define GRAVITY 6.67408e-8
#define LIGHT 2.99792458e10
#define STEFAN_BOLTZMANN 5.670373e-5

static double Omega0 = 0.3, OmegaLambda = 0.7, HubbleParam = 0.7, UnitTime_in_s;
int (*kspace_shim_allreduce_hook)(void *buf, int count, MPI_Datatype dt) = NULL;

/* The host's hubble function (gadget-2/0003-...patch:38-52 with KSPACE_NEUTRINOS_2 and
 * INCLUDE_RADIATION) */
double hubble_function(double a)
{
    const double OMEGAG = 4 * STEFAN_BOLTZMANN * 8 * M_PI * GRAVITY / (3 * LIGHT * LIGHT * LIGHT * HUBBLE * HUBBLE) *
                          pow(2.7255, 4) / HubbleParam / HubbleParam;
    double omega_tot = Omega0 / pow(a, 3) + OmegaLambda + (1. - OmegaLambda - Omega0) / (a * a);
    omega_tot += OmegaNu(a) - OmegaNu(1) / pow(a, 3);
    omega_tot += OMEGAG / pow(a, 4);
    return HUBBLE * UnitTime_in_s * sqrt(omega_tot);
}

void terminate(int ierr, const char *fmt, ...)
{
    va_list va;
    va_start(va, fmt);
    fprintf(stderr, "terminate(%d): ", ierr);
    vfprintf(stderr, fmt, va);
    va_end(va);
    exit(ierr % 256 ? ierr % 256 : 1);
}

void message(int ierr, const char *fmt, ...)
{
    (void)ierr;
    va_list va;
    va_start(va, fmt);
    vprintf(fmt, va);
    va_end(va);
}

int main(int argc, char **argv)
{
    if (argc < 11) {
        fprintf(stderr, "usage: %s transfer state grid_in grid_out outdir N nbins L TimeMax a...\n", argv[0]);
        return 2;
    }
    const char *transfer = argv[1], *state = argv[2], *gin = argv[3], *gout = argv[4], *outdir = argv[5];
    const int N = atoi(argv[6]), nbins = atoi(argv[7]);
    const double L = atof(argv[8]), TimeMax = atof(argv[9]);
    const double UnitLength_in_cm = 3.085678e24;
    UnitTime_in_s = UnitLength_in_cm / 1e5;
    /* parameters as read by set_kspace_vars */
    char tag[20][50];
    void *addr[20];
    int id[20];
    int nt = set_kspace_vars(tag, addr, id, 0);
    if (nt != 9) return 3;
    strcpy(kspace_params.KspaceTransferFunction, transfer);
    kspace_params.TimeTransfer = 0.01;
    kspace_params.InputSpectrum_UnitLength_in_cm = UnitLength_in_cm;
    kspace_params.MNu[0] = kspace_params.MNu[1] = kspace_params.MNu[2] = 0.1;
    kspace_params.hybrid_neutrinos_on = 0;
    /* begrun */
    InitOmegaNu(HubbleParam, 2.7255, MPI_COMM_WORLD);
    /* Gadget's Omega0 includes the neutrinos; hubble_function above subtracts OmegaNu(1) */
    allocate_kspace_memory(nbins, 0, L, UnitTime_in_s, UnitLength_in_cm, Omega0, (char *)state, TimeMax, MPI_COMM_WORLD);
    const size_t nmodes = (size_t)N * N * (N / 2 + 1);
    fftw_complex *grid = (fftw_complex *)malloc(nmodes * sizeof(fftw_complex));
    FILE *f = fopen(gin, "rb");
    if (!f || fread(grid, sizeof(fftw_complex), nmodes, f) != nmodes) return 4;
    fclose(f);
    /* PM steps */
    for (int i = 10; i < argc; i++) {
        const double a = atof(argv[i]);
        add_nu_power_to_rhogrid(a, L, grid, N, 0, N, MPI_COMM_WORLD);
    }
    f = fopen(gout, "wb");
    fwrite(grid, sizeof(fftw_complex), nmodes, f);
    fclose(f);
    /* snapshot outputs */
    char buf[1000];
    snprintf(buf, sizeof(buf), "%s/delta_tot_nu.txt", outdir);
    save_nu_state(buf);
    const double alast = atof(argv[argc - 1]);
    if (save_neutrino_power(alast, 1, outdir) != 0) return 5;
    if (save_total_power(alast, 1, outdir) != 0) return 6;
    size_t nk, ia;
    double *sf, *dt;
    get_nu_state(&sf, &dt, &nk, &ia);
    printf("state nk=%zu ia=%zu particle_nu_active=%d OmegaNu(1)=%.17g\n", nk, ia, particle_nu_active(alast),
           OmegaNu(1));
    free(sf);
    free(dt);
    free(grid);
    return 0;
}
