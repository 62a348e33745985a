/* A C host that drives the integrator-level interface (kspace_delta_tot_table.h:
 * delta_tot_table.h, delta_pow.h, omega_nu_single.h, transfer_init.h) through the
 * sequences of the reference's own test suite (delta_tot_table_test.c), linked against
 * dropin/kspace_delta_tot_table.c and libkspace_gb300.so.  Test infrastructure: the
 * pytest wrapper compares the values it prints with the reference's outputs on the
 * same inputs (tests/golden/ref_testdata.npz).
 *
 * usage: dtt_harness indir n t_n outdir
 *   indir: keff.bin, dcdm.bin (n doubles: k, not log k, and sqrt(P_cdm)), tlogk.bin,
 *          tT.bin (t_n doubles: the transfer table), delta_tot_nu.txt (a saved state)
 * Prints one line per result: name count values...  (%.17g), and "check name 0|1" for
 * the assertions of the reference tests.
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
#include "kspace_delta_tot_table.h"

#define T_CMB0 2.7255
#define HUBBLE 3.24077929e-18
#define BOLEVK 8.61734e-5
#define TNUCMB (pow(4 / 11., 1 / 3.) * 1.00328)

/* delta_tot_table_test.c:20-45: the host's hubble function with global state */
static _omega_nu *m_omnu;
static double Omega_nonu, OmegaLambda, m_Hubble;

static void init_hubble_function(_omega_nu *omnu, const double Omega0, const double UnitTime_in_s)
{
    m_omnu = omnu;
    Omega_nonu = Omega0 - get_omega_nu(omnu, 1);
    OmegaLambda = 1 - Omega0;
    m_Hubble = HUBBLE * UnitTime_in_s;
}

double hubble_function(double a)
{
    if (!m_omnu)
        terminate(1, "init_hubble_function was not called\n");
    double omega_tot = Omega_nonu / pow(a, 3) + OmegaLambda;
    omega_tot += get_omega_nu(m_omnu, a);
    omega_tot += get_omegag(m_omnu, a);
    return m_Hubble * sqrt(omega_tot);
}

void terminate(int ierr, const char *fmt, ...)
{
    va_list va;
    va_start(va, fmt);
    fprintf(stderr, "terminate(%d): ", ierr);
    vfprintf(stderr, fmt, va);
    va_end(va);
    printf("terminated %d\n", ierr);
    fflush(stdout);
    exit(ierr % 256 ? ierr % 256 : 1);
}

void message(int ierr, const char *fmt, ...)
{
    (void)ierr;
    (void)fmt;
}

static void put(const char *name, const double *v, int n)
{
    printf("%s %d", name, n);
    for (int i = 0; i < n; i++)
        printf(" %.17g", v[i]);
    printf("\n");
}

static void put1(const char *name, double v) { put(name, &v, 1); }

static void check(const char *name, int ok) { printf("check %s %d\n", name, ok ? 1 : 0); }

static double *read_bin(const char *dir, const char *name, int n)
{
    char path[2000];
    snprintf(path, sizeof(path), "%s/%s", dir, name);
    FILE *f = fopen(path, "rb");
    double *v = (double *)malloc(sizeof(double) * (n > 0 ? n : 1));
    if (!f || fread(v, sizeof(double), n, f) != (size_t)n) {
        fprintf(stderr, "cannot read %s\n", path);
        exit(2);
    }
    fclose(f);
    return v;
}

static void row(const _delta_tot_table *d, int col, double *out)
{
    for (int k = 0; k < d->nk; k++)
        out[k] = d->delta_tot[k][col];
}

int main(int argc, char **argv)
{
    if (argc < 5) {
        fprintf(stderr, "usage: %s indir n t_n outdir\n", argv[0]);
        return 2;
    }
    const char *indir = argv[1], *outdir = argv[4];
    const int n = atoi(argv[2]), tn = atoi(argv[3]);
    double *keff = read_bin(indir, "keff.bin", n), *dcdm = read_bin(indir, "dcdm.bin", n);
    _transfer_init_table transfer;
    transfer.NPowerTable = tn;
    transfer.logk = (double *)malloc(2 * sizeof(double) * tn);
    transfer.T_nu = transfer.logk + tn;
    double *tl = read_bin(indir, "tlogk.bin", tn), *tt = read_bin(indir, "tT.bin", tn);
    memcpy(transfer.logk, tl, sizeof(double) * tn);
    memcpy(transfer.T_nu, tt, sizeof(double) * tn);
    char state[2000], saved[2000];
    snprintf(state, sizeof(state), "%s/delta_tot_nu.txt", indir);
    snprintf(saved, sizeof(saved), "%s/saved_delta_tot_nu.txt", outdir);
    const double UnitLength_in_cm = 3.085678e21, UnitTime_in_s = UnitLength_in_cm / 1e5;
    double *buf = (double *)malloc(sizeof(double) * n), *buf2 = (double *)malloc(sizeof(double) * n);

    /* the test suite's set-up (delta_tot_table_test.c:368-455) */
    _omega_nu omnu;
    const double MNu[3] = {0.15, 0.15, 0.15};
    init_omega_nu(&omnu, MNu, 0.01, 0.7, T_CMB0);
    init_hubble_function(&omnu, 0.2793, UnitTime_in_s);

    /* test_delta_tot_init (:127-152) */
    {
        _delta_tot_table d;
        allocate_delta_tot_table(&d, n, 0.01, 1, 0.2793, &omnu, UnitTime_in_s, UnitLength_in_cm, 0);
        delta_tot_init(&d, n, keff, dcdm, &transfer, 0.01);
        check("init_ia", d.ia == 1);
        check("init_scalefact0", d.scalefact[0] == log(0.01));
        const double OmegaNua3 = get_omega_nu(&omnu, 0.01) * pow(0.01, 3);
        const double OmegaNu1 = get_omega_nu(&omnu, 1);
        int ok = 1;
        for (int ik = 0; ik < d.nk; ik++) {
            ok &= d.delta_nu_init[ik] > 0 && d.delta_nu_last[ik] > 0;
            ok &= fabs(d.delta_nu_last[ik] / d.delta_nu_init[ik] - 1) < 1e-4;
            const double before = get_delta_tot(d.delta_nu_init[ik], dcdm[ik], OmegaNua3, d.Omeganonu, OmegaNu1, 0);
            ok &= fabs(d.delta_tot[ik][0] / before - 1) < 1e-4;
        }
        check("init_known_answers", ok);
        put("init_fresh_nu_init", d.delta_nu_init, d.nk);
        put("init_fresh_nu_last", d.delta_nu_last, d.nk);
        row(&d, 0, buf);
        put("init_fresh_row0", buf, d.nk);
        free_delta_tot_table(&d);
    }

    /* test_save_resume (:83-124) and test_get_delta_nu_update (:193-228) */
    _delta_tot_table d;
    {
        allocate_delta_tot_table(&d, n, 0.01, 1, 0.2793, &omnu, UnitTime_in_s, UnitLength_in_cm, 0);
        read_all_nu_state(&d, state);
        check("resume_ia", d.ia == 25);
        check("resume_scalefact0", fabs(d.scalefact[0] / log(0.01) - 1) < 1e-5);
        int ok = 1;
        for (int i = 1; i < d.ia; i++) {
            ok &= d.scalefact[i] > d.scalefact[i - 1];
            for (int kk = 0; kk < d.nk; kk++)
                ok &= d.delta_tot[kk][i] > 0;
        }
        check("resume_table_positive", ok);
        delta_tot_init(&d, n, keff, dcdm, &transfer, 0.33333333);
        check("resume_init_ia", d.ia == 25);
        ok = 1;
        for (int ik = 0; ik < d.nk; ik++)
            ok &= d.delta_nu_init[ik] > 0 && d.delta_nu_last[ik] > 0;
        check("resume_init_positive", ok);
        put("resume_nu_init", d.delta_nu_init, d.nk);
        put("resume_nu_last", d.delta_nu_last, d.nk);
        check("resume_will_update", log(0.3333333) - d.scalefact[d.ia - 1] > 1e-5);
        /* the integrals alone at the last stored time */
        const double a_last = exp(d.scalefact[d.ia - 1]);
        get_delta_nu(&d, a_last, keff, buf, 0.15);
        put("resume_getdnu_m015", buf, d.nk);
        get_delta_nu(&d, a_last, keff, buf, 0.05);
        put("resume_getdnu_m005", buf, d.nk);
        get_delta_nu_combined(&d, a_last, keff, buf);
        put("resume_getdnu_combined", buf, d.nk);
        /* update, then throw the last row away by hand and update again (:214-227) */
        get_delta_nu_update(&d, 0.33333333, n, keff, dcdm, buf, &transfer);
        put1("update1_ia", d.ia);
        put("update1_dnu", buf, n);
        d.ia--;
        get_delta_nu_update(&d, 0.33333333, n, keff, dcdm, buf, &transfer);
        put1("update2_ia", d.ia);
        put("update2_dnu", buf, n);
        /* update_delta_tot: a new row, then the same row overwritten */
        for (int i = 0; i < n; i++)
            buf2[i] = buf[i] * 1.01;
        update_delta_tot(&d, 0.345, dcdm, buf2, 0);
        put1("update_new_ia", d.ia);
        row(&d, d.ia - 1, buf);
        put("update_new_row", buf, d.nk);
        double *dc2 = (double *)malloc(sizeof(double) * n);
        for (int i = 0; i < n; i++)
            dc2[i] = dcdm[i] * 1.02;
        update_delta_tot(&d, 0.35, dc2, buf2, 1);
        put1("update_over_ia", d.ia);
        row(&d, d.ia - 1, buf);
        put("update_over_row", buf, d.nk);
        put1("update_over_loga", d.scalefact[d.ia - 1]);
        free(dc2);
        /* save, read back into a second table (:106-123), save again (.bak rotation) */
        unlink(saved);
        save_all_nu_state(&d, saved);
        _delta_tot_table d2;
        allocate_delta_tot_table(&d2, n, 0.01, 1, 0.2793, &omnu, UnitTime_in_s, UnitLength_in_cm, 0);
        read_all_nu_state(&d2, saved);
        ok = d.ia == d2.ia && d.nk == d2.nk;
        for (int i = 1; i < d.ia && ok; i++) {
            ok &= fabs(d.scalefact[i] / d2.scalefact[i] - 1) < 1e-6;
            for (int kk = 0; kk < d.nk; kk++)
                ok &= fabs(d.delta_tot[kk][i] / d2.delta_tot[kk][i] - 1) < 1e-6;
        }
        check("save_resume_roundtrip", ok);
        /* the state read back, initialised (delta_nu_init from its first row, nothing
         * truncated), drives the integrator like the original */
        delta_tot_init(&d2, n, keff, dcdm, &transfer, exp(d2.scalefact[d2.ia - 1]) * (1 + 1e-9));
        get_delta_nu_combined(&d2, exp(d2.scalefact[d2.ia - 1]), keff, buf);
        get_delta_nu_combined(&d, exp(d.scalefact[d.ia - 1]), keff, buf2);
        double worst = 0;
        for (int i = 0; i < n; i++)
            worst = fmax(worst, fabs(buf[i] / buf2[i] - 1));
        put1("roundtrip_combined_rel", worst);
        save_all_nu_state(&d2, saved);
        char bak[2100];
        snprintf(bak, sizeof(bak), "%s.bak", saved);
        check("save_bak_rotation", access(bak, F_OK) == 0);
        save_nu_power(&d, 0.35, 4, outdir);
        free_delta_tot_table(&d2);
    }

    /* test_allocate_delta_tot_table (:57-80): massless neutrinos, a table in other units */
    _delta_tot_table d0;
    {
        _omega_nu omnu0;
        const double M0[3] = {0, 0, 0};
        init_omega_nu(&omnu0, M0, 0.01, 0.7, T_CMB0);
        allocate_delta_tot_table(&d0, 300, 0.01, 1, 0.2793, &omnu0, 1, 1, 0);
        int ok = d0.ia == 0 && d0.namax > 10 && d0.scalefact && d0.delta_nu_init && d0.delta_nu_last &&
                 d0.delta_tot;
        for (int i = 0; i < d0.nk_allocated; i++)
            ok &= d0.delta_tot[i] != NULL;
        check("allocate_fields", ok);
        get_delta_nu_update(&d0, 0.02, n, keff, dcdm, buf, &transfer);
        put("massless_dnu", buf, n);
        put1("massless_ia", d0.ia);
    }

    /* test_specialJ (:156-172) */
    {
        int ok = specialJ(0, -1, 0) == 1;
        ok &= fabs(specialJ(1, -1, 0) - 0.2117) < 1e-3;
        ok &= fabs(specialJ(2, -1, 0) - 0.0223807) < 1e-3;
        ok &= fabs(specialJ(0.5, -1, 0) - 0.614729) < 1e-3;
        ok &= fabs(specialJ(0.3, -1, 0) - 0.829763) < 1e-3;
        ok &= fabs(specialJ(0, 1, 0) - 0.940437) < 1e-4;
        ok &= fabs(specialJ(0.5, 1e-2, 0.5) - 0.614729 / 0.5) < 1e-3;
        ok &= fabs(specialJ(0.5, 1, 0.5) - 0.556557 / 0.5) < 1e-4;
        ok &= fabs(specialJ(1, 0.1, 0.5) - 0.211662 / 0.5) < 1e-4;
        check("specialJ_known_answers", ok);
        const double xs[10] = {0.0, 1e-3, 0.1, 0.3, 0.5, 1, 2, 5, 20, 100};
        const double qn[5][2] = {{-1.0, 0.0}, {1e-2, 0.5}, {0.5, 0.2}, {1.0, 0.5}, {3.0, 0.1}};
        double v[12];
        for (int j = 0; j < 5; j++) {
            v[0] = qn[j][0];
            v[1] = qn[j][1];
            for (int i = 0; i < 10; i++)
                v[2 + i] = specialJ(xs[i], qn[j][0], qn[j][1]);
            char name[32];
            snprintf(name, sizeof(name), "sj_row%d", j);
            put(name, v, 12);
        }
        const double qcs[7] = {0.0, 0.1, 0.5, 1.0, 2.0, 3.0, 10.0};
        for (int i = 0; i < 7; i++)
            v[i] = nufrac_low(qcs[i]);
        put("nufrac_val", v, 7);
    }

    /* test_fslength (:174-189), with the H(a) of the last allocated table */
    {
        const double kT = BOLEVK * TNUCMB * T_CMB0;
        int ok = fabs(fslength(log(0.5), log(1), 299792.) / 1272.92 / (0.45 / kT) - 1) < 1e-5;
        ok &= fabs(fslength(log(0.1), log(0.5), 299792.) / 5427.8 / (0.6 / kT) - 1) < 1e-5;
        check("fslength_known_answers", ok);
        const double iv[5][2] = {{log(0.5), 0.0}, {log(0.1), log(0.5)}, {log(0.01), log(0.3)},
                                 {log(0.02), log(0.021)}, {0.0, -1.0}};
        double v[5];
        for (int i = 0; i < 5; i++)
            v[i] = fslength(iv[i][0], iv[i][1], 299792.);
        put("fsl_val", v, 5);
    }
    /* delta_pow.h: init_delta_pow borrows the arrays, get_dnudcdm_powerspec interpolates */
    {
        double lk[3] = {0.0, 1.0, 2.0}, r[3] = {1.0, 3.0, 2.0};
        _delta_pow dp;
        init_delta_pow(&dp, lk, r, 3, 2.0);
        double v[4] = {get_dnudcdm_powerspec(&dp, 0.5), get_dnudcdm_powerspec(&dp, 1.5),
                       get_dnudcdm_powerspec(&dp, 5.0), get_dnudcdm_powerspec(&dp, -0.1)};
        put("dpow_vals", v, 4);
        free_d_pow(&dp);
    }
    free_delta_tot_table(&d0);
    free_delta_tot_table(&d);
    printf("done\n");
    return 0;
}
