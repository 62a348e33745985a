/* kspace_delta_tot_table.c -- the integrator-level kspace-neutrinos interface
 * (delta_tot_table.h, delta_pow.h, omega_nu_single.h, transfer_init.h) on the C ABI of
 * libkspace_gb300.so.  Compile into the host program and link the library:
 *
 *   cc -I<repo>/include -c kspace_delta_tot_table.c && link with -L... -lkspace_gb300
 *
 * Each _omega_nu and each _delta_tot_table owns a GPU context (omega_nu: the
 * Fermi-Dirac tables; delta_tot_table: its own copy of the background plus the history
 * on the device).  The reference's structures are kept field for field and stay the
 * truth between calls: on entry a call compares the host fields with what it last
 * exchanged with the GPU and sends any difference (the reference's own tests edit
 * d_tot.ia directly, delta_tot_table_test.c:220; set_nu_state fills the arrays,
 * interface_common.c:166-180); on return it copies back what the call changed.  File
 * I/O (the state file, P_nu output, the transfer table) runs here in the reference's
 * formats, on those host fields.  The GPU used is KSPACE_GPU_DEVICE, else 0.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
#include "kspace_delta_tot_table.h"
#include "kspace_gpu.h"
#include "kspace_hubble_match.h"

#define KSP_LIGHTCGS 2.99792458e10
#define KSP_HUBBLE 3.24077929e-18

/* what the host held when it last exchanged state with an omega_nu's context */
struct kspace_omnu_priv {
    kspace_ctx *ctx;
    double MNu[NUSPECIES], a0, HubbleParam, tcmb0;
    _rho_nu_single tab[NUSPECIES];
    _hybrid_nu hyb_sent;
    struct kspace_omnu_priv *next; /* registry of live omega_nu objects */
    const _omega_nu *owner;
};

struct kspace_dtt_priv {
    kspace_ctx *ctx;
    _hybrid_nu hyb_sent;
    double Omega0, UnitTime_in_s, TimeMax;
    int hubble_matched;
    /* the host fields as last exchanged with the GPU */
    int nk, ia, init_done;
    double *sf;  /* [namax] */
    double *tab; /* [nk_allocated][namax] */
    double *vec; /* init | last | wavenum, [nk_allocated] each */
    /* the transfer table last sent */
    double *t_copy;
    int t_n;
};

static struct kspace_omnu_priv *g_omnus = NULL;
static struct kspace_dtt_priv *g_last_table = NULL;

static void check(int st, const char *where)
{
    if (st != KSPACE_OK)
        terminate(st, "%s: %s\n", where, kspace_gpu_error_string(st));
}

static int pick_device(void)
{
    const char *e = getenv("KSPACE_GPU_DEVICE");
    return e ? atoi(e) : 0;
}

static void *xmalloc(size_t n)
{
    void *p = malloc(n ? n : 1);
    if (!p)
        terminate(1, "kspace_delta_tot_table: out of host memory (%zu bytes)\n", n);
    return p;
}

/* ------------------------------------------------------------------ omega_nu_single.h */
static struct kspace_omnu_priv *omnu_priv(const _omega_nu *omnu, const char *where)
{
    if (!omnu || !omnu->gpu)
        terminate(10003, "%s: _omega_nu not initialised by init_omega_nu\n", where);
    struct kspace_omnu_priv *P = omnu->gpu;
    /* hybrid parameters the host changed since (init_hybrid_nu or a direct edit) */
    if (memcmp(&P->hyb_sent, &omnu->hybnu, sizeof(_hybrid_nu)) != 0) {
        check(kspace_gpu_set_hybrid(P->ctx, omnu->hybnu.enabled, omnu->hybnu.vcrit, omnu->hybnu.nu_crit_time,
                                    omnu->hybnu.nufrac_low), where);
        P->hyb_sent = omnu->hybnu;
    }
    return P;
}

/* omega_nu_single.c:16-51 */
void init_omega_nu(_omega_nu *const omnu, const double MNu[], const double a0, const double HubbleParam,
                   const double tcmb0)
{
    struct kspace_omnu_priv *P = (struct kspace_omnu_priv *)xmalloc(sizeof(*P));
    memset(P, 0, sizeof(*P));
    check(kspace_gpu_create(&P->ctx, pick_device()), "init_omega_nu");
    check(kspace_gpu_init_omega_nu(P->ctx, MNu, a0, HubbleParam, tcmb0), "init_omega_nu");
    for (int i = 0; i < NUSPECIES; i++)
        P->MNu[i] = MNu[i];
    P->a0 = a0;
    P->HubbleParam = HubbleParam;
    P->tcmb0 = tcmb0;
    memset(&omnu->hybnu, 0, sizeof(omnu->hybnu)); /* hybrid neutrinos off (:19-20) */
    P->hyb_sent = omnu->hybnu;
    omnu->tcmb0 = tcmb0;
    check(kspace_gpu_background_info(P->ctx, &omnu->rhocrit, &omnu->kBtnu, omnu->nu_degeneracies, NULL),
          "init_omega_nu");
    for (int i = 0; i < NUSPECIES; i++) {
        P->tab[i].loga = P->tab[i].rhonu = NULL; /* the tables live on the GPU */
        P->tab[i].interp = P->tab[i].acc = NULL;
        P->tab[i].mnu = MNu[i];
        omnu->RhoNuTab[i] = omnu->nu_degeneracies[i] ? &P->tab[i] : NULL;
    }
    P->owner = omnu;
    P->next = g_omnus;
    g_omnus = P;
    omnu->gpu = P;
}

double get_omega_nu(const _omega_nu *const omnu, const double a)
{
    double o = 0;
    check(kspace_gpu_omega_nu(omnu_priv(omnu, "get_omega_nu")->ctx, a, &o, NULL), "get_omega_nu");
    return o;
}

double get_omega_nu_nopart(const _omega_nu *const omnu, const double a)
{
    double o = 0;
    check(kspace_gpu_omega_nu(omnu_priv(omnu, "get_omega_nu_nopart")->ctx, a, NULL, &o), "get_omega_nu_nopart");
    return o;
}

double get_omegag(const _omega_nu *const omnu, const double a)
{
    double o = 0;
    check(kspace_gpu_omega_g(omnu_priv(omnu, "get_omegag")->ctx, a, &o), "get_omegag");
    return o;
}

double omega_nu_single(const _omega_nu *const omnu, const double a, const int i)
{
    double o = 0;
    check(kspace_gpu_omega_nu_single(omnu_priv(omnu, "omega_nu_single")->ctx, a, i, &o), "omega_nu_single");
    return o;
}

/* omega_nu_single.c:214-228 */
double nufrac_low(const double qc)
{
    double out = 0;
    check(kspace_gpu_nufrac_low(NULL, &qc, 1, &out), "nufrac_low");
    return out;
}

/* omega_nu_single.c:230-240: the fractions are integrated on the device of the
 * _omega_nu the structure belongs to (the current device otherwise) */
void init_hybrid_nu(_hybrid_nu *const hybnu, const double mnu[], const double vcrit, const double light,
                    const double nu_crit_time, const double kBtnu)
{
    kspace_ctx *ctx = NULL;
    for (struct kspace_omnu_priv *P = g_omnus; P; P = P->next)
        if (&P->owner->hybnu == hybnu)
            ctx = P->ctx;
    double qc[NUSPECIES];
    for (int i = 0; i < NUSPECIES; i++)
        qc[i] = mnu[i] * vcrit / light / kBtnu;
    hybnu->enabled = 1;
    hybnu->nu_crit_time = nu_crit_time;
    hybnu->vcrit = vcrit / light;
    check(kspace_gpu_nufrac_low(ctx, qc, NUSPECIES, hybnu->nufrac_low), "init_hybrid_nu");
}

/* omega_nu_single.c:246-257 */
double particle_nu_fraction(const _hybrid_nu *const hybnu, const double a, int i)
{
    if (!hybnu->enabled)
        return 0;
    if (a > hybnu->nu_crit_time)
        return hybnu->nufrac_low[i];
    return 0;
}

/* ------------------------------------------------------------------ transfer_init.h */
/* transfer_init.c:9-83 */
void allocate_transfer_init_table(_transfer_init_table *t_init, const double BoxSize, const double UnitLength_in_cm,
                                  const double InputSpectrum_UnitLength_in_cm, const char *KspaceTransferFunction)
{
    const double scale = InputSpectrum_UnitLength_in_cm / UnitLength_in_cm;
    const double kmin = M_PI / BoxSize * scale;
    char line[1000];
    FILE *fd = fopen(KspaceTransferFunction, "r");
    if (!fd)
        terminate(2019, "Can't read input transfer function in file '%s'\n", KspaceTransferFunction);
    int n = 0;
    while (fgets(line, sizeof(line), fd)) {
        double k, t[7];
        if (line[0] == '#')
            continue;
        if (sscanf(line, " %lg %lg %lg %lg %lg %lg %lg %lg", &k, t, t + 1, t + 2, t + 3, t + 4, t + 5, t + 6) != 8)
            break;
        if (k > kmin)
            n++;
    }
    fclose(fd);
    t_init->NPowerTable = n;
    t_init->logk = (double *)xmalloc(2 * (size_t)n * sizeof(double));
    t_init->T_nu = t_init->logk + n;
    if (!(fd = fopen(KspaceTransferFunction, "r")))
        terminate(2020, "Can't read input transfer function in file '%s'\n", KspaceTransferFunction);
    int count = 0;
    while (count < n && fgets(line, sizeof(line), fd)) {
        double k, Tc, Tb, Tg, Tr, Tnu, Ttot, Tnonu;
        if (line[0] == '#')
            continue;
        if (sscanf(line, " %lg %lg %lg %lg %lg %lg %lg %lg", &k, &Tc, &Tb, &Tg, &Tr, &Tnu, &Ttot, &Tnonu) != 8)
            break;
        if (k > kmin) {
            t_init->T_nu[count] = Tnu / Tnonu;
            t_init->logk[count] = log(k / scale);
            count++;
        }
    }
    fclose(fd);
    if (count < n)
        terminate(2021, "Expected %d rows in  file '%s' but only found %d\n", n, KspaceTransferFunction, count);
}

void free_transfer_init_table(_transfer_init_table *t_init)
{
    free(t_init->logk);
    t_init->logk = t_init->T_nu = NULL;
}

/* ------------------------------------------------------------------ delta_tot_table.h */
static struct kspace_dtt_priv *dtt_priv(const _delta_tot_table *d, const char *where)
{
    if (!d || !d->gpu)
        terminate(10003, "%s: table not allocated by allocate_delta_tot_table\n", where);
    return d->gpu;
}

/* Copy the host fields into the record of what the GPU holds. */
static void remember(const _delta_tot_table *d, struct kspace_dtt_priv *P)
{
    P->nk = d->nk;
    P->ia = d->ia;
    P->init_done = d->delta_tot_init_done;
    const size_t na = (size_t)d->namax;
    memcpy(P->sf, d->scalefact, sizeof(double) * (size_t)d->ia);
    for (int k = 0; k < d->nk; k++)
        memcpy(P->tab + k * na, d->delta_tot[k], sizeof(double) * (size_t)d->ia);
    const size_t nka = (size_t)d->nk_allocated;
    memcpy(P->vec, d->delta_nu_init, sizeof(double) * (size_t)d->nk);
    memcpy(P->vec + nka, d->delta_nu_last, sizeof(double) * (size_t)d->nk);
    memcpy(P->vec + 2 * nka, d->wavenum, sizeof(double) * (size_t)d->nk);
}

static int differs(const _delta_tot_table *d, const struct kspace_dtt_priv *P)
{
    if (d->nk != P->nk || d->ia != P->ia || d->delta_tot_init_done != P->init_done)
        return 1;
    if (memcmp(P->sf, d->scalefact, sizeof(double) * (size_t)d->ia))
        return 1;
    const size_t na = (size_t)d->namax, nka = (size_t)d->nk_allocated;
    for (int k = 0; k < d->nk; k++)
        if (memcmp(P->tab + k * na, d->delta_tot[k], sizeof(double) * (size_t)d->ia))
            return 1;
    return memcmp(P->vec, d->delta_nu_init, sizeof(double) * (size_t)d->nk) ||
           memcmp(P->vec + nka, d->delta_nu_last, sizeof(double) * (size_t)d->nk) ||
           memcmp(P->vec + 2 * nka, d->wavenum, sizeof(double) * (size_t)d->nk);
}

/* Before a call: the background's hybrid parameters, the match of the host's H(a), and
 * any change the host made to the table. */
static struct kspace_dtt_priv *push(const _delta_tot_table *d, const char *where)
{
    struct kspace_dtt_priv *P = dtt_priv(d, where);
    if (d->nk < 0 || d->nk > d->nk_allocated || d->ia < 0 || d->ia > d->namax)
        terminate(2011, "%s: nk=%d (allocated %d) or ia=%d (namax %d) out of range\n", where, d->nk,
                  d->nk_allocated, d->ia, d->namax);
    const _hybrid_nu *h = &d->omnu->hybnu;
    if (memcmp(&P->hyb_sent, h, sizeof(_hybrid_nu)) != 0) {
        check(kspace_gpu_set_hybrid(P->ctx, h->enabled, h->vcrit, h->nu_crit_time, h->nufrac_low), where);
        P->hyb_sent = *h;
    }
    if (!P->hubble_matched) {
        double err = 0;
        const int st = kspace_match_hubble(P->ctx, P->Omega0, P->UnitTime_in_s, d->TimeTransfer, P->TimeMax, &err);
        if (st)
            terminate(st, "%s: hubble_function could not be matched on the GPU (best relative difference %g)\n",
                      where, err);
        P->hubble_matched = 1;
    }
    if (differs(d, P)) {
        check(kspace_gpu_set_table(P->ctx, d->nk, d->ia, d->delta_tot_init_done, d->scalefact,
                                   d->nk > 0 ? d->delta_tot[0] : NULL, (size_t)d->namax, d->delta_nu_init,
                                   d->delta_nu_last, d->wavenum), where);
        remember(d, P);
    }
    return P;
}

/* After a call that changed the state: columns from col0 on, the vectors, nk, ia and
 * the init flag. */
static void pull(_delta_tot_table *d, struct kspace_dtt_priv *P, int col0, const char *where)
{
    int nk = 0, ia = 0, init = 0;
    check(kspace_gpu_get_table(P->ctx, col0, &nk, &ia, &init, d->scalefact, d->nk_allocated ? d->delta_tot[0] : NULL,
                               (size_t)d->namax, d->delta_nu_init, d->delta_nu_last, d->wavenum), where);
    d->nk = nk;
    d->ia = ia;
    d->delta_tot_init_done = init;
    remember(d, P);
}

static void push_transfer(struct kspace_dtt_priv *P, const _transfer_init_table *t, const char *where)
{
    if (!t || t->NPowerTable <= 0)
        return;
    const int n = t->NPowerTable;
    if (P->t_n == n && !memcmp(P->t_copy, t->logk, sizeof(double) * n) &&
        !memcmp(P->t_copy + n, t->T_nu, sizeof(double) * n))
        return;
    check(kspace_gpu_set_transfer(P->ctx, t->logk, t->T_nu, n), where);
    free(P->t_copy);
    P->t_copy = (double *)xmalloc(2 * sizeof(double) * (size_t)n);
    memcpy(P->t_copy, t->logk, sizeof(double) * n);
    memcpy(P->t_copy + n, t->T_nu, sizeof(double) * n);
    P->t_n = n;
}

/* delta_tot_table.c:25-60 */
void allocate_delta_tot_table(_delta_tot_table *d_tot, const int nk_in, const double TimeTransfer,
                              const double TimeMax, const double Omega0, const _omega_nu *const omnu,
                              const double UnitTime_in_s, const double UnitLength_in_cm, int debug)
{
    struct kspace_omnu_priv *O = omnu_priv(omnu, "allocate_delta_tot_table");
    d_tot->nk_allocated = nk_in;
    d_tot->nk = nk_in;
    d_tot->TimeTransfer = TimeTransfer;
    d_tot->namax = (int)ceil(100 * (TimeMax - TimeTransfer)) + 2;
    d_tot->ia = 0;
    d_tot->delta_tot_init_done = 0;
    const size_t na = (size_t)d_tot->namax;
    d_tot->delta_tot = (double **)xmalloc((size_t)nk_in * sizeof(double *));
    d_tot->scalefact = (double *)xmalloc(na * ((size_t)nk_in + 1) * sizeof(double));
    memset(d_tot->scalefact, 0, na * ((size_t)nk_in + 1) * sizeof(double));
    for (int k = 0; k < nk_in; k++)
        d_tot->delta_tot[k] = d_tot->scalefact + na + (size_t)k * na;
    d_tot->delta_nu_init = (double *)xmalloc(3 * (size_t)nk_in * sizeof(double));
    memset(d_tot->delta_nu_init, 0, 3 * (size_t)nk_in * sizeof(double));
    d_tot->delta_nu_last = d_tot->delta_nu_init + nk_in;
    d_tot->wavenum = d_tot->delta_nu_init + 2 * nk_in;
    d_tot->omnu = omnu;
    d_tot->light = KSP_LIGHTCGS * UnitTime_in_s / UnitLength_in_cm;
    d_tot->delta_nu_prefac = 1.5 * Omega0 * KSP_HUBBLE * KSP_HUBBLE * pow(UnitTime_in_s, 2) / d_tot->light;
    d_tot->Omeganonu = Omega0 - get_omega_nu(omnu, 1);
    d_tot->debug = debug;
    /* the table's own context: the same background, then the history buffers */
    struct kspace_dtt_priv *P = (struct kspace_dtt_priv *)xmalloc(sizeof(*P));
    memset(P, 0, sizeof(*P));
    check(kspace_gpu_create(&P->ctx, pick_device()), "allocate_delta_tot_table");
    check(kspace_gpu_init_omega_nu(P->ctx, O->MNu, O->a0, O->HubbleParam, O->tcmb0), "allocate_delta_tot_table");
    const _hybrid_nu *h = &omnu->hybnu;
    check(kspace_gpu_set_hybrid(P->ctx, h->enabled, h->vcrit, h->nu_crit_time, h->nufrac_low),
          "allocate_delta_tot_table");
    P->hyb_sent = *h;
    check(kspace_gpu_alloc_table(P->ctx, nk_in, TimeTransfer, TimeMax, Omega0, UnitTime_in_s, UnitLength_in_cm),
          "allocate_delta_tot_table");
    P->Omega0 = Omega0;
    P->UnitTime_in_s = UnitTime_in_s;
    P->TimeMax = TimeMax;
    P->sf = (double *)xmalloc(na * sizeof(double));
    P->tab = (double *)xmalloc(na * (size_t)nk_in * sizeof(double));
    P->vec = (double *)xmalloc(3 * (size_t)nk_in * sizeof(double));
    P->nk = nk_in; /* what the fresh context holds */
    P->ia = 0;
    P->init_done = 0;
    d_tot->gpu = P;
    g_last_table = P;
}

/* delta_tot_table.c:63-68 */
void free_delta_tot_table(_delta_tot_table *d_tot)
{
    struct kspace_dtt_priv *P = d_tot->gpu;
    free(d_tot->delta_tot);
    free(d_tot->scalefact);
    free(d_tot->delta_nu_init);
    if (P) {
        if (g_last_table == P)
            g_last_table = NULL;
        kspace_gpu_destroy(P->ctx);
        free(P->sf);
        free(P->tab);
        free(P->vec);
        free(P->t_copy);
        free(P);
    }
    d_tot->gpu = NULL;
}

/* delta_tot_table.c:79-149 */
void delta_tot_init(_delta_tot_table *const d_tot, const int nk_in, const double wavenum[],
                    const double delta_cdm_curr[], const _transfer_init_table *const t_init, const double Time)
{
    struct kspace_dtt_priv *P = push(d_tot, "delta_tot_init");
    push_transfer(P, t_init, "delta_tot_init");
    check(kspace_gpu_delta_tot_init(P->ctx, nk_in, wavenum, delta_cdm_curr, Time), "delta_tot_init");
    pull(d_tot, P, 0, "delta_tot_init");
    if (d_tot->ThisTask == 0 && d_tot->debug)
        save_all_nu_state(d_tot, NULL);
}

/* delta_tot_table.c:177-191 */
void update_delta_tot(_delta_tot_table *const d_tot, const double a, const double delta_cdm_curr[],
                      const double delta_nu_curr[], const int overwrite)
{
    struct kspace_dtt_priv *P = push(d_tot, "update_delta_tot");
    const int ia0 = d_tot->ia;
    check(kspace_gpu_update_delta_tot(P->ctx, a, delta_cdm_curr, delta_nu_curr, overwrite), "update_delta_tot");
    pull(d_tot, P, ia0 > 0 ? ia0 - 1 : 0, "update_delta_tot");
}

/* delta_tot_table.c:193-250 */
void get_delta_nu_update(_delta_tot_table *const d_tot, const double a, const int nk_in, const double keff[],
                         const double P_cdm_curr[], double delta_nu_curr[], _transfer_init_table *transfer_init)
{
    if (!d_tot->delta_tot_init_done)
        delta_tot_init(d_tot, nk_in, keff, P_cdm_curr, transfer_init, a);
    struct kspace_dtt_priv *P = push(d_tot, "get_delta_nu_update");
    const int ia0 = d_tot->ia;
    check(kspace_gpu_get_delta_nu_update(P->ctx, a, nk_in, keff, P_cdm_curr, delta_nu_curr), "get_delta_nu_update");
    pull(d_tot, P, ia0 > 0 ? ia0 - 1 : 0, "get_delta_nu_update");
    if (d_tot->ia > ia0 && d_tot->ThisTask == 0 && d_tot->debug)
        save_delta_tot(d_tot, d_tot->ia - 1, NULL);
}

/* delta_tot_table.c:507-611 (nk = d_tot->nk values) */
void get_delta_nu(const _delta_tot_table *const d_tot, const double a, const double wavenum[],
                  double delta_nu_curr[], const double mnu)
{
    struct kspace_dtt_priv *P = push(d_tot, "get_delta_nu");
    if (d_tot->nk > 0)
        check(kspace_gpu_get_delta_nu(P->ctx, a, d_tot->nk, wavenum, delta_nu_curr, mnu), "get_delta_nu");
}

/* delta_tot_table.c:153-172 */
void get_delta_nu_combined(const _delta_tot_table *const d_tot, const double a, const double wavenum[],
                           double delta_nu_curr[])
{
    struct kspace_dtt_priv *P = push(d_tot, "get_delta_nu_combined");
    if (d_tot->nk > 0)
        check(kspace_gpu_get_delta_nu_combined(P->ctx, a, d_tot->nk, wavenum, delta_nu_curr),
              "get_delta_nu_combined");
}

/* delta_tot_table.c:304-325 */
void save_delta_tot(const _delta_tot_table *const d_tot, const int iia, char *savefile)
{
    const char *dfile = savefile ? savefile : "delta_tot_nu.txt";
    FILE *fd = fopen(dfile, "a");
    if (!fd)
        terminate(2012, "Could not open %s for writing!\n", dfile);
    fprintf(fd, "# %le ", d_tot->scalefact[iia]);
    for (int i = 0; i < d_tot->nk; i++)
        fprintf(fd, "%le ", d_tot->delta_tot[i][iia]);
    fprintf(fd, "\n");
    fclose(fd);
}

/* delta_tot_table.c:327-352: an existing file is renamed to <file>.bak first */
void save_all_nu_state(const _delta_tot_table *const d_tot, char *savefile)
{
    const char *f = savefile ? savefile : "delta_tot_nu.txt";
    if (access(f, F_OK) != -1) {
        const size_t n = strlen(f) + 6;
        char *bak = (char *)xmalloc(n);
        snprintf(bak, n, "%s.bak", f);
        rename(f, bak);
        free(bak);
    }
    for (int ik = 0; ik < d_tot->ia; ik++)
        save_delta_tot(d_tot, ik, (char *)f);
}

/* delta_tot_table.c:356-374 */
int save_nu_power(const _delta_tot_table *const d_tot, const double Time, const int snapnum, const char *OutputDir)
{
    char fname[1000];
    snprintf(fname, sizeof(fname), "%s/powerspec_nu_%03d.txt", OutputDir, snapnum);
    FILE *fd = fopen(fname, "w");
    if (!fd) {
        fprintf(stderr, "can't open file `%s` for writing\n", fname);
        return -1;
    }
    fprintf(fd, "# k P_nu(k)\n");
    fprintf(fd, "# a = %g\n", Time);
    fprintf(fd, "# nbins = %d\n", d_tot->nk);
    for (int i = 0; i < d_tot->nk; i++)
        fprintf(fd, "%g %g\n", d_tot->wavenum[i], d_tot->delta_nu_last[i] * d_tot->delta_nu_last[i]);
    fclose(fd);
    return 0;
}

/* delta_tot_table.c:254-301: rows into the host fields; the next call sends them */
void read_all_nu_state(_delta_tot_table *const d_tot, char *savefile)
{
    const char *dfile = savefile ? savefile : "delta_tot_nu.txt";
    FILE *fd = fopen(dfile, "r");
    if (!fd)
        return;
    int iia;
    for (iia = 0; iia < d_tot->namax; iia++) {
        double scale;
        if (fscanf(fd, "# %lg ", &scale) != 1)
            break;
        d_tot->scalefact[iia] = scale;
        for (int ik = 0; ik < d_tot->nk; ik++) {
            if (fscanf(fd, "%lg ", &(d_tot->delta_tot[ik][iia])) != 1) {
                if (iia != 0) {
                    fclose(fd);
                    terminate(2006, "Expected %d k values, got %d for delta_tot in %s; a=%g\n", d_tot->nk, ik, dfile,
                              exp(d_tot->scalefact[iia]));
                } else {
                    d_tot->nk = ik;
                    break;
                }
            }
        }
    }
    fclose(fd);
    if (fabs(d_tot->scalefact[0] - log(d_tot->TimeTransfer)) > 1e-4)
        terminate(2007, "%s starts wih a=%g, transfer function is at a=%g\n", dfile, exp(d_tot->scalefact[0]),
                  d_tot->TimeTransfer);
    if (iia > 0)
        d_tot->ia = iia;
}

/* delta_tot_table.c:457-463 */
double specialJ(const double x, const double vcmnubylight, const double nufrac_low)
{
    double out = 0;
    check(kspace_gpu_special_j(NULL, &x, 1, vcmnubylight, nufrac_low, &out), "specialJ");
    return out;
}

/* delta_tot_table.c:394-407, with the H(a) of the most recently allocated table */
double fslength(const double logai, const double logaf, const double light)
{
    if (logai >= logaf)
        return 0;
    struct kspace_dtt_priv *P = g_last_table;
    if (!P)
        terminate(10003, "fslength: needs H(a); allocate a delta_tot table first\n");
    if (!P->hubble_matched) {
        double err = 0;
        const double alo = exp(logai) < 0.01 ? exp(logai) : 0.01;
        const double ahi = exp(logaf) > P->TimeMax ? exp(logaf) : P->TimeMax;
        const int st = kspace_match_hubble(P->ctx, P->Omega0, P->UnitTime_in_s, alo, ahi, &err);
        if (st)
            terminate(st, "fslength: hubble_function does not match the GPU model (%g)\n", err);
        P->hubble_matched = 1;
    }
    double out = 0;
    check(kspace_gpu_fslength(P->ctx, &logai, &logaf, 1, light, &out), "fslength");
    return out;
}

/* delta_tot_table.c:613-617 */
double get_delta_tot(const double delta_nu_curr, const double delta_cdm_curr, const double OmegaNua3,
                     const double Omeganonu, const double Omeganu1, const double partnu)
{
    const double fcdm = 1 - OmegaNua3 / (Omeganonu + Omeganu1);
    return fcdm * (delta_cdm_curr + delta_nu_curr * OmegaNua3 / (Omeganonu + Omeganu1 * partnu));
}

/* ------------------------------------------------------------------ delta_pow.h */
/* delta_pow.c:6-17: the table is borrowed, not copied */
void init_delta_pow(_delta_pow *d_pow, double logkk[], double delta_ratio[], int nbins, double norm)
{
    d_pow->logkk = logkk;
    d_pow->delta_ratio = delta_ratio;
    d_pow->nbins = nbins;
    d_pow->norm = norm;
    d_pow->spline = NULL;
    d_pow->acc = NULL;
}

/* delta_pow.c:19-37 */
double get_dnudcdm_powerspec(_delta_pow *d_pow, double kk)
{
    const double *x = d_pow->logkk, *y = d_pow->delta_ratio;
    const int n = d_pow->nbins;
    if (kk < x[0] && kk > x[0] - log(2))
        kk = x[0];
    if (kk < x[0] - log(2)) {
        fprintf(stderr, "trying to extract a k= %g < min stored = %g \n", kk, x[0]);
        kk = x[0];
    }
    if (kk > x[n - 1])
        kk = x[n - 1];
    int lo = 0, hi = n - 1;
    while (hi > lo + 1) {
        const int mid = (lo + hi) / 2;
        if (x[mid] > kk)
            hi = mid;
        else
            lo = mid;
    }
    return d_pow->norm * (y[lo] + (kk - x[lo]) * ((y[lo + 1] - y[lo]) / (x[lo + 1] - x[lo])));
}

/* delta_pow.c:39-43 */
void free_d_pow(_delta_pow *d_pow)
{
    d_pow->spline = NULL;
    d_pow->acc = NULL;
}
