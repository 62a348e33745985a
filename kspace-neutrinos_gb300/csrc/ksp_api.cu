// ksp_api.cu -- host side of libkspace_gb300.so: the C ABI of include/kspace_gpu.h.
//
// The control flow of the reference's integrator bookkeeping (which row is provisional,
// when a row is committed, resume truncation, error checks) runs here on the host
// exactly as in delta_tot_table.c:79-250; every number is computed on the device.
// A context holds what the reference keeps in process-global singletons
// (interface_common.c:17-26, interface_gadget.c:19-21).
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
#include <atomic>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <vector>
#include "ksp_ctx.h"

using namespace ksp;

namespace ksp {
std::atomic<long long> g_launches{0};
}

// ------------------------------------------------------------------ helpers
#define CK(x)                                                                                         \
    do {                                                                                              \
        cudaError_t e__ = (x);                                                                        \
        if (e__ != cudaSuccess) {                                                                     \
            fprintf(stderr, "kspace_gpu: CUDA error %s at %s:%d\n", cudaGetErrorString(e__), __FILE__, __LINE__); \
            return KSPACE_ERR_CUDA;                                                                   \
        }                                                                                             \
    } while (0)

#define NEED(cond, code) \
    do {                 \
        if (!(cond)) return (code); \
    } while (0)

template <class T>
static cudaError_t dalloc(T** p, size_t n) {
    return cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (n ? n : 1));
}

int ksp::map_status(unsigned s) {
    if (s & kStTimeout) return KSPACE_ERR_TIMEOUT;
    if (s & kStKmax) return KSPACE_ERR_KMAX;
    if (s & kStDnuNaN) return KSPACE_ERR_DNU_NAN;
    if (s & kStGsl) return KSPACE_ERR_GSL;
    if (s & kStGridNaN) return KSPACE_ERR_GRID_NAN;
    return KSPACE_OK;
}

// Synchronise with the stream and convert the device status word.
static int sync_status(kspace_ctx* c) {
    CK(cudaMemcpyAsync(c->status_h, c->status_d, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    const unsigned s = *c->status_h;
    if (s & kStKWarn)
        fprintf(stderr, "kspace_gpu: a mode with k below half the smallest binned k was clamped to it\n");
    if (s) CK(cudaMemsetAsync(c->status_d, 0, sizeof(unsigned), c->stream));
    return map_status(s);
}

int ksp::raise_dynamic_smem_limit(const void* kernel) {
    static std::mutex m;
    static std::set<std::pair<const void*, int>> done;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    std::lock_guard<std::mutex> lock(m);
    if (done.count(std::make_pair(kernel, dev))) return 0;
    cudaFuncAttributes fa;
    int optin = 0;
    if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return -1;
    const int lim = optin - (int)fa.sharedSizeBytes;
    if (lim <= 0 || cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, lim) != cudaSuccess)
        return -1;
    done.insert(std::make_pair(kernel, dev));
    return 0;
}

bool ksp::is_device_ptr(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// ------------------------------------------------------------------ lifecycle
extern "C" int kspace_gpu_create(kspace_ctx** out, int device) {
    NEED(out, KSPACE_ERR_ARG);
    kspace_ctx* c = new kspace_ctx();
    c->device = device;
    CK(cudaSetDevice(device));
    CK(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
    c->stream = c->own_stream;
    CK(dalloc(&c->status_d, 1));
    CK(cudaMemset(c->status_d, 0, sizeof(unsigned)));
    CK(cudaMallocHost(reinterpret_cast<void**>(&c->status_h), sizeof(unsigned)));
    CK(dalloc(&c->dB, 1));
    for (int i = 0; i < 5; i++) CK(cudaEventCreate(&c->ev[i]));
    CK(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking));
    for (int i = 0; i < kspace_ctx::kChunks; i++) {
        CK(cudaEventCreateWithFlags(&c->ev_up[i], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c->ev_done[i], cudaEventDisableTiming));
    }
    CK(cudaEventCreateWithFlags(&c->ev_copy_start, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_copy_end, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    if (const char* e = getenv("KSPACE_GPU_TMA")) c->tma = atoi(e);
    if (const char* e = getenv("KSPACE_GPU_CHUNKS")) c->chunks = atoi(e);
    if (const char* e = getenv("KSPACE_GPU_ROWS")) c->rows = atoi(e);
    if (const char* e = getenv("KSPACE_GPU_STAGES")) c->stages = atoi(e);
    if (const char* e = getenv("KSPACE_GPU_QAG_WARPS")) c->qag_warps = atoi(e);
    if (const char* e = getenv("KSPACE_GPU_QAG_SPLIT")) c->qag_split = atoi(e);
    if (const char* e = getenv("KSPACE_GPU_NC_LEVELS")) {
        const int l = atoi(e);
        c->nc_levels = l < 0 ? 0 : (l > kNcMaxLevels ? kNcMaxLevels : l);
    }
    *out = c;
    return KSPACE_OK;
}

static void free_table(kspace_ctx* c) {
    IntegratorDev& I = c->I;
    void* ptrs[] = {I.scalefact, I.dtot, I.coef, I.nu_init, I.nu_last, I.wavenum, I.dcdm, I.dnu_s, I.dnu,
                    I.knot_invdiag, I.knot_fac, I.knot_invh, I.knot_h3, I.knot_ih3, I.nc_g, I.nc_fsl,
                    I.nc_dx, I.nc_j, I.fs_x, I.fs_y, I.fs_c, I.fs_seg, I.t_logk, I.t_T, I.t_c, I.sc,
                    I.qag_max, I.qag_total, I.coef_unit};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    memset(&I, 0, sizeof(I));
    void* bufs[] = {c->bin_sum_d, c->power_d, c->keffg_d, c->keff_d, c->logk_d, c->ratio_d,
                    c->norm_d, c->dnu_out_d, c->io_d, c->corr.xf, c->corr.rn, c->corr.sn};
    for (void* p : bufs)
        if (p) cudaFree(p);
    c->bin_sum_d = c->F0sq_d = c->power_d = c->keffg_d = c->keff_d = nullptr;
    c->logk_d = c->ratio_d = c->norm_d = c->dnu_out_d = c->io_d = nullptr;
    c->corr = CorrTable{};
    if (c->ar_h) cudaFreeHost(c->ar_h);
    c->ar_h = nullptr;
    void* adj[] = {c->ivals_d, c->adj_node_d, c->adj_Dbar_d, c->adj_mbar_d, c->adj_Q_d, c->adj_dcsum_d,
                   c->adj_dnubar_d, c->adj_rbar_d, c->nivals_d};
    for (void* p : adj)
        if (p) cudaFree(p);
    c->ivals_d = c->adj_node_d = c->adj_Dbar_d = c->adj_mbar_d = c->adj_Q_d = c->adj_dcsum_d = nullptr;
    c->adj_dnubar_d = c->adj_rbar_d = nullptr;
    c->nivals_d = nullptr;
    c->adj_cap_nb = 0;
    c->diff_ready = false;
    c->table_ready = false;
}

extern "C" int kspace_gpu_destroy(kspace_ctx* c) {
    if (!c) return KSPACE_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    if (c->side) cudaStreamSynchronize(c->side);
    free_table(c);
    for (auto& kv : c->geos) {
        Geo& g = kv.second;
        cudaFree(g.g.thresh);
        cudaFree(g.g.w1);
        cudaFree(g.g.cmap);
        if (g.g.runtab) cudaFree(g.g.runtab);
        cudaFree(g.count_d);
        cudaFree(g.ksum_d);
        cudaFree(g.compact_d);
    }
    if (c->stage_d) cudaFree(c->stage_d);
    if (c->htab_dev) cudaFree(c->htab_dev);
    if (c->dB) cudaFree(c->dB);
    if (c->status_d) cudaFree(c->status_d);
    if (c->status_h) cudaFreeHost(c->status_h);
    for (int i = 0; i < 5; i++)
        if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->side) cudaStreamDestroy(c->side);
    for (int i = 0; i < kspace_ctx::kChunks; i++) {
        if (c->ev_up[i]) cudaEventDestroy(c->ev_up[i]);
        if (c->ev_done[i]) cudaEventDestroy(c->ev_done[i]);
    }
    if (c->ev_copy_start) cudaEventDestroy(c->ev_copy_start);
    if (c->ev_copy_end) cudaEventDestroy(c->ev_copy_end);
    if (c->copy) cudaStreamDestroy(c->copy);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
    return KSPACE_OK;
}

extern "C" const char* kspace_gpu_error_string(int s) {
    switch (s) {
    case KSPACE_OK: return "success";
    case KSPACE_ERR_NOMEM: return "could not allocate memory";
    case KSPACE_ERR_KMAX: return "k beyond the largest k of the transfer table";
    case KSPACE_ERR_GRID_NAN: return "delta_nu or delta_cdm is nan";
    case KSPACE_ERR_GSL: return "integration or interpolation failed";
    case KSPACE_ERR_NK_MISMATCH: return "number of k bins differs from the stored delta_tot";
    case KSPACE_ERR_NK_SMALL: return "number of k bins is unreasonably small";
    case KSPACE_ERR_DNU_NAN: return "delta_nu is nan";
    case KSPACE_ERR_STATE_SHORT: return "incomplete row in the saved delta_tot table";
    case KSPACE_ERR_STATE_START: return "saved delta_tot table starts at another scale factor";
    case KSPACE_ERR_NK_ALLOC: return "more k bins than allocated";
    case KSPACE_ERR_SAVE_OPEN: return "could not open the state file for writing";
    case KSPACE_ERR_TRANSFER_OPEN: return "cannot read the transfer function file";
    case KSPACE_ERR_TRANSFER_SHORT: return "transfer function file ended early";
    case KSPACE_ERR_NO_RESUME: return "no delta_tot history although the run starts after the transfer time";
    case KSPACE_ERR_TIME_BEFORE: return "scale factor before the transfer function time";
    case KSPACE_ERR_NAMAX: return "delta_tot history table is full";
    case KSPACE_ERR_CUDA: return "CUDA error";
    case KSPACE_ERR_ARG: return "invalid argument";
    case KSPACE_ERR_ORDER: return "call made before the state it needs was set up";
    case KSPACE_ERR_HUBBLE: return "host hubble_function differs from the device background model";
    case KSPACE_ERR_TIMEOUT: return "a bounded device wait expired";
    default: return "unknown status";
    }
}

extern "C" int kspace_gpu_set_stream(kspace_ctx* c, void* st) {
    NEED(c, KSPACE_ERR_ARG);
    c->stream = st ? reinterpret_cast<cudaStream_t>(st) : c->own_stream;
    return KSPACE_OK;
}

extern "C" int kspace_gpu_set_allreduce(kspace_ctx* c, kspace_allreduce_fn fn, void* user) {
    NEED(c, KSPACE_ERR_ARG);
    c->ar_fn = fn;
    c->ar_user = user;
    return KSPACE_OK;
}

extern "C" int kspace_gpu_set_tuning(kspace_ctx* c, int tma, int rows, int stages, int qag_warps) {
    NEED(c, KSPACE_ERR_ARG);
    if (tma >= 0) c->tma = tma;
    if (rows > 0) c->rows = rows;
    if (stages > 0) c->stages = stages;
    if (qag_warps > 0) c->qag_warps = qag_warps;
    return KSPACE_OK;
}

extern "C" long long kspace_gpu_launch_count(kspace_ctx* c) {
    (void)c;
    return g_launches.load();
}

// ------------------------------------------------------------------ background
static void upload_background(kspace_ctx* c) {
    cudaMemcpyAsync(c->dB, &c->hB, sizeof(Background), cudaMemcpyHostToDevice, c->stream);
}

extern "C" int kspace_gpu_init_omega_nu(kspace_ctx* c, const double MNu[3], double a0, double h, double tcmb0) {
    NEED(c && MNu, KSPACE_ERR_ARG);
    CK(cudaSetDevice(c->device));
    Background& B = c->hB;
    memset(&B, 0, sizeof(B));
    // omega_nu_single.c:16-51
    B.tcmb0 = tcmb0;
    B.kBtnu = kBolEvK * (pow(4 / 11., 1 / 3.) * 1.00328) * tcmb0;
    B.rhocrit = (3 * kHubble * h * kHubble * h) / (8 * kPi * kGravity);
    B.irhocrit = 1.0 / B.rhocrit;
    B.conv = rho_nu_conversion();
    B.omegag0 = 4 * kStefanBoltzmann / (kLightCgs * kLightCgs * kLightCgs) * pow(tcmb0, 4) / B.rhocrit;
    for (int mi = 0; mi < kNuSpecies; mi++) {
        int mmi;
        B.deg[mi] = 0;
        for (mmi = 0; mmi < mi; mmi++) {
            if (fabs(MNu[mi] - MNu[mmi]) < kFloatAcc) {
                B.deg[mmi] += 1;
                break;
            }
        }
        if (mmi == mi) B.deg[mi] = 1;
    }
    c->nspec = 0;
    for (int mi = 0; mi < kNuSpecies; mi++) {
        c->MNu[mi] = MNu[mi];
        B.mnu[mi] = MNu[mi];
        B.mnu_J[mi] = MNu[mi];
        RhoTable& T = B.tab[mi];
        T.mnu = MNu[mi];
        T.has_table = 0;
        if (B.deg[mi]) {
            c->spec_ids[c->nspec++] = mi;
            // omega_nu_single.c:122-130,143: table range and knots
            const double logA0 = log(a0) - log(1.2);
            const double logaf = log(kNuSw * B.kBtnu / MNu[mi]) + log(1.2);
            if (!(MNu[mi] < 1e-6 * B.kBtnu || logaf < logA0)) {
                T.has_table = 1;
                for (int i = 0; i < kNRhoTab; i++) T.loga[i] = logA0 + i * (logaf - logA0) / (kNRhoTab - 1);
            }
        }
    }
    c->bg_a0 = a0;
    upload_background(c);
    launch_background_tables(c->dB, a0, c->stream, c->status_d);
    g_launches += 2;
    int st = sync_status(c);
    if (st) return st;
    CK(cudaMemcpy(&c->hB, c->dB, sizeof(Background), cudaMemcpyDeviceToHost));
    c->bg_ready = true;
    c->hubble_ready = false;
    return KSPACE_OK;
}

extern "C" int kspace_gpu_init_hybrid_nu(kspace_ctx* c, double vcrit, double light, double nu_crit_time) {
    NEED(c, KSPACE_ERR_ARG);
    NEED(c->bg_ready, KSPACE_ERR_ORDER);
    c->hB.hyb_enabled = 1;
    c->hB.nu_crit_time = nu_crit_time;
    c->hB.vcrit = vcrit / light;
    upload_background(c);
    launch_nufrac_low(c->dB, light, vcrit, c->stream, c->status_d);
    g_launches += 1;
    int st = sync_status(c);
    if (st) return st;
    CK(cudaMemcpy(&c->hB, c->dB, sizeof(Background), cudaMemcpyDeviceToHost));
    return KSPACE_OK;
}

// The hybrid-neutrino parameters as a host's _hybrid_nu holds them (omega_nu_single.h:51-64):
// vcrit as a fraction of light speed, the switch-on time and the particle fractions.
extern "C" int kspace_gpu_set_hybrid(kspace_ctx* c, int enabled, double vcrit_frac, double nu_crit_time,
                                     const double* nufrac_low) {
    NEED(c && nufrac_low, KSPACE_ERR_ARG);
    NEED(c->bg_ready, KSPACE_ERR_ORDER);
    Background& B = c->hB;
    B.hyb_enabled = enabled ? 1 : 0;
    B.vcrit = vcrit_frac;
    B.nu_crit_time = nu_crit_time;
    for (int i = 0; i < kNuSpecies; i++) B.nufrac_low[i] = nufrac_low[i];
    upload_background(c);
    CK(cudaStreamSynchronize(c->stream));
    return KSPACE_OK;
}

extern "C" int kspace_gpu_set_hubble(kspace_ctx* c, double Omega0, double OmegaLambda, double UnitTime_in_s,
                                     int radiation) {
    NEED(c, KSPACE_ERR_ARG);
    NEED(c->bg_ready, KSPACE_ERR_ORDER);
    Background& B = c->hB;
    B.htab_n = 0;  // the analytic form
    B.Omega_nonu_H = Omega0 - omega_nu(B, 1);
    B.OmegaLambda = OmegaLambda;
    B.OmegaK = 1.0 - Omega0 - OmegaLambda;
    B.hubble = kHubble * UnitTime_in_s;
    B.radiation = radiation;
    upload_background(c);
    CK(cudaStreamSynchronize(c->stream));
    c->hubble_ready = true;
    return KSPACE_OK;
}

// A host H(a) of any form: n >= 4 samples H[i] = H(exp(loga_lo + i * dloga)); log H is
// interpolated by a natural cubic spline in log a (built on the device), continued by
// the end segments outside the table.
extern "C" int kspace_gpu_set_hubble_table(kspace_ctx* c, double loga_lo, double dloga, int n, const double* H) {
    NEED(c && H && n >= 4 && dloga > 0, KSPACE_ERR_ARG);
    NEED(c->bg_ready, KSPACE_ERR_ORDER);
    for (int i = 0; i < n; i++) NEED(H[i] > 0 && isfinite(H[i]), KSPACE_ERR_ARG);
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    if (c->htab_dev) cudaFree(c->htab_dev);
    c->htab_dev = nullptr;
    CK(dalloc(&c->htab_dev, 4 * (size_t)n));  // 4 coefficients per segment (n - 1 segments)
    double* scratch = nullptr;
    CK(dalloc(&scratch, 2 * (size_t)n));
    CK(cudaMemcpyAsync(scratch, H, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    launch_hubble_table(scratch, n, dloga, c->htab_dev, scratch + n, c->stream);
    g_launches += 1;
    c->htab_host.assign(4 * (size_t)n, 0.0);
    CK(cudaMemcpyAsync(c->htab_host.data(), c->htab_dev, sizeof(double) * 4 * (n - 1), cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    cudaFree(scratch);
    Background& B = c->hB;
    B.htab_d = c->htab_dev;
    B.htab_h = c->htab_host.data();
    B.htab_n = n;
    B.htab_lo = loga_lo;
    B.htab_dx = dloga;
    upload_background(c);
    CK(cudaStreamSynchronize(c->stream));
    c->hubble_ready = true;
    return KSPACE_OK;
}

extern "C" int kspace_gpu_check_hubble(kspace_ctx* c, const double* a, const double* H, int n, double rtol,
                                       double* max_rel) {
    NEED(c && a && H, KSPACE_ERR_ARG);
    NEED(c->hubble_ready, KSPACE_ERR_ORDER);
    double mx = 0;
    for (int i = 0; i < n; i++) {
        const double h = hubble(c->hB, a[i]);
        const double r = fabs(h / H[i] - 1);
        if (!(r <= mx)) mx = r;
    }
    if (max_rel) *max_rel = mx;
    return mx <= rtol ? KSPACE_OK : KSPACE_ERR_HUBBLE;
}

extern "C" int kspace_gpu_omega_nu(kspace_ctx* c, double a, double* om, double* om_nop) {
    NEED(c, KSPACE_ERR_ARG);
    NEED(c->bg_ready, KSPACE_ERR_ORDER);
    if (om) *om = omega_nu(c->hB, a);
    if (om_nop) *om_nop = omega_nu_nopart(c->hB, a);
    return KSPACE_OK;
}

extern "C" int kspace_gpu_particle_nu_active(kspace_ctx* c, double a, int* active) {
    NEED(c && active, KSPACE_ERR_ARG);
    NEED(c->bg_ready, KSPACE_ERR_ORDER);
    *active = particle_nu_fraction(c->hB, a, 0) == 0. ? 0 : 1;
    return KSPACE_OK;
}

extern "C" int kspace_gpu_hubble(kspace_ctx* c, double a, double* H) {
    NEED(c && H, KSPACE_ERR_ARG);
    NEED(c->hubble_ready, KSPACE_ERR_ORDER);
    *H = hubble(c->hB, a);
    return KSPACE_OK;
}

// ------------------------------------------------------------------ table
extern "C" int kspace_gpu_alloc_table(kspace_ctx* c, int nk_alloc, double TimeTransfer, double TimeMax, double Omega0,
                                      double UnitTime_in_s, double UnitLength_in_cm) {
    NEED(c && nk_alloc > 0, KSPACE_ERR_ARG);
    NEED(c->bg_ready, KSPACE_ERR_ORDER);
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    free_table(c);
    IntegratorDev& I = c->I;
    I.B = c->dB;
    I.nk_alloc = nk_alloc;
    I.namax = (int)ceil(100 * (TimeMax - TimeTransfer)) + 2;  // delta_tot_table.c:36
    NEED(I.namax > 1, KSPACE_ERR_ARG);
    I.ld = (I.namax + 1) & ~1;  // even: every row starts on a 16-byte boundary
    const size_t nk = nk_alloc, ld = I.ld;
    CK(dalloc(&I.scalefact, ld));
    CK(dalloc(&I.dtot, nk * ld));
    CK(dalloc(&I.coef, nk * ld));
    CK(cudaMemset(I.dtot, 0, sizeof(double) * nk * ld));
    CK(cudaMemset(I.coef, 0, sizeof(double) * nk * ld));
    CK(dalloc(&I.coef_unit, ld));
    CK(dalloc(&I.nu_init, nk));
    CK(dalloc(&I.nu_last, nk));
    CK(dalloc(&I.wavenum, nk));
    CK(dalloc(&I.dcdm, nk));
    CK(dalloc(&I.dnu_s, kNuSpecies * nk));
    CK(dalloc(&I.dnu, nk));
    CK(dalloc(&I.knot_invdiag, ld));
    CK(dalloc(&I.knot_fac, ld));
    CK(dalloc(&I.knot_invh, ld));
    CK(dalloc(&I.knot_h3, ld));
    CK(dalloc(&I.knot_ih3, ld));
    CK(dalloc(&I.nc_g, kNcNodes));
    CK(dalloc(&I.nc_fsl, kNcNodes));
    CK(dalloc(&I.nc_dx, kNcNodes));
    CK(dalloc(&I.nc_j, kNcNodes));
    I.nc_slots = c->nc_levels > 0 ? 1 + 2 * c->nc_levels : 0;
    I.fs_cap = 16 * (int)ld + 16;
    CK(dalloc(&I.fs_x, I.fs_cap));
    CK(dalloc(&I.fs_y, I.fs_cap));
    CK(dalloc(&I.fs_c, I.fs_cap));
    CK(dalloc(&I.fs_seg, I.fs_cap));
    CK(dalloc(&I.sc, 1));
    CK(dalloc(&I.qag_max, 1));
    CK(dalloc(&I.qag_total, 1));
    I.status = c->status_d;
    StepScalars S;
    memset(&S, 0, sizeof(S));
    S.light = kLightCgs * UnitTime_in_s / UnitLength_in_cm;                   // :52
    S.prefac = 1.5 * Omega0 * kHubble * kHubble * pow(UnitTime_in_s, 2) / S.light;  // :53
    S.Omeganonu = Omega0 - omega_nu(c->hB, 1);                                 // :55
    c->Omeganonu = S.Omeganonu;
    CK(cudaMemcpy(I.sc, &S, sizeof(S), cudaMemcpyHostToDevice));
    // step buffers
    c->buf_nb = nk_alloc;
    CK(dalloc(&c->bin_sum_d, nk + 1));
    c->F0sq_d = c->bin_sum_d + nk;
    CK(dalloc(&c->power_d, nk));
    CK(dalloc(&c->keffg_d, nk));
    CK(dalloc(&c->keff_d, nk));
    CK(dalloc(&c->logk_d, nk));
    CK(dalloc(&c->ratio_d, nk));
    CK(dalloc(&c->norm_d, 1));
    CK(dalloc(&c->dnu_out_d, nk));
    CK(dalloc(&c->io_d, 4 * nk));
    CK(dalloc(&c->corr.xf, nk));
    CK(dalloc(&c->corr.rn, nk));
    CK(dalloc(&c->corr.sn, nk));
    CK(cudaMallocHost(reinterpret_cast<void**>(&c->ar_h), sizeof(double) * (nk + 1)));
    c->TimeTransfer = TimeTransfer;
    c->loga0 = log(TimeTransfer);
    c->nk = nk_alloc;
    c->ia = 0;
    c->init_done = 0;
    c->fact_valid = 0;
    c->h_scalefact.assign(I.namax, 0.0);
    c->table_ready = true;
    if (c->transfer_ready) {
        // re-upload the transfer table for the new allocation
        std::vector<double> lk = c->t_logk, tt = c->t_T;
        c->transfer_ready = false;
        return kspace_gpu_set_transfer(c, lk.data(), tt.data(), (int)lk.size());
    }
    return KSPACE_OK;
}

extern "C" int kspace_gpu_set_transfer(kspace_ctx* c, const double* logk, const double* T, int n) {
    NEED(c && logk && T && n >= 3, KSPACE_ERR_ARG);
    c->t_logk.assign(logk, logk + n);
    c->t_T.assign(T, T + n);
    c->transfer_ready = true;
    if (!c->table_ready) return KSPACE_OK;
    IntegratorDev& I = c->I;
    if (I.t_logk) cudaFree(I.t_logk);
    if (I.t_T) cudaFree(I.t_T);
    if (I.t_c) cudaFree(I.t_c);
    CK(dalloc(&I.t_logk, n));
    CK(dalloc(&I.t_T, n));
    CK(dalloc(&I.t_c, 3 * n));
    I.ntrans = n;
    CK(cudaMemcpy(I.t_logk, logk, sizeof(double) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(I.t_T, T, sizeof(double) * n, cudaMemcpyHostToDevice));
    launch_spline_coeffs_1thread(I.t_logk, I.t_T, I.t_c, I.t_c + n, n, c->stream);
    g_launches += 1;
    CK(cudaStreamSynchronize(c->stream));
    return KSPACE_OK;
}

// transfer_init.c:9-83 (host reader of a CAMB transfer file; 8 leading columns)
extern "C" int kspace_gpu_read_transfer_file(kspace_ctx* c, double BoxSize, double UnitLength_in_cm,
                                             double InputUnit, const char* path, int* nrows) {
    NEED(c && path, KSPACE_ERR_ARG);
    const double scale = (InputUnit / UnitLength_in_cm);
    const double kmin = kPi / BoxSize * scale;
    FILE* fd = fopen(path, "r");
    if (!fd) return KSPACE_ERR_TRANSFER_OPEN;
    std::vector<double> lk, tt;
    char line[1000];
    while (fgets(line, sizeof(line), fd)) {
        if (line[0] == '#') continue;
        double k, Tc, Tb, Tg, Tr, Tnu, Ttot, Tnonu;
        if (sscanf(line, " %lg %lg %lg %lg %lg %lg %lg %lg", &k, &Tc, &Tb, &Tg, &Tr, &Tnu, &Ttot, &Tnonu) != 8) break;
        if (k > kmin) {
            tt.push_back(Tnu / Tnonu);
            lk.push_back(log(k / scale));
        }
    }
    fclose(fd);
    if (nrows) *nrows = (int)lk.size();
    if (lk.size() < 3) return KSPACE_ERR_TRANSFER_SHORT;
    return kspace_gpu_set_transfer(c, lk.data(), tt.data(), (int)lk.size());
}

extern "C" int kspace_gpu_set_nu_state(kspace_ctx* c, const double* scalefact, const double* delta_tot, size_t nk,
                                       size_t ia) {
    NEED(c && scalefact && delta_tot, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    IntegratorDev& I = c->I;
    NEED((int)ia <= I.namax && (int)nk <= I.nk_alloc, KSPACE_ERR_NK_ALLOC);
    c->nk = (int)nk;
    c->ia = (int)ia;
    for (size_t i = 0; i < ia; i++) c->h_scalefact[i] = scalefact[i];
    CK(cudaMemcpyAsync(I.scalefact, scalefact, sizeof(double) * ia, cudaMemcpyHostToDevice, c->stream));
    if (ia > 0 && nk > 0)  // delta_tot may be host or device memory
        CK(cudaMemcpy2DAsync(I.dtot, sizeof(double) * I.ld, delta_tot, sizeof(double) * ia, sizeof(double) * ia, nk,
                             cudaMemcpyDefault, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->fact_valid = 0;
    return KSPACE_OK;
}

extern "C" int kspace_gpu_get_nu_state(kspace_ctx* c, double* scalefact, double* delta_tot, size_t* nk, size_t* ia) {
    NEED(c, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    if (nk) *nk = c->nk;
    if (ia) *ia = c->ia;
    if (scalefact) memcpy(scalefact, c->h_scalefact.data(), sizeof(double) * c->ia);
    if (delta_tot && c->ia > 0 && c->nk > 0)
        CK(cudaMemcpy2D(delta_tot, sizeof(double) * c->ia, c->I.dtot, sizeof(double) * c->I.ld,
                        sizeof(double) * c->ia, c->nk, cudaMemcpyDeviceToHost));
    return KSPACE_OK;
}

extern "C" int kspace_gpu_table_info(kspace_ctx* c, int* ints) {
    NEED(c && ints, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    ints[0] = c->nk;
    ints[1] = c->I.nk_alloc;
    ints[2] = c->I.namax;
    ints[3] = c->ia;
    ints[4] = c->init_done;
    return KSPACE_OK;
}

extern "C" int kspace_gpu_get_vectors(kspace_ctx* c, double* nu_init, double* nu_last, double* wavenum) {
    NEED(c, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    CK(cudaStreamSynchronize(c->stream));
    const size_t n = sizeof(double) * c->I.nk_alloc;
    if (nu_init) CK(cudaMemcpy(nu_init, c->I.nu_init, n, cudaMemcpyDeviceToHost));
    if (nu_last) CK(cudaMemcpy(nu_last, c->I.nu_last, n, cudaMemcpyDeviceToHost));
    if (wavenum) CK(cudaMemcpy(wavenum, c->I.wavenum, n, cudaMemcpyDeviceToHost));
    return KSPACE_OK;
}

// read_all_nu_state (delta_tot_table.c:254-301)
extern "C" int kspace_gpu_read_nu_state(kspace_ctx* c, const char* path) {
    NEED(c, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    FILE* fd = fopen(path ? path : "delta_tot_nu.txt", "r");
    if (!fd) return KSPACE_OK;  // no file: nothing to resume
    const int namax = c->I.namax;
    int nk = c->nk;
    std::vector<double> sf(namax, 0.0), tab((size_t)c->I.nk_alloc * namax, 0.0);
    int iia;
    for (iia = 0; iia < namax; iia++) {
        double scale;
        if (fscanf(fd, "# %lg ", &scale) != 1) break;
        sf[iia] = scale;
        for (int ik = 0; ik < nk; ik++) {
            if (fscanf(fd, "%lg ", &tab[(size_t)ik * namax + iia]) != 1) {
                if (iia != 0) {
                    fclose(fd);
                    return KSPACE_ERR_STATE_SHORT;
                }
                nk = ik;
                break;
            }
        }
    }
    fclose(fd);
    if (fabs(sf[0] - log(c->TimeTransfer)) > 1e-4) return KSPACE_ERR_STATE_START;
    const int ia = iia > 0 ? iia : c->ia;
    // repack [nk][namax] -> [nk][ia]
    std::vector<double> flat((size_t)nk * (ia > 0 ? ia : 1));
    for (int ik = 0; ik < nk; ik++)
        for (int i = 0; i < ia; i++) flat[(size_t)ik * ia + i] = tab[(size_t)ik * namax + i];
    if (iia == 0) return KSPACE_OK;
    return kspace_gpu_set_nu_state(c, sf.data(), flat.data(), nk, ia);
}

static int save_rows(kspace_ctx* c, const char* path, int from, int to) {
    FILE* fd = fopen(path, "a");
    if (!fd) return KSPACE_ERR_SAVE_OPEN;
    std::vector<double> row((size_t)c->nk);
    std::vector<double> tab((size_t)c->nk * c->I.ld);
    if (c->nk > 0)
        CK(cudaMemcpy(tab.data(), c->I.dtot, sizeof(double) * tab.size(), cudaMemcpyDeviceToHost));
    for (int iia = from; iia < to; iia++) {
        fprintf(fd, "# %le ", c->h_scalefact[iia]);
        for (int i = 0; i < c->nk; i++) fprintf(fd, "%le ", tab[(size_t)i * c->I.ld + iia]);
        fprintf(fd, "\n");
    }
    fclose(fd);
    return KSPACE_OK;
}

// save_all_nu_state (delta_tot_table.c:331-352): old file renamed to .bak
extern "C" int kspace_gpu_save_nu_state(kspace_ctx* c, const char* path) {
    NEED(c, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    CK(cudaStreamSynchronize(c->stream));
    std::string p = path ? path : "delta_tot_nu.txt";
    if (access(p.c_str(), F_OK) != -1) rename(p.c_str(), (p + ".bak").c_str());
    return save_rows(c, p.c_str(), 0, c->ia);
}

// save_nu_power (delta_tot_table.c:356-374)
extern "C" int kspace_gpu_save_nu_power(kspace_ctx* c, double Time, int snapnum, const char* dir) {
    NEED(c && dir, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    char fname[1000];
    snprintf(fname, sizeof(fname), "%s/powerspec_nu_%03d.txt", dir, snapnum);
    FILE* fd = fopen(fname, "w");
    if (!fd) {
        fprintf(stderr, "can't open file `%s` for writing\n", fname);
        return -1;
    }
    std::vector<double> last(c->I.nk_alloc), wn(c->I.nk_alloc);
    int st = kspace_gpu_get_vectors(c, nullptr, last.data(), wn.data());
    if (st) {
        fclose(fd);
        return st;
    }
    fprintf(fd, "# k P_nu(k)\n");
    fprintf(fd, "# a = %g\n", Time);
    fprintf(fd, "# nbins = %d\n", c->nk);
    for (int i = 0; i < c->nk; i++) fprintf(fd, "%g %g\n", wn[i], last[i] * last[i]);
    fclose(fd);
    return 0;
}

// ------------------------------------------------------------------ integrator
// delta_tot_table.c:79-149 (host bookkeeping; numbers on the device)
static int delta_tot_init(kspace_ctx* c, int nk_in, const double* keff_d, const double* dcdm_d, double Time) {
    for (int ik = 0; ik < c->ia; ik++) {
        if (log(Time) <= c->h_scalefact[ik]) {
            c->ia = ik;
            c->fact_valid = 0;
            break;
        }
    }
    if (Time > c->TimeTransfer + 0.01 && c->ia == 0) return KSPACE_ERR_NO_RESUME;
    if (Time < c->TimeTransfer - 1e-5) return KSPACE_ERR_TIME_BEFORE;
    if (nk_in > c->I.nk_alloc) return KSPACE_ERR_NK_ALLOC;
    NEED(c->transfer_ready && c->I.t_logk, KSPACE_ERR_ORDER);
    c->nk = nk_in;
    const int fresh = c->ia == 0;
    launch_delta_tot_init(c->I, nk_in, keff_d, dcdm_d, fresh, c->TimeTransfer, c->stream);
    g_launches += 1;
    if (fresh) {
        c->h_scalefact[0] = log(c->TimeTransfer);
        CK(cudaMemcpyAsync(c->I.scalefact, &c->h_scalefact[0], sizeof(double), cudaMemcpyHostToDevice, c->stream));
        c->ia = 1;
    }
    int st = sync_status(c);
    if (st) return st;
    // delta_nu_last = delta_nu at the last stored time (delta_tot_table.c:146)
    const double a_last = exp(c->h_scalefact[c->ia - 1]);
    launch_delta_nu_combined(c->I, c->nk, c->ia, a_last, c->h_scalefact[c->ia - 1], c->loga0, c->TimeTransfer,
                             0, c->nspec, c->spec_ids, c->qag_warps, c->stream, c->qag_split);
    g_launches += 8;
    CK(cudaMemcpyAsync(c->I.nu_last, c->I.dnu, sizeof(double) * c->nk, cudaMemcpyDeviceToDevice, c->stream));
    c->fact_valid = 0;
    c->init_done = 1;
    return sync_status(c);
}

// get_delta_nu_update (delta_tot_table.c:193-250) on device arrays.  Optionally
// produces the correction table of interface_common.c:134-146.
// fin: the binning pass's normalisation when it was deferred (see bin_grid): folded into
// the row-spline kernel of a prepared step, else launched first.
// sync = false (a step whose correction pass follows on the stream): no host round trip
// at the end; the correction pass reads the status word itself and leaves the grid as it
// is after an error, which the step's final status check reports.
static int update_device(kspace_ctx* c, double a, int nk_in, const double* keff_d, const double* dcdm_d,
                         double* dnu_out_d, bool want_corr, const FinalizeArgs* fin = nullptr, bool sync = true) {
    NEED(c->table_ready && c->hubble_ready, KSPACE_ERR_ORDER);
    IntegratorDev& I = c->I;
    // side-stream work queued by start_prep writes the integrator's tables (the row
    // splines among them): nothing below runs before it, used or not
    if (c->prep_valid) CK(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
    if (fin && fin->active) {
        const double la = log(a);
        const bool will_prepare = c->prep_valid && c->init_done && nk_in == c->nk && c->nk >= 2 && c->ia >= 1 &&
                                  c->prep_Na == c->ia + 1 && c->prep_loga == la &&
                                  !(la - c->h_scalefact[c->ia - 1] < kFloatAcc) && c->ia < I.namax;
        if (!will_prepare) {
            launch_finalize_power(fin->bin_sum, fin->F0sq, fin->count, fin->ksum, fin->compact_bins, nk_in,
                                  fin->BoxSize, fin->power_out, fin->keff_out, fin->dcdm_out, fin->keffphys_out,
                                  c->stream);
            g_launches += 1;
            fin = nullptr;
        }
    }
    if (dcdm_d != I.dcdm)
        CK(cudaMemcpyAsync(I.dcdm, dcdm_d, sizeof(double) * nk_in, cudaMemcpyDeviceToDevice, c->stream));
    if (!c->init_done) {
        int st = delta_tot_init(c, nk_in, keff_d, I.dcdm, a);
        if (st) return st;
    }
    if (nk_in != c->nk) return KSPACE_ERR_NK_MISMATCH;
    if (c->nk < 2) return KSPACE_ERR_NK_SMALL;
    const double loga = log(a);
    // the delta_cdm-independent part already ran beside the binning pass (it also zeroes
    // the QAG statistics)
    const bool prepared = c->prep_valid && c->prep_Na == c->ia + 1 && c->prep_loga == loga &&
                          !(loga - c->h_scalefact[c->ia - 1] < kFloatAcc) && c->ia < I.namax;
    if (!prepared) {
        CK(cudaMemsetAsync(I.qag_max, 0, sizeof(int), c->stream));
        CK(cudaMemsetAsync(I.qag_total, 0, sizeof(long long), c->stream));
    }
    if (loga - c->h_scalefact[c->ia - 1] < kFloatAcc) {
        // same scale factor: return delta_nu_last unchanged (delta_tot_table.c:209-213)
        CK(cudaMemcpyAsync(I.dnu, I.nu_last, sizeof(double) * c->nk, cudaMemcpyDeviceToDevice, c->stream));
        if (want_corr || dnu_out_d) {
            // scalars at a (kspace_prefac) without integrating, then the table from
            // delta_nu_last passed through unclamped, as the reference returns it
            launch_delta_nu_combined(I, 0, 1, a, loga, c->loga0, c->TimeTransfer, -1, 0, c->spec_ids, c->qag_warps,
                                     c->stream);
            CK(cudaMemcpyAsync(I.dnu, I.nu_last, sizeof(double) * c->nk, cudaMemcpyDeviceToDevice, c->stream));
            launch_finish_update(I, c->nk, -2, a, loga, want_corr ? keff_d : nullptr, dnu_out_d,
                                 want_corr ? c->logk_d : nullptr, want_corr ? c->ratio_d : nullptr,
                                 want_corr ? c->corr : CorrTable{}, c->norm_d, c->stream);
            g_launches += 3;
        }
        return sync_status(c);
    }
    if (c->ia >= I.namax) return KSPACE_ERR_NAMAX;
    // provisional row from delta_nu_last (delta_tot_table.c:222): written here, or, after
    // the prepared scalars, as the rows' splines are solved
    const int prov_row = c->ia;
    if (!prepared) launch_update_row(I, c->nk, prov_row, a, loga, I.dcdm, I.nu_last, c->stream);
    c->h_scalefact[c->ia] = loga;
    c->ia++;
    const int Na = c->ia;
    I.kq = keff_d;  // the integrals at this call's k (delta_tot_table.c:224)
    if (prepared) {
        CK(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
        launch_integrator_rest(I, c->nk, Na, c->nspec, c->spec_ids, c->qag_warps, c->stream, c->qag_split, prov_row,
                               true, fin, c->prep_base);
    } else {
        launch_delta_nu_combined(I, c->nk, Na, a, loga, c->loga0, c->TimeTransfer, c->fact_valid, c->nspec,
                                 c->spec_ids, c->qag_warps, c->stream, c->qag_split);
    }
    I.kq = nullptr;
    c->prep_valid = false;
    // keep the row if far enough from the previous one (delta_tot_table.c:229-237)
    const bool commit = a >= exp(c->h_scalefact[Na - 2]) + 0.009;
    launch_finish_update(I, c->nk, commit ? Na - 1 : -1, a, loga, want_corr ? keff_d : nullptr, dnu_out_d,
                         want_corr ? c->logk_d : nullptr, want_corr ? c->ratio_d : nullptr,
                         want_corr ? c->corr : CorrTable{}, c->norm_d, c->stream, prepared);
    g_launches += 10;
    if (commit) {
        c->fact_valid = Na - 2 > 0 ? Na - 2 : 0;
    } else {
        c->ia--;
        c->fact_valid = Na - 3 > 0 ? Na - 3 : 0;
    }
    return sync ? sync_status(c) : KSPACE_OK;
}

extern "C" int kspace_gpu_get_delta_nu_update(kspace_ctx* c, double a, int nk, const double* keff,
                                              const double* P_cdm_sqrt, double* delta_nu) {
    NEED(c && keff && P_cdm_sqrt && delta_nu && nk > 0, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    NEED(nk <= c->I.nk_alloc, KSPACE_ERR_NK_ALLOC);
    double* kd = c->io_d;
    double* dd = c->io_d + c->I.nk_alloc;
    CK(cudaMemcpyAsync(kd, keff, sizeof(double) * nk, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(dd, P_cdm_sqrt, sizeof(double) * nk, cudaMemcpyHostToDevice, c->stream));
    int st = update_device(c, a, nk, kd, dd, c->dnu_out_d, false);
    if (st) return st;
    CK(cudaMemcpy(delta_nu, c->dnu_out_d, sizeof(double) * nk, cudaMemcpyDeviceToHost));
    return KSPACE_OK;
}

// delta_tot_init (delta_tot_table.c:79-149) on its own: wavenum = k (not log k) and
// dcdm = sqrt(P_cdm) of the nk bins, host or device memory.
extern "C" int kspace_gpu_delta_tot_init(kspace_ctx* c, int nk, const double* wavenum, const double* dcdm,
                                         double Time) {
    NEED(c && wavenum && dcdm && nk > 0, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    NEED(nk <= c->I.nk_alloc, KSPACE_ERR_NK_ALLOC);
    CK(cudaSetDevice(c->device));
    double* kd = c->io_d;
    CK(cudaMemcpyAsync(kd, wavenum, sizeof(double) * nk, cudaMemcpyDefault, c->stream));
    CK(cudaMemcpyAsync(c->I.dcdm, dcdm, sizeof(double) * nk, cudaMemcpyDefault, c->stream));
    return delta_tot_init(c, nk, kd, c->I.dcdm, Time);
}

// The integrals of get_delta_nu over the stored rows [0, ia) at scale factor a and the
// call's k (host or device): nspec mass states spec_ids, species sum into I.dnu.
static int integrate_stored(kspace_ctx* c, double a, int nk, const double* wavenum, int nspec, const int* spec_ids) {
    NEED(c->table_ready && c->hubble_ready, KSPACE_ERR_ORDER);
    NEED(c->transfer_ready || c->init_done || c->ia > 0, KSPACE_ERR_ORDER);
    NEED(nk > 0 && nk <= c->I.nk_alloc, KSPACE_ERR_NK_ALLOC);
    NEED(c->ia >= 1, KSPACE_ERR_ORDER);
    CK(cudaSetDevice(c->device));
    IntegratorDev& I = c->I;
    double* kd = c->io_d + 2 * (size_t)I.nk_alloc;
    CK(cudaMemcpyAsync(kd, wavenum, sizeof(double) * nk, cudaMemcpyDefault, c->stream));
    CK(cudaMemsetAsync(I.qag_max, 0, sizeof(int), c->stream));
    CK(cudaMemsetAsync(I.qag_total, 0, sizeof(long long), c->stream));
    I.kq = kd;
    // the knot factorisation is rebuilt from the first row: rows may have changed since
    launch_delta_nu_combined(I, nk, c->ia, a, log(a), c->loga0, c->TimeTransfer, 0, nspec, spec_ids, c->qag_warps,
                             c->stream, c->qag_split);
    I.kq = nullptr;
    g_launches += 8;
    c->fact_valid = 0;
    return KSPACE_OK;
}

// get_delta_nu (delta_tot_table.c:507-611): delta_nu of one mass state of mass mnu (eV)
// from the stored rows.
extern "C" int kspace_gpu_get_delta_nu(kspace_ctx* c, double a, int nk, const double* wavenum, double* delta_nu,
                                       double mnu) {
    NEED(c && wavenum && delta_nu, KSPACE_ERR_ARG);
    NEED(c->bg_ready, KSPACE_ERR_ORDER);
    // the mass enters only through m/kT in J's argument: species slot 0 carries it
    Background& B = c->hB;
    const double keep = B.mnu_J[0];
    B.mnu_J[0] = mnu;
    CK(cudaMemcpyAsync(&c->dB->mnu_J[0], &B.mnu_J[0], sizeof(double), cudaMemcpyHostToDevice, c->stream));
    const int ids[3] = {0, 0, 0};
    int st = integrate_stored(c, a, nk, wavenum, 1, ids);
    B.mnu_J[0] = keep;
    if (!st)
        CK(cudaMemcpyAsync(delta_nu, c->I.dnu_s, sizeof(double) * nk, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&c->dB->mnu_J[0], &B.mnu_J[0], sizeof(double), cudaMemcpyHostToDevice, c->stream));
    const int st2 = sync_status(c);
    return st ? st : st2;
}

// get_delta_nu_combined (delta_tot_table.c:153-172) from the stored rows.
extern "C" int kspace_gpu_get_delta_nu_combined(kspace_ctx* c, double a, int nk, const double* wavenum,
                                                double* delta_nu) {
    NEED(c && wavenum && delta_nu, KSPACE_ERR_ARG);
    int st = integrate_stored(c, a, nk, wavenum, c->nspec, c->spec_ids);
    if (st) return st;
    CK(cudaMemcpyAsync(delta_nu, c->I.dnu, sizeof(double) * nk, cudaMemcpyDeviceToHost, c->stream));
    return sync_status(c);
}

// update_delta_tot (delta_tot_table.c:177-191): row ia-1 (overwrite) or a new row ia from
// dcdm = sqrt(P_cdm) and delta_nu of the nk stored bins (host or device memory).
extern "C" int kspace_gpu_update_delta_tot(kspace_ctx* c, double a, const double* dcdm, const double* dnu,
                                           int overwrite) {
    NEED(c && dcdm && dnu, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    NEED(overwrite ? c->ia >= 1 : c->ia < c->I.namax, overwrite ? KSPACE_ERR_ORDER : KSPACE_ERR_NAMAX);
    CK(cudaSetDevice(c->device));
    const int nk = c->nk;
    double* dc = c->io_d;
    double* dn = c->io_d + c->I.nk_alloc;
    if (nk > 0) {
        CK(cudaMemcpyAsync(dc, dcdm, sizeof(double) * nk, cudaMemcpyDefault, c->stream));
        CK(cudaMemcpyAsync(dn, dnu, sizeof(double) * nk, cudaMemcpyDefault, c->stream));
    }
    if (!overwrite) c->ia++;
    const int row = c->ia - 1;
    c->h_scalefact[row] = log(a);
    launch_update_row(c->I, nk, row, a, c->h_scalefact[row], dc, dn, c->stream);
    g_launches += 1;
    c->fact_valid = 0;
    return sync_status(c);
}

// The whole integrator state in the reference's layout (delta_tot_table.h:17-57):
// scalefact[ia], delta_tot rows of stride ld (row ik at delta_tot + ik * ld), the three
// per-bin vectors (nk each), and the init flag.  Host memory.
extern "C" int kspace_gpu_set_table(kspace_ctx* c, int nk, int ia, int init_done, const double* scalefact,
                                    const double* delta_tot, size_t ld, const double* nu_init,
                                    const double* nu_last, const double* wavenum) {
    NEED(c && nk >= 0 && ia >= 0, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    IntegratorDev& I = c->I;
    NEED(nk <= I.nk_alloc && ia <= I.namax, KSPACE_ERR_NK_ALLOC);
    NEED(ia == 0 || (scalefact && delta_tot && ld >= (size_t)ia), KSPACE_ERR_ARG);
    CK(cudaSetDevice(c->device));
    c->nk = nk;
    c->ia = ia;
    for (int i = 0; i < ia; i++) c->h_scalefact[i] = scalefact[i];
    if (ia > 0) {
        CK(cudaMemcpyAsync(I.scalefact, scalefact, sizeof(double) * ia, cudaMemcpyHostToDevice, c->stream));
        if (nk > 0)
            CK(cudaMemcpy2DAsync(I.dtot, sizeof(double) * I.ld, delta_tot, sizeof(double) * ld, sizeof(double) * ia,
                                 nk, cudaMemcpyHostToDevice, c->stream));
    }
    if (nk > 0) {
        if (nu_init) CK(cudaMemcpyAsync(I.nu_init, nu_init, sizeof(double) * nk, cudaMemcpyHostToDevice, c->stream));
        if (nu_last) CK(cudaMemcpyAsync(I.nu_last, nu_last, sizeof(double) * nk, cudaMemcpyHostToDevice, c->stream));
        if (wavenum) CK(cudaMemcpyAsync(I.wavenum, wavenum, sizeof(double) * nk, cudaMemcpyHostToDevice, c->stream));
    }
    c->init_done = init_done ? 1 : 0;
    c->fact_valid = 0;
    c->prep_valid = false;
    CK(cudaStreamSynchronize(c->stream));
    return KSPACE_OK;
}

// Read the state back: columns [col0, ia) of scalefact and of every row (so a caller that
// holds the earlier columns copies only what a call may have changed), the vectors, nk,
// ia and the init flag.  Any output may be NULL.
extern "C" int kspace_gpu_get_table(kspace_ctx* c, int col0, int* nk, int* ia, int* init_done, double* scalefact,
                                    double* delta_tot, size_t ld, double* nu_init, double* nu_last,
                                    double* wavenum) {
    NEED(c && col0 >= 0, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->stream));
    const IntegratorDev& I = c->I;
    if (nk) *nk = c->nk;
    if (ia) *ia = c->ia;
    if (init_done) *init_done = c->init_done;
    if (scalefact)
        for (int i = col0; i < c->ia; i++) scalefact[i] = c->h_scalefact[i];
    if (delta_tot && c->ia > col0 && c->nk > 0) {
        NEED(ld >= (size_t)c->ia, KSPACE_ERR_ARG);
        CK(cudaMemcpy2D(delta_tot + col0, sizeof(double) * ld, I.dtot + col0, sizeof(double) * I.ld,
                        sizeof(double) * (c->ia - col0), c->nk, cudaMemcpyDeviceToHost));
    }
    if (c->nk > 0) {
        if (nu_init) CK(cudaMemcpy(nu_init, I.nu_init, sizeof(double) * c->nk, cudaMemcpyDeviceToHost));
        if (nu_last) CK(cudaMemcpy(nu_last, I.nu_last, sizeof(double) * c->nk, cudaMemcpyDeviceToHost));
        if (wavenum) CK(cudaMemcpy(wavenum, I.wavenum, sizeof(double) * c->nk, cudaMemcpyDeviceToHost));
    }
    return KSPACE_OK;
}

// ------------------------------------------------------------------ scalar functions on the device
// specialJ, nufrac_low and fslength of n arguments at once, computed by the same device
// functions the integrator uses.  ctx may be NULL for the first two (current device,
// default stream); fslength needs the context's H(a).
template <class F>
static int device_values(kspace_ctx* c, int nin, const double* in0, const double* in1, int n, double* out, F launch) {
    NEED(n >= 0 && out, KSPACE_ERR_ARG);
    if (n == 0) return KSPACE_OK;
    if (c) CK(cudaSetDevice(c->device));
    cudaStream_t st = c ? c->stream : 0;
    double* buf = nullptr;
    unsigned* status = nullptr;
    CK(cudaMalloc(&buf, sizeof(double) * (size_t)n * (nin + 1)));
    if (cudaMalloc(&status, sizeof(unsigned)) != cudaSuccess) {
        cudaFree(buf);
        return KSPACE_ERR_CUDA;
    }
    cudaError_t e = cudaMemsetAsync(status, 0, sizeof(unsigned), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf, in0, sizeof(double) * n, cudaMemcpyDefault, st);
    if (e == cudaSuccess && nin > 1) e = cudaMemcpyAsync(buf + n, in1, sizeof(double) * n, cudaMemcpyDefault, st);
    if (e == cudaSuccess) {
        launch(buf, buf + n, buf + (size_t)nin * n, status, st);
        g_launches += 1;
        e = cudaGetLastError();
    }
    unsigned s = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, buf + (size_t)nin * n, sizeof(double) * n, cudaMemcpyDefault, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&s, status, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(buf);
    cudaFree(status);
    if (e != cudaSuccess) {
        fprintf(stderr, "kspace_gpu: CUDA error %s\n", cudaGetErrorString(e));
        return KSPACE_ERR_CUDA;
    }
    return map_status(s);
}

extern "C" int kspace_gpu_special_j(kspace_ctx* c, const double* x, int n, double qc, double nufrac_low, double* out) {
    NEED(x, KSPACE_ERR_ARG);
    return device_values(c, 1, x, nullptr, n, out,
                         [&](const double* a, const double*, double* o, unsigned*, cudaStream_t st) {
                             launch_special_j(a, n, qc, nufrac_low, o, st);
                         });
}

extern "C" int kspace_gpu_nufrac_low(kspace_ctx* c, const double* qc, int n, double* out) {
    NEED(qc, KSPACE_ERR_ARG);
    return device_values(c, 1, qc, nullptr, n, out,
                         [&](const double* a, const double*, double* o, unsigned* status, cudaStream_t st) {
                             launch_nufrac_low_values(a, n, o, status, st);
                         });
}

extern "C" int kspace_gpu_fslength(kspace_ctx* c, const double* logai, const double* logaf, int n, double light,
                                   double* out) {
    NEED(c && logai && logaf, KSPACE_ERR_ARG);
    NEED(c->hubble_ready, KSPACE_ERR_ORDER);
    const Background* dB = c->dB;
    return device_values(c, 2, logai, logaf, n, out,
                         [&](const double* a, const double* b, double* o, unsigned*, cudaStream_t st) {
                             launch_fslength_values(dB, a, b, n, light, o, st);
                         });
}

// omega_nu_single (omega_nu_single.c:262-279), get_omegag (:77-81) and the fields of
// _omega_nu a host mirror needs (rhocrit, kBtnu, degeneracies, nufrac_low).
extern "C" int kspace_gpu_omega_nu_single(kspace_ctx* c, double a, int i, double* out) {
    NEED(c && out && i >= 0 && i < kNuSpecies, KSPACE_ERR_ARG);
    NEED(c->bg_ready, KSPACE_ERR_ORDER);
    *out = omega_nu_single(c->hB, a, i);
    return KSPACE_OK;
}

extern "C" int kspace_gpu_omega_g(kspace_ctx* c, double a, double* out) {
    NEED(c && out, KSPACE_ERR_ARG);
    NEED(c->bg_ready, KSPACE_ERR_ORDER);
    *out = c->hB.omegag0 / pow(a, 4);  // omega_nu_single.c:77-81
    return KSPACE_OK;
}

extern "C" int kspace_gpu_background_info(kspace_ctx* c, double* rhocrit, double* kBtnu, int* deg,
                                          double* nufrac_low) {
    NEED(c, KSPACE_ERR_ARG);
    NEED(c->bg_ready, KSPACE_ERR_ORDER);
    if (rhocrit) *rhocrit = c->hB.rhocrit;
    if (kBtnu) *kBtnu = c->hB.kBtnu;
    for (int i = 0; i < kNuSpecies; i++) {
        if (deg) deg[i] = c->hB.deg[i];
        if (nufrac_low) nufrac_low[i] = c->hB.nufrac_low[i];
    }
    return KSPACE_OK;
}

// ------------------------------------------------------------------ geometry
static int get_geo(kspace_ctx* c, int N, int nrbins, Geo** out) {
    auto key = std::make_pair(N, nrbins);
    auto it = c->geos.find(key);
    if (it != c->geos.end()) {
        *out = &it->second;
        return KSPACE_OK;
    }
    NEED(N >= 2 && (N % 2) == 0 && nrbins >= 2, KSPACE_ERR_ARG);
    NEED((long long)3 * (N / 2) * (N / 2) < (1LL << 24), KSPACE_ERR_ARG);  // k^2 exact in float
    Geo G;
    const int nz = N / 2 + 1;
    const long long k2max = 3LL * (N / 2) * (N / 2);
    // reference bin of each integer k^2 (powerspectrum.c:40,67,75,83) -> thresholds
    const double bpu = (nrbins - 1) / log(sqrt(3) * N / 2.0);
    std::vector<int> thr(nrbins + 1, (int)(k2max + 1));
    {
        int b_prev = -1;
        for (long long k2 = 1; k2 <= k2max; k2++) {
            int b = (int)floor(bpu * log(sqrt((double)k2)));
            if (b < 0) b = 0;
            if (b > nrbins - 1) b = nrbins - 1;
            NEED(b >= b_prev, KSPACE_ERR_ARG);  // monotone (always true for a monotone log)
            for (int bb = b_prev + 1; bb <= b; bb++) thr[bb] = (int)k2;
            b_prev = b;
        }
        thr[0] = 1;
    }
    // full-grid mode histogram over k^2 -> counts and sum |k| per bin
    unsigned long long* hist_d = nullptr;
    CK(dalloc(&hist_d, k2max + 1));
    CK(cudaMemsetAsync(hist_d, 0, sizeof(unsigned long long) * (k2max + 1), c->stream));
    launch_k2_histogram(N, 0, N, hist_d, c->stream);
    g_launches += 1;
    std::vector<unsigned long long> hist(k2max + 1);
    CK(cudaMemcpyAsync(hist.data(), hist_d, sizeof(unsigned long long) * (k2max + 1), cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    cudaFree(hist_d);
    G.count.assign(nrbins, 0);
    G.ksum.assign(nrbins, 0.0);
    {
        int b = 0;
        for (long long k2 = 1; k2 <= k2max; k2++) {
            while (b < nrbins - 1 && k2 >= thr[b + 1]) b++;
            if (hist[k2]) {
                G.count[b] += (long long)hist[k2];
                G.ksum[b] += (double)hist[k2] * sqrt((double)k2);
            }
        }
    }
    std::vector<int> cmap(nrbins, -1);
    for (int b = 0; b < nrbins; b++)
        if (G.count[b]) {
            cmap[b] = (int)G.compact.size();
            G.compact.push_back(b);
        }
    G.nk = (int)G.compact.size();
    // 1-D inverse window in float (powerspectrum.c:8-12)
    std::vector<float> w1(nz);
    for (int k = 0; k < nz; k++)
        w1[k] = k ? (float)(kPi * k / (N * sin(kPi * k / (float)N))) : 1.0f;
    GridGeom& g = G.g;
    g.N = N;
    g.nrbins = nrbins;
    g.bin_c1 = (float)(bpu * 0.5 * log(2.0));
    CK(dalloc(&g.thresh, nrbins + 1));
    CK(dalloc(&g.w1, nz));
    CK(dalloc(&g.cmap, nrbins));
    CK(dalloc(&G.count_d, nrbins));
    CK(dalloc(&G.ksum_d, nrbins));
    CK(dalloc(&G.compact_d, G.nk));
    CK(cudaMemcpy(g.thresh, thr.data(), sizeof(int) * (nrbins + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(g.w1, w1.data(), sizeof(float) * nz, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(g.cmap, cmap.data(), sizeof(int) * nrbins, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(G.count_d, G.count.data(), sizeof(long long) * nrbins, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(G.ksum_d, G.ksum.data(), sizeof(double) * nrbins, cudaMemcpyHostToDevice));
    if (G.nk) CK(cudaMemcpy(G.compact_d, G.compact.data(), sizeof(int) * G.nk, cudaMemcpyHostToDevice));
    if (build_run_table(g, c->stream) < 0) return KSPACE_ERR_CUDA;
    g_launches += g.runtab ? 1 : 0;
    c->geos[key] = G;
    *out = &c->geos[key];
    return KSPACE_OK;
}

// Device pointer for the grid: the caller's device memory, or the staging buffer after
// a host->device copy.
static int stage_alloc(kspace_ctx* c, size_t bytes) {
    if (c->stage_bytes < bytes) {
        if (c->stage_d) cudaFree(c->stage_d);
        c->stage_d = nullptr;
        c->stage_bytes = 0;
        CK(cudaMalloc(&c->stage_d, bytes));
        c->stage_bytes = bytes;
    }
    return KSPACE_OK;
}

static int grid_in(kspace_ctx* c, const void* grid, size_t bytes, float** gd, bool* staged) {
    if (is_device_ptr(grid)) {
        *gd = const_cast<float*>(reinterpret_cast<const float*>(grid));
        *staged = false;
        return KSPACE_OK;
    }
    const int st = stage_alloc(c, bytes);
    if (st) return st;
    CK(cudaMemcpyAsync(c->stage_d, grid, bytes, cudaMemcpyHostToDevice, c->stream));
    *gd = reinterpret_cast<float*>(c->stage_d);
    *staged = true;
    return KSPACE_OK;
}

// Slab chunks of a host grid: chunk k covers local slabs [first[k], first[k+1]).
struct SlabChunks {
    int n = 0;
    int first[kspace_ctx::kChunks + 1];
    size_t slab_bytes = 0;
};
static SlabChunks make_chunks(int nslab, int pmgrid, int want) {
    SlabChunks ch;
    want = want < 1 ? 1 : (want > kspace_ctx::kChunks ? kspace_ctx::kChunks : want);
    ch.n = nslab < want ? (nslab > 0 ? nslab : 1) : want;
    for (int k = 0; k <= ch.n; k++) ch.first[k] = (int)((long long)nslab * k / ch.n);
    ch.slab_bytes = sizeof(float) * 2 * (size_t)pmgrid * (pmgrid / 2 + 1);
    return ch;
}

// The integrator work that does not depend on this step's delta_cdm (scalars, knot
// factorisation, fslength and node tables), on the side stream beside the binning pass;
// update_device waits for it.  Only for the common case: a new scale factor on an
// initialised table with room for the provisional row.  Queued after the binning pass
// (but ordered only after ev_fork, recorded before it), so that the device starts on
// the grid without waiting for these launches.
static int start_prep(kspace_ctx* c, const Geo* G, double Time) {
    c->prep_valid = false;
    if (!(c->init_done && c->ia >= 1 && c->ia < c->I.namax && G->nk == c->nk && c->nk >= 2)) return KSPACE_OK;
    const double loga = log(Time);
    if (loga - c->h_scalefact[c->ia - 1] < kFloatAcc) return KSPACE_OK;
    const int Na = c->ia + 1;
    CK(cudaStreamWaitEvent(c->side, c->ev_fork, 0));  // recorded before the binning pass
    launch_integrator_prepare(c->I, Na, Time, loga, c->loga0, c->TimeTransfer, c->fact_valid, 1, false, c->side);
    c->prep_base = launch_dtot_base(c->I, c->nk, Na, c->side);
    CK(cudaEventRecord(c->ev_join, c->side));
    g_launches += c->prep_base ? 6 : 5;
    c->prep_valid = true;
    c->prep_Na = Na;
    c->prep_loga = loga;
    return KSPACE_OK;
}

// K1 + allreduce + normalisation into compacted arrays (device): power, keff (grid
// units), dcdm and keff (physical) for the integrator.  prep_time > 0: start the
// integrator's preparation for that scale factor once the binning pass is queued.
static int bin_grid(kspace_ctx* c, Geo* G, const float* gd, int pmgrid, int slab0, int nslab, double BoxSize,
                    const SlabChunks* ch = nullptr, double prep_time = 0) {
    NEED(c->table_ready && c->buf_nb >= G->g.nrbins, KSPACE_ERR_ORDER);
    const int nb = G->g.nrbins;
    G->g.slab0 = slab0;
    G->g.nslab = nslab;
    G->g.nmodes = (long long)nslab * pmgrid * (pmgrid / 2 + 1);
    CK(cudaMemsetAsync(c->bin_sum_d, 0, sizeof(double) * (nb + 1), c->stream));
    c->F0sq_d = c->bin_sum_d + nb;
    if (c->prof) cudaEventRecord(c->ev[0], c->stream);
    if (!ch) {
        if (launch_bin_power(G->g, gd, c->bin_sum_d, c->F0sq_d, c->status_d, c->tma, c->rows, c->stages,
                             c->stream) < 0)
            return KSPACE_ERR_CUDA;
        g_launches += 1;
    } else {
        // each chunk as soon as its upload has landed
        for (int k = 0; k < ch->n; k++) {
            GridGeom gk = G->g;
            gk.slab0 = slab0 + ch->first[k];
            gk.nslab = ch->first[k + 1] - ch->first[k];
            gk.nmodes = (long long)gk.nslab * pmgrid * (pmgrid / 2 + 1);
            CK(cudaStreamWaitEvent(c->stream, c->ev_up[k], 0));
            if (gk.nslab > 0 &&
                launch_bin_power(gk, gd + (ch->first[k] * ch->slab_bytes) / sizeof(float), c->bin_sum_d, c->F0sq_d,
                                 c->status_d, c->tma, c->rows, c->stages, c->stream) < 0)
                return KSPACE_ERR_CUDA;
            g_launches += 1;
        }
    }
    if (c->prof) cudaEventRecord(c->ev[1], c->stream);
    if (prep_time > 0) {
        const int sp = start_prep(c, G, prep_time);
        if (sp) return sp;
    }
    if (c->ar_fn) {
        CK(cudaMemcpyAsync(c->ar_h, c->bin_sum_d, sizeof(double) * (nb + 1), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (c->ar_fn(c->ar_h, nb + 1, c->ar_user) != 0) return KSPACE_ERR_ARG;
        CK(cudaMemcpyAsync(c->bin_sum_d, c->ar_h, sizeof(double) * (nb + 1), cudaMemcpyHostToDevice, c->stream));
    }
    c->fin = FinalizeArgs{c->bin_sum_d, c->F0sq_d, G->count_d, G->ksum_d, G->compact_d, BoxSize, c->power_d,
                          c->keffg_d, c->I.dcdm, c->keff_d, 1};
    c->fin.scale = pow(BoxSize, -3.0);
    c->fin.kfac = 2 * kPi / BoxSize;
    if (!(prep_time > 0 && c->prep_valid)) {
        // a prepared step does it in its row-spline kernel instead (update_device)
        launch_finalize_power(c->bin_sum_d, c->F0sq_d, G->count_d, G->ksum_d, G->compact_d, G->nk, BoxSize,
                              c->power_d, c->keffg_d, c->I.dcdm, c->keff_d, c->stream);
        g_launches += 1;
        c->fin.active = 0;
    }
    return KSPACE_OK;
}

extern "C" int kspace_gpu_total_powerspectrum(kspace_ctx* c, int dims, const void* grid, int nrbins, int startslab,
                                              int nslab, double* power, long long* count, double* keffs, int* nk_out) {
    NEED(c && grid && power && count && keffs && nrbins > 1, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    NEED(nrbins <= c->buf_nb, KSPACE_ERR_NK_ALLOC);
    Geo* G = nullptr;
    int st = get_geo(c, dims, nrbins, &G);
    if (st) return st;
    const size_t bytes = sizeof(float) * 2 * (size_t)nslab * dims * (dims / 2 + 1);
    float* gd;
    bool staged;
    st = grid_in(c, grid, bytes, &gd, &staged);
    if (st) return st;
    st = bin_grid(c, G, gd, dims, startslab, nslab, 1.0);
    if (st) return st;
    st = sync_status(c);
    if (st) return st;
    CK(cudaMemcpy(power, c->power_d, sizeof(double) * G->nk, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(keffs, c->keffg_d, sizeof(double) * G->nk, cudaMemcpyDeviceToHost));
    for (int i = 0; i < G->nk; i++) count[i] = G->count[G->compact[i]];
    // like the reference: entries beyond nk keep the pre-compaction values; we zero them
    for (int i = G->nk; i < nrbins; i++) {
        power[i] = 0;
        keffs[i] = 0;
        count[i] = 0;
    }
    if (nk_out) *nk_out = G->nk;
    return KSPACE_OK;
}

static int correct_grid(kspace_ctx* c, Geo* G, float* gd, double BoxSize, int nk, const SlabChunks* ch = nullptr,
                        void* host = nullptr) {
    CorrTable corr = c->corr;
    corr.nk = nk;
    const float lnscale = (float)log(2 * kPi / BoxSize);
    if (c->prof) cudaEventRecord(c->ev[2], c->stream);
    if (!ch) {
        if (launch_apply_correction(G->g, gd, corr, lnscale, c->status_d, c->tma, c->rows, c->stages, c->stream) < 0)
            return KSPACE_ERR_CUDA;
        g_launches += 1;
    } else {
        // each chunk goes back to the host while the next one is corrected
        for (int k = 0; k < ch->n; k++) {
            GridGeom gk = G->g;
            gk.slab0 = G->g.slab0 + ch->first[k];
            gk.nslab = ch->first[k + 1] - ch->first[k];
            gk.nmodes = (long long)gk.nslab * G->g.N * (G->g.N / 2 + 1);
            const size_t off = ch->first[k] * ch->slab_bytes, len = (size_t)gk.nslab * ch->slab_bytes;
            if (gk.nslab > 0 && launch_apply_correction(gk, gd + off / sizeof(float), corr, lnscale, c->status_d,
                                                        c->tma, c->rows, c->stages, c->stream) < 0)
                return KSPACE_ERR_CUDA;
            g_launches += 1;
            CK(cudaEventRecord(c->ev_done[k], c->stream));
            CK(cudaStreamWaitEvent(c->copy, c->ev_done[k], 0));
            if (len)
                CK(cudaMemcpyAsync(reinterpret_cast<char*>(host) + off, reinterpret_cast<char*>(gd) + off, len,
                                   cudaMemcpyDeviceToHost, c->copy));
        }
        CK(cudaEventRecord(c->ev_copy_end, c->copy));
        CK(cudaStreamWaitEvent(c->stream, c->ev_copy_end, 0));
    }
    if (c->prof) cudaEventRecord(c->ev[3], c->stream);
    return KSPACE_OK;
}

extern "C" int kspace_gpu_add_nu_power_to_rhogrid(kspace_ctx* c, double Time, double BoxSize, void* grid, int pmgrid,
                                                  int slab0, int nslab) {
    NEED(c && grid && pmgrid > 1 && nslab >= 0, KSPACE_ERR_ARG);
    NEED(c->table_ready && c->hubble_ready, KSPACE_ERR_ORDER);
    CK(cudaSetDevice(c->device));
    Geo* G = nullptr;
    int st = get_geo(c, pmgrid, c->I.nk_alloc, &G);
    if (st) return st;
    if (c->prof) cudaEventRecord(c->ev[4], c->stream);
    const size_t bytes = sizeof(float) * 2 * (size_t)nslab * pmgrid * (pmgrid / 2 + 1);
    float* gd;
    const bool staged = !is_device_ptr(grid);
    SlabChunks ch;
    if (staged) {
        // a host grid: upload in slab chunks on the copy stream (after the work queued so
        // far on the context's stream, which may still read the staging buffer)
        st = stage_alloc(c, bytes);
        if (st) return st;
        gd = reinterpret_cast<float*>(c->stage_d);
        ch = make_chunks(nslab, pmgrid, c->chunks);
        CK(cudaEventRecord(c->ev_copy_start, c->stream));
        CK(cudaStreamWaitEvent(c->copy, c->ev_copy_start, 0));
        for (int k = 0; k < ch.n; k++) {
            const size_t off = ch.first[k] * ch.slab_bytes, len = (size_t)(ch.first[k + 1] - ch.first[k]) * ch.slab_bytes;
            if (len)
                CK(cudaMemcpyAsync(reinterpret_cast<char*>(gd) + off, reinterpret_cast<const char*>(grid) + off, len,
                                   cudaMemcpyHostToDevice, c->copy));
            CK(cudaEventRecord(c->ev_up[k], c->copy));
        }
    } else {
        gd = reinterpret_cast<float*>(grid);
    }
    // compute_neutrino_power_spectrum (interface_gadget.c:75-102); the integrator's
    // delta_cdm-independent work starts beside the binning pass (start_prep), after the
    // work queued so far on the context's stream
    c->prep_valid = false;
    CK(cudaEventRecord(c->ev_fork, c->stream));
    st = bin_grid(c, G, gd, pmgrid, slab0, nslab, BoxSize, staged ? &ch : nullptr, Time);
    if (st) return st;
    // the integrator (interface_common.c:125-148), then the multiply (interface_gadget.c:
    // 163-188) on the same stream without a host round trip: an error of the integrator
    // leaves the grid as it is (the correction kernels read the status word) and comes
    // back from the status check below
    st = update_device(c, Time, G->nk, c->keff_d, c->I.dcdm, c->dnu_out_d, true, c->fin.active ? &c->fin : nullptr,
                       false);
    c->fin.active = 0;
    if (st) return st;
    st = correct_grid(c, G, gd, BoxSize, G->nk, staged ? &ch : nullptr, staged ? grid : nullptr);
    if (st) return st;
    st = sync_status(c);
    if (st == KSPACE_OK) {
        c->last_nk = G->nk;
        c->last_BoxSize = BoxSize;
    }
    if (c->prof) {
        cudaEventElapsedTime(&c->stage_ms[0], c->ev[0], c->ev[1]);
        cudaEventElapsedTime(&c->stage_ms[1], c->ev[1], c->ev[2]);
        cudaEventElapsedTime(&c->stage_ms[2], c->ev[2], c->ev[3]);
        cudaEventElapsedTime(&c->stage_ms[3], c->ev[4], c->ev[3]);
    }
    return st;
}

extern "C" int kspace_gpu_apply_delta_pow(kspace_ctx* c, double BoxSize, void* grid, int pmgrid, int slab0, int nslab,
                                          int nrbins, const double* logk, const double* ratio, int nk, double norm) {
    NEED(c && grid && logk && ratio && nk >= 2, KSPACE_ERR_ARG);
    NEED(c->table_ready && nk <= c->buf_nb, KSPACE_ERR_ORDER);
    Geo* G = nullptr;
    int st = get_geo(c, pmgrid, nrbins, &G);
    if (st) return st;
    NEED(nk == G->nk, KSPACE_ERR_NK_MISMATCH);
    // host-built float table (same formula as k_finish)
    std::vector<float> xf(nk), rn(nk), sn(nk);
    for (int j = 0; j < nk; j++) {
        xf[j] = (float)logk[j];
        rn[j] = (float)(norm * ratio[j]);
        sn[j] = j + 1 < nk ? (float)(norm * (ratio[j + 1] - ratio[j]) / (logk[j + 1] - logk[j])) : 0.f;
        if (!isfinite(norm * ratio[j]) || !isfinite((double)sn[j])) return KSPACE_ERR_GRID_NAN;
    }
    CK(cudaMemcpyAsync(c->corr.xf, xf.data(), sizeof(float) * nk, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->corr.rn, rn.data(), sizeof(float) * nk, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->corr.sn, sn.data(), sizeof(float) * nk, cudaMemcpyHostToDevice, c->stream));
    G->g.slab0 = slab0;
    G->g.nslab = nslab;
    G->g.nmodes = (long long)nslab * pmgrid * (pmgrid / 2 + 1);
    const size_t bytes = sizeof(float) * 2 * (size_t)G->g.nmodes;
    float* gd;
    bool staged;
    st = grid_in(c, grid, bytes, &gd, &staged);
    if (st) return st;
    st = correct_grid(c, G, gd, BoxSize, nk);
    if (st) return st;
    if (staged) CK(cudaMemcpyAsync(grid, gd, bytes, cudaMemcpyDeviceToHost, c->stream));
    return sync_status(c);
}

// compute_neutrino_power_from_cdm (interface_common.c:106-123)
extern "C" int kspace_gpu_compute_neutrino_power_from_cdm(kspace_ctx* c, double Time, const double* keff_in,
                                                          const double* P_cdm, const long* Nmodes, int nk_in,
                                                          double* logk, double* ratio, double* norm, int* nbins) {
    NEED(c && keff_in && P_cdm && Nmodes, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    std::vector<double> kk, dc;
    for (int i = 0; i < nk_in; i++) {
        if (Nmodes[i] == 0) continue;
        dc.push_back(sqrt(P_cdm[i]));
        kk.push_back(keff_in[i]);
    }
    const int nk = (int)kk.size();
    NEED(nk <= c->I.nk_alloc, KSPACE_ERR_NK_ALLOC);
    double* kd = c->io_d;
    double* dd = c->io_d + c->I.nk_alloc;
    if (nk) {
        CK(cudaMemcpyAsync(kd, kk.data(), sizeof(double) * nk, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(dd, dc.data(), sizeof(double) * nk, cudaMemcpyHostToDevice, c->stream));
    }
    int st = update_device(c, Time, nk, kd, dd, c->dnu_out_d, true);
    if (st) return st;
    if (logk) CK(cudaMemcpy(logk, c->logk_d, sizeof(double) * nk, cudaMemcpyDeviceToHost));
    if (ratio) CK(cudaMemcpy(ratio, c->ratio_d, sizeof(double) * nk, cudaMemcpyDeviceToHost));
    if (norm) CK(cudaMemcpy(norm, c->norm_d, sizeof(double), cudaMemcpyDeviceToHost));
    if (nbins) *nbins = nk;
    c->last_nk = nk;
    return KSPACE_OK;
}

// compute_total_power_spectrum (interface_gadget.c:114-144): binning into pmgrid/2 bins
// for runs without the integrator (gadget-2 patch 0004 calls it without InitOmegaNu or
// allocate_kspace_memory: a context with neither gets bin buffers of its own); saved
// by kspace_gpu_save_total_power.
extern "C" int kspace_gpu_compute_total_power_spectrum(kspace_ctx* c, double Time, double BoxSize, const void* grid,
                                                       int pmgrid, int slab0, int nslab) {
    (void)Time;
    NEED(c && grid && pmgrid > 1, KSPACE_ERR_ARG);
    if (!c->table_ready) {
        // buffers only: a background without neutrinos and a table of pmgrid/2 bins
        int st = KSPACE_OK;
        if (!c->bg_ready) {
            const double zero[3] = {0, 0, 0};
            st = kspace_gpu_init_omega_nu(c, zero, 0.01, 0.7, 2.7255);
        }
        if (!st) st = kspace_gpu_alloc_table(c, pmgrid / 2, 0.01, 1.0, 0.3, 1.0, 1.0);
        if (st) return st;
    }
    const int nrbins = pmgrid / 2;
    NEED(nrbins <= c->buf_nb, KSPACE_ERR_NK_ALLOC);
    Geo* G = nullptr;
    int st = get_geo(c, pmgrid, nrbins, &G);
    if (st) return st;
    const size_t bytes = sizeof(float) * 2 * (size_t)nslab * pmgrid * (pmgrid / 2 + 1);
    float* gd;
    bool staged;
    st = grid_in(c, grid, bytes, &gd, &staged);
    if (st) return st;
    st = bin_grid(c, G, gd, pmgrid, slab0, nslab, BoxSize);
    if (st) return st;
    c->last_nk = G->nk;
    c->last_BoxSize = BoxSize;
    CK(cudaMemsetAsync(c->ratio_d, 0, sizeof(double) * G->nk, c->stream));
    c->init_done = c->init_done;  // the integrator state is untouched
    return sync_status(c);
}

// save_total_power (interface_gadget.c:196-224): k and the total power of the last
// binned grid; with the integrator active the total is get_delta_tot of delta_nu_last.
extern "C" int kspace_gpu_save_total_power(kspace_ctx* c, double Time, int snapnum, const char* dir) {
    NEED(c && dir, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    char fname[1000];
    snprintf(fname, sizeof(fname), "%s/powerspec_tot_%03d.txt", dir, snapnum);
    FILE* fd = fopen(fname, "w");
    if (!fd) {
        fprintf(stderr, "can't open file `%s` for writing\n", fname);
        return -1;
    }
    const int n = c->last_nk;
    std::vector<double> keff(n > 0 ? n : 1), dcdm(n > 0 ? n : 1), last(c->I.nk_alloc);
    CK(cudaStreamSynchronize(c->stream));
    if (n) {
        CK(cudaMemcpy(keff.data(), c->keff_d, sizeof(double) * n, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(dcdm.data(), c->I.dcdm, sizeof(double) * n, cudaMemcpyDeviceToHost));
    }
    CK(cudaMemcpy(last.data(), c->I.nu_last, sizeof(double) * c->I.nk_alloc, cudaMemcpyDeviceToHost));
    const Background& B = c->hB;
    const double OmegaNua3 = omega_nu_nopart(B, Time) * pow(Time, 3);
    const double OmegaNu1 = omega_nu(B, 1);
    const double partnu = particle_nu_fraction(B, Time, 0);
    double Omeganonu;
    StepScalars S;
    CK(cudaMemcpy(&S, c->I.sc, sizeof(S), cudaMemcpyDeviceToHost));
    Omeganonu = S.Omeganonu;
    fprintf(fd, "# k P_nu(k)\n");
    fprintf(fd, "# a = %g\n", Time);
    fprintf(fd, "# nbins = %d\n", n);
    for (int i = 0; i < n; i++) {
        if (c->init_done) {
            // a neutrino run (the library built with KSPACE_NEUTRINOS_2, interface_gadget.c:215-216)
            const double d_tot = get_delta_tot(last[i], dcdm[i], OmegaNua3, Omeganonu, OmegaNu1, partnu);
            fprintf(fd, "%g %g\n", keff[i], d_tot * d_tot);
        } else {
            // without the integrator (interface_gadget.c:218): the k column is what the
            // reference writes, exp(log(delta_cdm * 2 pi / BoxSize)): there its keff and
            // delta_cdm_last share storage (3/2*pmgrid == pmgrid in integer arithmetic,
            // :118-119), so the stored log k is overwritten with log(delta_cdm 2 pi / L)
            const double kq = exp(log(dcdm[i] * 2 * kPi / c->last_BoxSize));
            fprintf(fd, "%g %g\n", kq, dcdm[i] * dcdm[i]);
        }
    }
    fclose(fd);
    return 0;
}

// ------------------------------------------------------------------ diagnostics
extern "C" int kspace_gpu_last_correction(kspace_ctx* c, int* nk, double* logk, double* ratio, double* norm,
                                          double* dcdm, double* keff) {
    NEED(c, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    CK(cudaStreamSynchronize(c->stream));
    const int n = c->last_nk;
    if (nk) *nk = n;
    if (n <= 0) return KSPACE_OK;
    if (logk) CK(cudaMemcpy(logk, c->logk_d, sizeof(double) * n, cudaMemcpyDeviceToHost));
    if (ratio) CK(cudaMemcpy(ratio, c->ratio_d, sizeof(double) * n, cudaMemcpyDeviceToHost));
    if (norm) CK(cudaMemcpy(norm, c->norm_d, sizeof(double), cudaMemcpyDeviceToHost));
    if (dcdm) CK(cudaMemcpy(dcdm, c->I.dcdm, sizeof(double) * n, cudaMemcpyDeviceToHost));
    if (keff) CK(cudaMemcpy(keff, c->keff_d, sizeof(double) * n, cudaMemcpyDeviceToHost));
    return KSPACE_OK;
}

extern "C" int kspace_gpu_set_profiling(kspace_ctx* c, int on) {
    NEED(c, KSPACE_ERR_ARG);
    c->prof = on != 0;
    return KSPACE_OK;
}

extern "C" int kspace_gpu_stage_times(kspace_ctx* c, float* ms4) {
    NEED(c && ms4, KSPACE_ERR_ARG);
    for (int i = 0; i < 4; i++) ms4[i] = c->stage_ms[i];
    return KSPACE_OK;
}

extern "C" int kspace_gpu_qag_stats(kspace_ctx* c, int* mx, long long* tot) {
    NEED(c, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    CK(cudaStreamSynchronize(c->stream));
    int m = 0;
    long long t = 0;
    CK(cudaMemcpy(&m, c->I.qag_max, sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&t, c->I.qag_total, sizeof(long long), cudaMemcpyDeviceToHost));
    if (mx) *mx = m;
    if (tot) *tot = t;
    return KSPACE_OK;
}

// ------------------------------------------------------------------ differentiable step
extern "C" int kspace_gpu_set_vectors(kspace_ctx* c, const double* nu_init, const double* nu_last,
                                      const double* wavenum, int nk) {
    NEED(c && nu_init && nu_last && wavenum, KSPACE_ERR_ARG);
    NEED(c->table_ready, KSPACE_ERR_ORDER);
    NEED(nk <= c->I.nk_alloc && nk > 0, KSPACE_ERR_NK_ALLOC);
    CK(cudaMemcpyAsync(c->I.nu_init, nu_init, sizeof(double) * nk, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->I.nu_last, nu_last, sizeof(double) * nk, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->I.wavenum, wavenum, sizeof(double) * nk, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->nk = nk;
    c->init_done = 1;
    return KSPACE_OK;
}

extern "C" int kspace_gpu_set_jmass(kspace_ctx* c, const double* MNu) {
    NEED(c, KSPACE_ERR_ARG);
    NEED(c->bg_ready, KSPACE_ERR_ORDER);
    for (int i = 0; i < kNuSpecies; i++) c->hB.mnu_J[i] = MNu ? MNu[i] : c->hB.mnu[i];
    CK(cudaMemcpyAsync(&c->dB->mnu_J[0], &c->hB.mnu_J[0], sizeof(double) * kNuSpecies, cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return KSPACE_OK;
}

__global__ void k_square(const double* v, double* out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = v[i] * v[i];
}

static int ensure_adj_buffers(kspace_ctx* c, int nrbins) {
    const size_t nk = c->I.nk_alloc, ld = c->I.ld;
    if (!c->ivals_d) {
        CK(dalloc(&c->ivals_d, (size_t)kNuSpecies * nk * kQagLimit * 2));
        CK(dalloc(&c->nivals_d, (size_t)kNuSpecies * nk));
        CK(dalloc(&c->adj_node_d, nk));
        CK(dalloc(&c->adj_Dbar_d, nk * ld));
        CK(dalloc(&c->adj_mbar_d, kNuSpecies));
        CK(dalloc(&c->adj_dcsum_d, 1));
        CK(dalloc(&c->adj_dnubar_d, nk));
        CK(dalloc(&c->adj_rbar_d, nk));
    }
    if (c->adj_cap_nb < nrbins) {
        if (c->adj_Q_d) cudaFree(c->adj_Q_d);
        CK(dalloc(&c->adj_Q_d, nrbins));
        c->adj_cap_nb = nrbins;
    }
    return KSPACE_OK;
}

// One step at `Time` with the integrator state held fixed (interface_gadget.c:158-194
// without the state update): grid_out = grid_in * (1 + correction); pnu_out = delta_nu^2.
// Device pointers only.  store_intervals keeps every QAG subdivision for the adjoint.
extern "C" int kspace_gpu_diff_forward(kspace_ctx* c, double Time, double BoxSize, const void* grid_in,
                                       void* grid_out, int pmgrid, double* pnu_out, int store_intervals) {
    NEED(c && grid_in && grid_out && pnu_out, KSPACE_ERR_ARG);
    NEED(c->table_ready && c->hubble_ready && c->init_done, KSPACE_ERR_ORDER);
    NEED(is_device_ptr(grid_in) && is_device_ptr(grid_out) && is_device_ptr(pnu_out), KSPACE_ERR_ARG);
    Geo* G = nullptr;
    int st = get_geo(c, pmgrid, c->I.nk_alloc, &G);
    if (st) return st;
    st = ensure_adj_buffers(c, G->g.nrbins);
    if (st) return st;
    st = bin_grid(c, G, reinterpret_cast<const float*>(grid_in), pmgrid, 0, pmgrid, BoxSize);
    if (st) return st;
    if (G->nk != c->nk) return KSPACE_ERR_NK_MISMATCH;
    if (c->ia >= c->I.namax) return KSPACE_ERR_NAMAX;
    IntegratorDev& I = c->I;
    const double loga = log(Time);
    launch_update_row(I, c->nk, c->ia, Time, loga, I.dcdm, I.nu_last, c->stream);
    const int Na = c->ia + 1;
    int start = c->fact_valid < Na - 3 ? c->fact_valid : Na - 3;
    if (start < 0) start = 0;
    IntegratorDev Is = I;
    if (store_intervals) {
        Is.ivals = c->ivals_d;
        Is.nivals = c->nivals_d;
    }
    CK(cudaMemsetAsync(I.qag_max, 0, sizeof(int), c->stream));
    CK(cudaMemsetAsync(I.qag_total, 0, sizeof(long long), c->stream));
    launch_delta_nu_combined(Is, c->nk, Na, Time, loga, c->loga0, c->TimeTransfer, start, c->nspec, c->spec_ids,
                             c->qag_warps, c->stream, c->qag_split);
    c->fact_valid = start;
    launch_finish_update(I, c->nk, -3, Time, loga, c->keff_d, c->dnu_out_d, c->logk_d, c->ratio_d, c->corr,
                         c->norm_d, c->stream);
    k_square<<<(c->nk + 127) / 128, 128, 0, c->stream>>>(c->dnu_out_d, pnu_out, c->nk);
    g_launches += 11;
    const size_t bytes = sizeof(float) * 2 * (size_t)pmgrid * pmgrid * (pmgrid / 2 + 1);
    if (grid_out != grid_in) CK(cudaMemcpyAsync(grid_out, grid_in, bytes, cudaMemcpyDeviceToDevice, c->stream));
    st = correct_grid(c, G, reinterpret_cast<float*>(grid_out), BoxSize, c->nk);
    if (st) return st;
    st = sync_status(c);
    if (st) return st;
    c->diff_ready = true;
    c->diff_ia = c->ia;
    c->diff_Na = Na;
    c->diff_nk = c->nk;
    c->diff_time = Time;
    c->diff_box = BoxSize;
    c->diff_store = store_intervals;
    c->diff_pmgrid = pmgrid;
    c->diff_gen++;
    c->last_nk = c->nk;
    c->last_BoxSize = BoxSize;
    return KSPACE_OK;
}

// The number of successful diff_forward calls on the context so far: the generation a
// diff_backward must name.
extern "C" int kspace_gpu_diff_generation(kspace_ctx* c, long long* generation) {
    NEED(c && generation, KSPACE_ERR_ARG);
    *generation = c->diff_gen;
    return KSPACE_OK;
}

// Adjoint of the last kspace_gpu_diff_forward (no other call in between).  generation:
// the value kspace_gpu_diff_generation gave right after that forward; a later forward
// on the same context replaces the state the adjoint reads, and the call is refused
// (KSPACE_ERR_ORDER) instead of returning the later step's gradients.
//   gbar_out: dL/d grid_out (device c64), grid_in: the forward's input (device),
//   pnu_bar: dL/dP_nu (device, nk), gbar_in: out dL/d grid_in (device c64),
//   Dbar: out dL/d history (device, [nk][ia] of the current table), mbar: out
//   dL/dm per mass state (host, 3; through the free-streaming argument of J),
//   recompute: 1 = re-run every QAG instead of reading the stored subdivisions.
extern "C" int kspace_gpu_diff_backward(kspace_ctx* c, const void* gbar_out, const void* grid_in,
                                        const double* pnu_bar, void* gbar_in, double* Dbar, double* mbar,
                                        int recompute, long long generation) {
    NEED(c && gbar_out && grid_in && pnu_bar && gbar_in, KSPACE_ERR_ARG);
    NEED(c->diff_ready && generation == c->diff_gen, KSPACE_ERR_ORDER);
    NEED(recompute || c->diff_store, KSPACE_ERR_ORDER);
    Geo* G = nullptr;
    int st = get_geo(c, c->diff_pmgrid, c->I.nk_alloc, &G);
    if (st) return st;
    IntegratorDev& I = c->I;
    const int nk = c->diff_nk, Na = c->diff_Na;
    const double a = c->diff_time, L = c->diff_box;
    CK(cudaMemsetAsync(c->adj_node_d, 0, sizeof(double) * nk, c->stream));
    CK(cudaMemsetAsync(c->adj_Dbar_d, 0, sizeof(double) * (size_t)I.nk_alloc * I.ld, c->stream));
    CK(cudaMemsetAsync(c->adj_mbar_d, 0, sizeof(double) * kNuSpecies, c->stream));
    CK(cudaMemsetAsync(c->adj_Q_d, 0, sizeof(double) * G->g.nrbins, c->stream));
    CorrTable corr = c->corr;
    corr.nk = nk;
    const float lnscale = (float)log(2 * kPi / L);
    G->g.slab0 = 0;
    G->g.nslab = c->diff_pmgrid;
    G->g.nmodes = (long long)c->diff_pmgrid * c->diff_pmgrid * (c->diff_pmgrid / 2 + 1);
    launch_adj_reduce(G->g, corr, lnscale, reinterpret_cast<const float*>(gbar_out),
                      reinterpret_cast<const float*>(grid_in), c->adj_node_d, c->stream);
    const Background& B = c->hB;
    const double OmegaNua3 = omega_nu_nopart(B, a) * (a * a * a);
    const double OmegaNu1 = omega_nu(B, 1);
    const double OmegaNu_nop = omega_nu_nopart(B, a);
    const double norm = OmegaNu_nop / (c->Omeganonu / (a * a * a) + (omega_nu(B, a) - OmegaNu_nop));
    AdjBinsHost h;
    h.node_sum = c->adj_node_d;
    h.pnu_bar = pnu_bar;
    h.dnu = I.dnu;
    h.dcdm = I.dcdm;
    h.power = c->power_d;
    h.count = G->count_d;
    h.compact = G->compact_d;
    h.F0sq = c->F0sq_d;
    h.dnu_bar = c->adj_dnubar_d;
    h.dprov_bar = c->adj_Dbar_d + (Na - 1);  // provisional column, stride ld
    h.rbar = c->adj_rbar_d;
    h.Q = c->adj_Q_d;
    h.dc_sum = c->adj_dcsum_d;
    h.norm = norm;
    h.L3 = L * L * L;
    h.fcdm = 1 - OmegaNua3 / (c->Omeganonu + OmegaNu1);
    h.nk = nk;
    h.ld = I.ld;
    launch_adj_bins(h, c->stream);
    launch_dnu_adj(I, c->adj_dnubar_d, c->adj_Dbar_d, c->adj_mbar_d, c->ivals_d, c->nivals_d, recompute, nk, Na,
                   c->nspec, c->spec_ids, c->qag_warps, c->stream);
    launch_adj_bins2(h, c->stream);
    launch_adj_grid(G->g, corr, lnscale, reinterpret_cast<const float*>(gbar_out),
                    reinterpret_cast<const float*>(grid_in), reinterpret_cast<float*>(gbar_in), c->adj_Q_d,
                    c->adj_dcsum_d, c->F0sq_d, c->stream);
    g_launches += 5;
    if (Dbar && Na > 1)
        CK(cudaMemcpy2DAsync(Dbar, sizeof(double) * (Na - 1), c->adj_Dbar_d, sizeof(double) * I.ld,
                             sizeof(double) * (Na - 1), nk, cudaMemcpyDeviceToDevice, c->stream));
    if (mbar) CK(cudaMemcpyAsync(mbar, c->adj_mbar_d, sizeof(double) * kNuSpecies, cudaMemcpyDeviceToHost, c->stream));
    return sync_status(c);
}

// ------------------------------------------------------------------ shared with the batch ABI
int ksp::ctx_delta_tot_init(kspace_ctx* c, int nk_in, const double* keff_d, const double* dcdm_d, double Time) {
    return delta_tot_init(c, nk_in, keff_d, dcdm_d, Time);
}
int ksp::ctx_get_geo(kspace_ctx* c, int N, int nrbins, Geo** out) { return get_geo(c, N, nrbins, out); }
int ksp::ctx_bin_grid(kspace_ctx* c, Geo* G, const float* gd, int pmgrid, int slab0, int nslab, double BoxSize) {
    return bin_grid(c, G, gd, pmgrid, slab0, nslab, BoxSize);
}
int ksp::ctx_sync_status(kspace_ctx* c) { return sync_status(c); }
