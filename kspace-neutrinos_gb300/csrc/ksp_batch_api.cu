// ksp_batch_api.cu -- host side of the batch ABI (kspace_gpu_batch_*).
//
// The bookkeeping of every instance (which history row is provisional, whether it is
// committed, the same-scale-factor shortcut; delta_tot_table.c:193-250) runs on the
// host exactly as for a single context (ksp_api.cu, update_device); the per-instance
// parameters of the call are packed into one pinned buffer, copied with one
// cudaMemcpyAsync, and the kernels of ksp_batch.cu (plus the binning and correction
// of bound grids) are replayed from one captured CUDA graph.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <stdlib.h>
#include <algorithm>
#include <vector>
#include "ksp_batch.h"
#include "ksp_ctx.h"

using namespace ksp;

namespace {
struct BoundGrid {
    int inst;
    float* grid;
    int N;
    double BoxSize;
    Geo* G;
};
}  // namespace

struct kspace_batch {
    int device = 0, M = 0;
    cudaStream_t stream = nullptr;
    std::vector<kspace_ctx*> ctx;
    std::vector<BoundGrid> grids;
    bool laid_out = false;
    std::vector<int> nk, off;           // pool layout
    // device
    IntegratorDev* insts_d = nullptr;
    BatchHeader* hdr_d = nullptr;
    unsigned char* upload_d = nullptr;  // calls | fs_off | fsc_off | bin_off | task_off | header
    unsigned char* upload_h = nullptr;  // pinned mirror
    size_t upload_bytes = 0;
    double* dcdm_pool = nullptr;
    double* dnu_pool = nullptr;
    unsigned* status_d = nullptr;       // [M]
    unsigned* status_h = nullptr;       // pinned [M]
    BatchGridCorr* gcorr_d = nullptr;
    int total_bins = 0, ldmax = 0;
    // tuning
    int wpb = 4, blocks_per_sm = 2, use_graph = 1;
    int nc_slots = 17;  // node-table slots per instance (8 levels of the right spine)
    bool eager_done = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float last_ms = 0;
    std::vector<int> last_status;
    int sm_count = 152;
};

#define CKB(x)                                                                                              \
    do {                                                                                                    \
        cudaError_t e__ = (x);                                                                              \
        if (e__ != cudaSuccess) {                                                                           \
            fprintf(stderr, "kspace_gpu batch: CUDA error %s at %s:%d\n", cudaGetErrorString(e__), __FILE__, \
                    __LINE__);                                                                              \
            return KSPACE_ERR_CUDA;                                                                         \
        }                                                                                                   \
    } while (0)

static void drop_graph(kspace_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

extern "C" int kspace_gpu_batch_create(kspace_batch** out, kspace_ctx* const* ctxs, int M) {
    if (!out || !ctxs || M <= 0) return KSPACE_ERR_ARG;
    *out = nullptr;
    const int dev = ctxs[0]->device;
    for (int i = 0; i < M; i++) {
        kspace_ctx* c = ctxs[i];
        if (!c || c->device != dev) return KSPACE_ERR_ARG;
        if (!c->table_ready || !c->hubble_ready || !c->transfer_ready) return KSPACE_ERR_ORDER;
        for (int j = 0; j < i; j++)
            if (ctxs[j] == c) return KSPACE_ERR_ARG;  // an instance appears once
    }
    CKB(cudaSetDevice(dev));
    kspace_batch* b = new kspace_batch;
    b->device = dev;
    b->M = M;
    b->ctx.assign(ctxs, ctxs + M);
    cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
        cudaMalloc(&b->status_d, sizeof(unsigned) * M) != cudaSuccess ||
        cudaMallocHost(&b->status_h, sizeof(unsigned) * M) != cudaSuccess ||
        cudaMalloc(&b->insts_d, sizeof(IntegratorDev) * M) != cudaSuccess) {
        kspace_gpu_batch_destroy(b);
        return KSPACE_ERR_CUDA;
    }
    cudaMemset(b->status_d, 0, sizeof(unsigned) * M);
    for (int i = 0; i < M; i++) {
        cudaStreamSynchronize(ctxs[i]->stream);
        b->ldmax = std::max(b->ldmax, ctxs[i]->I.ld);
    }
    b->last_status.assign(M, 0);
    if (const char* e = getenv("KSPACE_GPU_NC_LEVELS")) {
        const int l = atoi(e);
        const int lv = l < 0 ? 0 : (l > kNcMaxLevels ? kNcMaxLevels : l);
        b->nc_slots = lv > 0 ? 1 + 2 * lv : 0;
    }
    batch_set_attributes();
    *out = b;
    return KSPACE_OK;
}

extern "C" int kspace_gpu_batch_destroy(kspace_batch* b) {
    if (!b) return KSPACE_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graph(b);
    cudaFree(b->insts_d);
    cudaFree(b->upload_d);
    cudaFreeHost(b->upload_h);
    cudaFree(b->dcdm_pool);
    cudaFree(b->dnu_pool);
    cudaFree(b->status_d);
    cudaFreeHost(b->status_h);
    cudaFree(b->gcorr_d);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return KSPACE_OK;
}

extern "C" int kspace_gpu_batch_bind_grid(kspace_batch* b, int inst, void* grid, int pmgrid, double BoxSize) {
    if (!b || !grid || inst < 0 || inst >= b->M || pmgrid < 2 || !(BoxSize > 0)) return KSPACE_ERR_ARG;
    if (b->laid_out) return KSPACE_ERR_ORDER;
    if (!is_device_ptr(grid)) return KSPACE_ERR_ARG;
    for (const BoundGrid& g : b->grids)
        if (g.inst == inst || g.grid == grid) return KSPACE_ERR_ARG;
    kspace_ctx* c = b->ctx[inst];
    Geo* G = nullptr;
    int st = ctx_get_geo(c, pmgrid, c->I.nk_alloc, &G);
    if (st) return st;
    b->grids.push_back(BoundGrid{inst, reinterpret_cast<float*>(grid), pmgrid, BoxSize, G});
    return KSPACE_OK;
}

// Per-call upload layout (one pinned buffer, one copy).
struct UploadPlan {
    size_t calls, fs_off, fsc_off, bin_off, task_off, hdr, total;
};
static UploadPlan plan_upload(int M) {
    UploadPlan p;
    size_t o = 0;
    auto take = [&](size_t n) {
        const size_t at = o;
        o += (n + 255) & ~size_t(255);
        return at;
    };
    p.calls = take(sizeof(BatchCall) * M);
    p.fs_off = take(sizeof(int) * (M + 1));
    p.fsc_off = take(sizeof(int) * (M + 1));
    p.bin_off = take(sizeof(int) * (M + 1));
    p.task_off = take(sizeof(int) * (M + 1));
    p.hdr = take(sizeof(BatchHeader));
    p.total = o;
    return p;
}

static BatchDev dev_view(kspace_batch* b) {
    const UploadPlan p = plan_upload(b->M);
    BatchDev d;
    d.insts = b->insts_d;
    d.calls = reinterpret_cast<const BatchCall*>(b->upload_d + p.calls);
    d.hdr = reinterpret_cast<BatchHeader*>(b->upload_d + p.hdr);
    d.fs_off = reinterpret_cast<const int*>(b->upload_d + p.fs_off);
    d.fsc_off = reinterpret_cast<const int*>(b->upload_d + p.fsc_off);
    d.bin_off = reinterpret_cast<const int*>(b->upload_d + p.bin_off);
    d.task_off = reinterpret_cast<const int*>(b->upload_d + p.task_off);
    d.dnu_pool = b->dnu_pool;
    d.M = b->M;
    d.ldmax = b->ldmax;
    d.wpb = b->wpb;
    d.qag_blocks = b->sm_count * b->blocks_per_sm;
    d.nc_slots = b->nc_slots;
    return d;
}

// Fix the pool layout, allocate the pools and the per-instance device descriptors.
static int lay_out(kspace_batch* b, const int* nk_in) {
    const int M = b->M;
    b->nk.assign(M, 0);
    for (int i = 0; i < M; i++) b->nk[i] = nk_in ? nk_in[i] : 0;
    for (const BoundGrid& g : b->grids) b->nk[g.inst] = g.G->nk;
    b->off.assign(M + 1, 0);
    for (int i = 0; i < M; i++) {
        if (b->nk[i] < 0 || b->nk[i] > b->ctx[i]->I.nk_alloc) return KSPACE_ERR_NK_ALLOC;
        b->off[i + 1] = b->off[i] + b->nk[i];
    }
    b->total_bins = b->off[M];
    CKB(cudaMalloc(&b->dcdm_pool, sizeof(double) * std::max(1, b->total_bins)));
    CKB(cudaMalloc(&b->dnu_pool, sizeof(double) * std::max(1, b->total_bins)));
    CKB(cudaMemset(b->dcdm_pool, 0, sizeof(double) * std::max(1, b->total_bins)));
    const UploadPlan p = plan_upload(M);
    b->upload_bytes = p.total;
    CKB(cudaMalloc(&b->upload_d, p.total));
    CKB(cudaMallocHost(&b->upload_h, p.total));
    memset(b->upload_h, 0, p.total);
    std::vector<IntegratorDev> desc(M);
    for (int i = 0; i < M; i++) {
        desc[i] = b->ctx[i]->I;
        desc[i].dcdm = b->dcdm_pool + b->off[i];  // the instance's delta_cdm lives in the pool
        desc[i].status = b->status_d + i;
        desc[i].ivals = nullptr;
        desc[i].nivals = nullptr;
        desc[i].nc_slots = b->nc_slots;
    }
    CKB(cudaMemcpy(b->insts_d, desc.data(), sizeof(IntegratorDev) * M, cudaMemcpyHostToDevice));
    if (!b->grids.empty()) {
        std::vector<BatchGridCorr> gc(b->grids.size());
        for (size_t j = 0; j < b->grids.size(); j++) {
            kspace_ctx* c = b->ctx[b->grids[j].inst];
            gc[j].inst = b->grids[j].inst;
            gc[j].keff = c->keff_d;
            gc[j].corr = c->corr;
            gc[j].corr.nk = b->grids[j].G->nk;
            gc[j].norm_out = c->norm_d;
        }
        CKB(cudaMalloc(&b->gcorr_d, sizeof(BatchGridCorr) * gc.size()));
        CKB(cudaMemcpy(b->gcorr_d, gc.data(), sizeof(BatchGridCorr) * gc.size(), cudaMemcpyHostToDevice));
    }
    b->laid_out = true;
    return KSPACE_OK;
}

// Binning of a bound grid into its instance's delta_cdm (K1 + normalisation).
static int enqueue_bin(kspace_batch* b, const BoundGrid& g) {
    kspace_ctx* c = b->ctx[g.inst];
    GridGeom gg = g.G->g;
    gg.slab0 = 0;
    gg.nslab = g.N;
    gg.nmodes = (long long)g.N * g.N * (g.N / 2 + 1);
    const int nb = gg.nrbins;
    CKB(cudaMemsetAsync(c->bin_sum_d, 0, sizeof(double) * (nb + 1), b->stream));
    if (launch_bin_power(gg, g.grid, c->bin_sum_d, c->bin_sum_d + nb, b->status_d + g.inst, c->tma, c->rows,
                         c->stages, b->stream) < 0)
        return KSPACE_ERR_CUDA;
    launch_finalize_power(c->bin_sum_d, c->bin_sum_d + nb, g.G->count_d, g.G->ksum_d, g.G->compact_d, g.G->nk,
                          g.BoxSize, c->power_d, c->keffg_d, b->dcdm_pool + b->off[g.inst], c->keff_d, b->stream);
    return KSPACE_OK;
}

static int enqueue_correct(kspace_batch* b, const BoundGrid& g) {
    kspace_ctx* c = b->ctx[g.inst];
    GridGeom gg = g.G->g;
    gg.slab0 = 0;
    gg.nslab = g.N;
    gg.nmodes = (long long)g.N * g.N * (g.N / 2 + 1);
    CorrTable corr = c->corr;
    corr.nk = g.G->nk;
    const float lnscale = (float)log(2 * kPi / g.BoxSize);
    if (launch_apply_correction(gg, g.grid, corr, lnscale, b->status_d + g.inst, c->tma, c->rows, c->stages,
                                b->stream) < 0)
        return KSPACE_ERR_CUDA;
    return KSPACE_OK;
}

// The whole step's device work in stream order.
static int enqueue_step(kspace_batch* b, bool correct) {
    for (const BoundGrid& g : b->grids) {
        const int st = enqueue_bin(b, g);
        if (st) return st;
    }
    const BatchDev d = dev_view(b);
    launch_batch_update(d, b->stream);
    if (correct && !b->grids.empty()) {
        launch_batch_corr(d, b->gcorr_d, (int)b->grids.size(), b->stream);
        for (const BoundGrid& g : b->grids) {
            const int st = enqueue_correct(b, g);
            if (st) return st;
        }
    }
    CKB(cudaPeekAtLastError());
    return KSPACE_OK;
}

static int read_status(kspace_batch* b) {
    CKB(cudaMemcpyAsync(b->status_h, b->status_d, sizeof(unsigned) * b->M, cudaMemcpyDeviceToHost, b->stream));
    CKB(cudaStreamSynchronize(b->stream));
    int first = KSPACE_OK;
    bool any = false;
    for (int i = 0; i < b->M; i++) {
        const int s = map_status(b->status_h[i]);
        if (b->last_status[i] == KSPACE_OK) b->last_status[i] = s;
        if (b->status_h[i]) any = true;
        if (!first && b->last_status[i]) first = b->last_status[i];
    }
    if (any) CKB(cudaMemsetAsync(b->status_d, 0, sizeof(unsigned) * b->M, b->stream));
    return first;
}

extern "C" int kspace_gpu_batch_init(kspace_batch* b, const double* a, const int* nk, const double* keff,
                                     const double* dcdm) {
    if (!b || !a) return KSPACE_ERR_ARG;
    if (b->laid_out) return KSPACE_ERR_ORDER;
    CKB(cudaSetDevice(b->device));
    int st = lay_out(b, nk);
    if (st) return st;
    std::vector<char> bound(b->M, 0);
    for (const BoundGrid& g : b->grids) bound[g.inst] = 1;
    // per instance, as the first call of the single-context path (update_device); the
    // input pools hold the unbound instances only, laid out by nk (bound ones count 0)
    size_t in_off = 0;
    for (int i = 0; i < b->M; i++) {
        kspace_ctx* c = b->ctx[i];
        if (bound[i]) continue;
        const int n = b->nk[i];
        if (n > 0 && (!keff || !dcdm)) return KSPACE_ERR_ARG;
        double* kd = c->io_d;
        double* dd = c->io_d + c->I.nk_alloc;
        if (n > 0) {
            CKB(cudaMemcpyAsync(kd, keff + in_off, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
            CKB(cudaMemcpyAsync(dd, dcdm + in_off, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        }
        in_off += n;
        st = ctx_delta_tot_init(c, n, kd, dd, a[i]);
        if (st) return st;
    }
    for (const BoundGrid& g : b->grids) {
        kspace_ctx* c = b->ctx[g.inst];
        st = ctx_bin_grid(c, g.G, g.grid, g.N, 0, g.N, g.BoxSize);
        if (st) return st;
        st = ctx_delta_tot_init(c, g.G->nk, c->keff_d, c->I.dcdm, a[g.inst]);
        if (st) return st;
    }
    for (int i = 0; i < b->M; i++) CKB(cudaStreamSynchronize(b->ctx[i]->stream));
    return KSPACE_OK;
}

extern "C" int kspace_gpu_batch_layout(kspace_batch* b, int* nk, int* offset) {
    if (!b) return KSPACE_ERR_ARG;
    if (!b->laid_out) return KSPACE_ERR_ORDER;
    if (nk) memcpy(nk, b->nk.data(), sizeof(int) * b->M);
    if (offset) memcpy(offset, b->off.data(), sizeof(int) * (b->M + 1));
    return KSPACE_OK;
}

// Host bookkeeping of every instance for a call at a[i] (update_device's control flow);
// fills the upload buffer.  after[i] receives what to do with the instance's counters
// once the call is done: 0 nothing, 1 committed, 2 provisional row dropped.
static int plan_call(kspace_batch* b, const double* a, bool dry, std::vector<int>& after) {
    const int M = b->M;
    const UploadPlan p = plan_upload(M);
    BatchCall* calls = reinterpret_cast<BatchCall*>(b->upload_h + p.calls);
    int* fs_off = reinterpret_cast<int*>(b->upload_h + p.fs_off);
    int* fsc_off = reinterpret_cast<int*>(b->upload_h + p.fsc_off);
    int* bin_off = reinterpret_cast<int*>(b->upload_h + p.bin_off);
    int* task_off = reinterpret_cast<int*>(b->upload_h + p.task_off);
    BatchHeader* hdr = reinterpret_cast<BatchHeader*>(b->upload_h + p.hdr);
    after.assign(M, 0);
    fs_off[0] = fsc_off[0] = bin_off[0] = task_off[0] = 0;
    for (int i = 0; i < M; i++) {
        kspace_ctx* c = b->ctx[i];
        BatchCall& P = calls[i];
        memset(&P, 0, sizeof(P));
        P.nk = b->nk[i];
        P.dry = dry ? 1 : 0;
        int st = KSPACE_OK;
        if (!c->init_done) st = KSPACE_ERR_ORDER;
        else if (c->nk != b->nk[i]) st = KSPACE_ERR_NK_MISMATCH;
        else if (c->nk < 2) st = KSPACE_ERR_NK_SMALL;
        b->last_status[i] = st;
        if (st == KSPACE_OK) {
            const double loga = log(a[i]);
            P.a = a[i];
            P.loga = loga;
            P.loga0 = c->loga0;
            P.TimeTransfer = c->TimeTransfer;
            P.nspec = c->nspec;
            for (int s = 0; s < 3; s++) P.spec[s] = c->spec_ids[s];
            if (loga - c->h_scalefact[c->ia - 1] < kFloatAcc) {
                // same scale factor: delta_nu_last unchanged (delta_tot_table.c:209-213)
                P.active = 1;
                P.commit_row = -2;
                P.Na = c->ia;
            } else if (c->ia >= c->I.namax) {
                b->last_status[i] = KSPACE_ERR_NAMAX;
            } else {
                P.active = 1;
                const int Na = c->ia + 1;
                P.Na = Na;
                P.start_row = c->fact_valid;
                P.nfs = loga > c->loga0 ? 16 * Na : 0;
                const bool commit = a[i] >= exp(c->h_scalefact[Na - 2]) + 0.009;  // :229-237
                P.commit_row = commit ? Na - 1 : -1;
                after[i] = dry ? 0 : (commit ? 1 : 2);
            }
        }
        const bool integ = P.active && P.commit_row != -2;
        fs_off[i + 1] = fs_off[i] + (integ && P.nfs > 0 ? fs_groups(P.nfs, P.loga0, P.loga) : 0);
        fsc_off[i + 1] = fsc_off[i] + (integ && P.nfs > 2 ? P.nfs - 2 : 0);
        bin_off[i + 1] = b->off[i + 1];
        task_off[i + 1] = task_off[i] + (integ ? P.nspec * P.nk : 0);
    }
    memset(hdr, 0, sizeof(*hdr));
    hdr->M = M;
    hdr->total_segs = fs_off[M];
    hdr->total_fsc = fsc_off[M];
    hdr->total_bins = bin_off[M];
    hdr->total_tasks = task_off[M];
    return KSPACE_OK;
}

static void apply_after(kspace_batch* b, const double* a, const std::vector<int>& after) {
    for (int i = 0; i < b->M; i++) {
        kspace_ctx* c = b->ctx[i];
        if (!after[i]) continue;
        const int Na = c->ia + 1;
        c->h_scalefact[c->ia] = log(a[i]);
        if (after[i] == 1) {
            c->ia = Na;
            c->fact_valid = Na - 2 > 0 ? Na - 2 : 0;
        } else {
            c->fact_valid = Na - 3 > 0 ? Na - 3 : 0;
        }
    }
}

// Upload the call, then run the device work: from the graph, or launched one by one.
static int run_call(kspace_batch* b, bool dry, bool timed) {
    CKB(cudaMemcpyAsync(b->upload_d, b->upload_h, b->upload_bytes, cudaMemcpyHostToDevice, b->stream));
    if (timed) CKB(cudaEventRecord(b->ev0, b->stream));
    if (dry || !b->use_graph || !b->eager_done) {
        // launched one by one; the first real call always is (it loads the kernels and
        // sets their attributes before anything is captured)
        const int st = enqueue_step(b, !dry);
        if (st) return st;
        if (!dry) b->eager_done = true;
    } else {
        if (!b->exec) {
            CKB(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            const int st = enqueue_step(b, true);
            cudaGraph_t g = nullptr;
            const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
            if (st) {
                if (g) cudaGraphDestroy(g);
                return st;
            }
            CKB(e);
            b->graph = g;
            CKB(cudaGraphInstantiate(&b->exec, b->graph, 0));
        }
        CKB(cudaGraphLaunch(b->exec, b->stream));
    }
    if (timed) CKB(cudaEventRecord(b->ev1, b->stream));
    return KSPACE_OK;
}

extern "C" int kspace_gpu_batch_step(kspace_batch* b, const double* a, const double* dcdm, double* dnu) {
    if (!b || !a) return KSPACE_ERR_ARG;
    if (!b->laid_out) return KSPACE_ERR_ORDER;
    CKB(cudaSetDevice(b->device));
    if (b->grids.size() < (size_t)b->M && !dcdm && b->total_bins > 0) {
        // every unbound instance needs its delta_cdm
        bool need = false;
        std::vector<char> bound(b->M, 0);
        for (const BoundGrid& g : b->grids) bound[g.inst] = 1;
        for (int i = 0; i < b->M; i++)
            if (!bound[i] && b->nk[i] > 0) need = true;
        if (need) return KSPACE_ERR_ARG;
    }
    std::vector<int> after;
    int st = plan_call(b, a, false, after);
    if (st) return st;
    if (dcdm && b->total_bins > 0) {
        // bound instances' slices are overwritten by the binning inside the step
        CKB(cudaMemcpyAsync(b->dcdm_pool, dcdm, sizeof(double) * b->total_bins, cudaMemcpyDefault, b->stream));
    }
    st = run_call(b, false, true);
    if (st) return st;
    if (dnu && b->total_bins > 0)
        CKB(cudaMemcpyAsync(dnu, b->dnu_pool, sizeof(double) * b->total_bins, cudaMemcpyDefault, b->stream));
    const int rs = read_status(b);
    cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1);
    apply_after(b, a, after);
    return rs;
}

extern "C" int kspace_gpu_batch_status(kspace_batch* b, int* status) {
    if (!b || !status) return KSPACE_ERR_ARG;
    memcpy(status, b->last_status.data(), sizeof(int) * b->M);
    return KSPACE_OK;
}

extern "C" int kspace_gpu_batch_set_tuning(kspace_batch* b, int wpb, int blocks_per_sm, int use_graph) {
    if (!b || wpb < 1 || wpb > 4 || blocks_per_sm < 1 || blocks_per_sm > 16) return KSPACE_ERR_ARG;
    if (batch_qag_smem(b->ldmax, wpb) > 227 * 1024 - 256) return KSPACE_ERR_ARG;
    if (wpb != b->wpb || blocks_per_sm != b->blocks_per_sm) drop_graph(b);
    b->wpb = wpb;
    b->blocks_per_sm = blocks_per_sm;
    b->use_graph = use_graph ? 1 : 0;
    return KSPACE_OK;
}

extern "C" int kspace_gpu_batch_autotune(kspace_batch* b, const double* a, const double* dcdm, int reps, int* best,
                                         float* best_ms) {
    if (!b || !a || reps < 1) return KSPACE_ERR_ARG;
    if (!b->laid_out) return KSPACE_ERR_ORDER;
    CKB(cudaSetDevice(b->device));
    std::vector<int> after;
    int st = plan_call(b, a, true, after);
    if (st) return st;
    if (dcdm && b->total_bins > 0)
        CKB(cudaMemcpyAsync(b->dcdm_pool, dcdm, sizeof(double) * b->total_bins, cudaMemcpyDefault, b->stream));
    const int wpb0 = b->wpb, bps0 = b->blocks_per_sm;
    float best_t = 1e30f;
    int bw = wpb0, bb = bps0;
    for (int w = 1; w <= 4; w *= 2) {
        const size_t smem = batch_qag_smem(b->ldmax, w);
        if (smem > 227 * 1024 - 256) continue;
        const int fit = (int)((228 * 1024) / (smem + 1024));  // resident blocks by shared memory
        for (int bps = 1; bps <= std::min(fit, 8); bps++) {
            b->wpb = w;
            b->blocks_per_sm = bps;
            std::vector<float> ts;
            for (int r = 0; r < reps; r++) {
                st = run_call(b, true, true);
                if (st) break;
                CKB(cudaEventSynchronize(b->ev1));
                float ms = 0;
                cudaEventElapsedTime(&ms, b->ev0, b->ev1);
                ts.push_back(ms);
            }
            if (st) break;
            std::sort(ts.begin(), ts.end());
            const float t = ts[ts.size() / 2];
            if (t < best_t) {
                best_t = t;
                bw = w;
                bb = bps;
            }
        }
        if (st) break;
    }
    const int rs = read_status(b);
    b->wpb = wpb0;
    b->blocks_per_sm = bps0;
    if (st) return st;
    if (rs) return rs;
    kspace_gpu_batch_set_tuning(b, bw, bb, b->use_graph);
    if (best) {
        best[0] = bw;
        best[1] = bb;
    }
    if (best_ms) *best_ms = best_t;
    return KSPACE_OK;
}

extern "C" int kspace_gpu_batch_last_ms(kspace_batch* b, float* ms) {
    if (!b || !ms) return KSPACE_ERR_ARG;
    *ms = b->last_ms;
    return KSPACE_OK;
}
