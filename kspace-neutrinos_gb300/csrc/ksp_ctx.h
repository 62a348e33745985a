// ksp_ctx.h -- the library context (what the reference keeps in process-global
// singletons, interface_common.c:17-26 and interface_gadget.c:19-21) and the host
// helpers shared by the translation units of the C ABI.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <atomic>
#include <map>
#include <vector>
#include "ksp_internal.h"
#include "../../include/kspace_gpu.h"

namespace ksp {
extern std::atomic<long long> g_launches;  // kernels launched by the library (diagnostics)
}
using ksp::Background;
using ksp::CorrTable;
using ksp::GridGeom;
using ksp::IntegratorDev;

struct Geo {
    GridGeom g;                      // device tables + slab parameters (slab fields set per call)
    std::vector<long long> count;    // full-grid mode count per bin
    std::vector<double> ksum;        // full-grid sum |k| per bin (grid units)
    std::vector<int> compact;        // non-empty bins in order
    long long* count_d = nullptr;
    double* ksum_d = nullptr;
    int* compact_d = nullptr;
    int nk = 0;
};

struct kspace_ctx {
    int device = 0;
    cudaStream_t stream = nullptr, own_stream = nullptr;
    kspace_allreduce_fn ar_fn = nullptr;
    void* ar_user = nullptr;
    int tma = 5, rows = 256, stages = 2, qag_warps = 1;
    int nc_levels = 12;  // depths of QAG's rightmost bisections kept in the integrand node table (all)
    int qag_split = 0;  // warps per (species, bin) integral: 1, 2, 4, 8 (8: with look-ahead); 0 = by the task count
    // background
    bool bg_ready = false, hubble_ready = false;
    Background hB;
    Background* dB = nullptr;
    double MNu[3] = {0, 0, 0};
    double bg_a0 = 0.01;
    // a tabulated host H(a) (Background::htab_*): device coefficients and their host copy
    double* htab_dev = nullptr;
    std::vector<double> htab_host;
    int nspec = 0, spec_ids[3] = {0, 0, 0};
    // integrator table
    bool table_ready = false;
    IntegratorDev I{};
    double TimeTransfer = 0, loga0 = 0;
    int nk = 0, ia = 0, init_done = 0, fact_valid = 0;
    std::vector<double> h_scalefact;
    std::vector<double> t_logk, t_T;
    bool transfer_ready = false;
    // step buffers
    double *bin_sum_d = nullptr, *F0sq_d = nullptr, *power_d = nullptr, *keffg_d = nullptr, *keff_d = nullptr;
    double *logk_d = nullptr, *ratio_d = nullptr, *norm_d = nullptr, *dnu_out_d = nullptr, *io_d = nullptr;
    int buf_nb = 0;
    CorrTable corr{};
    unsigned* status_d = nullptr;
    unsigned* status_h = nullptr;
    double* ar_h = nullptr;
    int last_nk = 0;
    double last_BoxSize = 0;
    // geometry cache keyed by (N, nrbins)
    std::map<std::pair<int, int>, Geo> geos;
    // staging for host grids
    void* stage_d = nullptr;
    size_t stage_bytes = 0;
    // differentiable step
    double Omeganonu = 0;
    double *ivals_d = nullptr, *adj_node_d = nullptr, *adj_Dbar_d = nullptr, *adj_mbar_d = nullptr;
    double *adj_Q_d = nullptr, *adj_dcsum_d = nullptr, *adj_dnubar_d = nullptr, *adj_rbar_d = nullptr;
    int* nivals_d = nullptr;
    int adj_cap_nb = 0;
    bool diff_ready = false;
    int diff_ia = 0, diff_Na = 0, diff_nk = 0, diff_store = 0;
    long long diff_gen = 0;  // counts successful diff_forward calls
    double diff_time = 0, diff_box = 0;
    int diff_pmgrid = 0;
    // the delta_cdm-independent integrator work of a step, run on a side stream while the
    // binning pass runs (add_nu_power_to_rhogrid)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // host grids move in slab chunks on a copy stream: the binning pass runs behind the
    // upload, the download behind the correction pass
    static constexpr int kChunks = 16;
    int chunks = 8;  // slab chunks of a host grid (1..kChunks)
    cudaStream_t copy = nullptr;
    cudaEvent_t ev_up[kChunks] = {}, ev_done[kChunks] = {}, ev_copy_start = nullptr, ev_copy_end = nullptr;
    bool prep_valid = false;
    int prep_Na = 0;
    double prep_loga = 0;
    bool prep_base = false;  // launch_dtot_base ran with the preparation
    // the binning pass's normalisation, deferred into the row-spline kernel of a prepared
    // step (active = 0: already done)
    ksp::FinalizeArgs fin{};
    // profiling
    bool prof = false;
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    float stage_ms[4] = {0, 0, 0, 0};
};

// ---- host helpers (ksp_api.cu)
namespace ksp {
int map_status(unsigned s);
bool is_device_ptr(const void* p);
// delta_tot_init (delta_tot_table.c:79-149) on device keff / delta_cdm
int ctx_delta_tot_init(kspace_ctx* c, int nk_in, const double* keff_d, const double* dcdm_d, double Time);
// geometry (bin thresholds, counts, window) of an N^3 grid with nrbins bins, cached
int ctx_get_geo(kspace_ctx* c, int N, int nrbins, Geo** out);
// K1 + allreduce + normalisation: power, keff, delta_cdm (into c->I.dcdm)
int ctx_bin_grid(kspace_ctx* c, Geo* G, const float* gd, int pmgrid, int slab0, int nslab, double BoxSize);
int ctx_sync_status(kspace_ctx* c);
}  // namespace ksp
