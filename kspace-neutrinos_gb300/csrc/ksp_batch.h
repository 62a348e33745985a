// ksp_batch.h -- device-side description of a batch of independent integrator
// instances advanced by one captured sequence of kernels.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include "ksp_internal.h"

namespace ksp {

// Per-instance parameters of one batched call, filled on the host from the instance's
// bookkeeping exactly as the single-instance update does (delta_tot_table.c:193-250).
struct BatchCall {
    double a, loga, loga0, TimeTransfer;
    int Na;          // history rows used by this call (the provisional row included)
    int nk;          // bins of the instance
    int nfs;         // fslength table nodes (16*Na, 0 when log a <= log a0)
    int start_row;   // leading rows of the knot factorisation still valid
    int commit_row;  // >= 0 keep that row, -1 drop the provisional row, -2 same scale factor
    int active;      // 0: instance not advanced in this call
    int dry;         // 1: nothing committed and delta_nu_last kept (tuning runs)
    int nspec;
    int spec[3];
};

// Totals of the current call; the kernels are launched with fixed grids (so one
// captured graph serves every call) and stride over these.
struct BatchHeader {
    int M;
    int total_segs;   // fslength segment groups (fs_groups of each instance)
    int total_fsc;    // sum of max(nfs-2, 0): fslength spline unknowns
    int total_bins;   // sum of nk
    int total_tasks;  // sum of nspec*nk over integrating instances
    int counter;      // task queue of kb_dnu_qag (reset by kb_prologue)
    int pad[2];
};

// Device arrays of the batch (offsets have M+1 entries).
struct BatchDev {
    const IntegratorDev* insts;
    const BatchCall* calls;
    BatchHeader* hdr;
    const int* fs_off;
    const int* fsc_off;
    const int* bin_off;
    const int* task_off;
    double* dnu_pool;   // [total_bins] delta_nu returned by every instance
    int M, ldmax, wpb, qag_blocks;
    int nc_slots;       // node-table slots of every instance (their IntegratorDev.nc_slots)
};

// Correction table of a grid bound to instance `inst` (interface_common.c:134-146).
struct BatchGridCorr {
    int inst;
    const double* keff;  // physical keff of the grid's bins
    CorrTable corr;
    double* norm_out;
};

size_t batch_qag_smem(int ldmax, int wpb);
void batch_set_attributes();
void launch_batch_update(const BatchDev& b, cudaStream_t st);
void launch_batch_corr(const BatchDev& b, const BatchGridCorr* g, int ngrid, cudaStream_t st);

}  // namespace ksp
