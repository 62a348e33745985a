// ksp_noalloc.cu -- kspace_gpu_bin_power_noalloc: the binning pass (K1) for callers
// that must not allocate memory.
//
// Who cannot allocate: a host that owns all device memory through its own pool (and
// forbids the library its own cudaMalloc), code running where a device allocation
// would synchronise the device or fail (a memory-exhausted PM code at the end of a
// large run), and callers that want a fixed, known footprint.  The context-based entry
// points allocate their tables and step buffers once per context; this entry point
// needs no context and allocates nothing: its per-call scratch (bin thresholds, the
// 1-D window, the per-bin sums, a status word) lives in one file-scope __device__
// array of fixed size, and its host-side tables in fixed-size static arrays.
//
// Limits: nrbins <= kNoAllocMaxBins (4096) and dims <= kNoAllocMaxDims (4096); larger
// requests are refused with KSPACE_ERR_ARG and a message on stderr.  The scratch is
// about 57 KB.  Calls share the scratch, so calls that overlap (from two host threads, or
// queued on two streams at once) race; serialise them.  The first call on a device
// looks up the scratch address (cudaGetSymbolAddress) with that device current.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>
#include "ksp_internal.h"
#include "../../include/kspace_gpu.h"

namespace ksp {

constexpr int kNoAllocMaxBins = 4096;
constexpr int kNoAllocMaxDims = 4096;
constexpr int kNoAllocMaxDevices = 64;

// Layout of the scratch: sums[kNoAllocMaxBins + 1] (the last entry is |F(0)|^2),
// thresholds[kNoAllocMaxBins + 1], window[kNoAllocMaxDims / 2 + 1], status.
struct NoAllocScratch {
    double sums[kNoAllocMaxBins + 1];
    int thresh[kNoAllocMaxBins + 1];
    float w1[kNoAllocMaxDims / 2 + 1];
    unsigned status;
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

static NoAllocScratch* g_scratch_ptr[kNoAllocMaxDevices];

// host-side tables of the last call (fixed size, no allocation)
static int h_thresh[kNoAllocMaxBins + 1];
static float h_w1[kNoAllocMaxDims / 2 + 1];

// Bin of integer k^2 >= 1 as total_powerspectrum computes it (powerspectrum.c:40,67),
// clamped to the bins, and its smallest k^2: the thresholds the kernel settles on.
static int ref_bin(long long k2, double bpu, int nrbins) {
    int b = (int)floor(bpu * log(sqrt((double)k2)));
    if (b < 0) b = 0;
    if (b > nrbins - 1) b = nrbins - 1;
    return b;
}

}  // namespace ksp

using namespace ksp;

// No counterpart in the reference: see include/kspace_gpu.h.
extern "C" int kspace_gpu_bin_power_noalloc(int dims, const void* grid, int nrbins, int startslab, int nslab,
                                            double* bin_sums, void* cuda_stream) {
    if (!grid || !bin_sums || dims < 2 || (dims % 2) != 0 || nrbins < 2 || nslab < 0 || startslab < 0 ||
        startslab + nslab > dims)
        return KSPACE_ERR_ARG;
    if (nrbins > kNoAllocMaxBins || dims > kNoAllocMaxDims) {
        fprintf(stderr,
                "kspace_gpu_bin_power_noalloc: nrbins %d / dims %d exceed the fixed scratch (at most %d bins, "
                "dims %d)\n",
                nrbins, dims, kNoAllocMaxBins, kNoAllocMaxDims);
        return KSPACE_ERR_ARG;
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(cuda_stream);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) return KSPACE_ERR_CUDA;
    // set-up, once per device, with that device current
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            fprintf(stderr, "kspace_gpu_bin_power_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
            return KSPACE_ERR_CUDA;
        }
        g_scratch_ptr[dev] = reinterpret_cast<NoAllocScratch*>(p);
    }
    NoAllocScratch* S = g_scratch_ptr[dev];
    // bin thresholds: the smallest k^2 of each bin, by bisection on the monotone bin
    // function (k2max + 1 for bins no k^2 reaches)
    const long long k2max = 3LL * (dims / 2) * (dims / 2);
    if (k2max >= (1LL << 24)) return KSPACE_ERR_ARG;  // k^2 must stay exact in float
    const double bpu = (nrbins - 1) / log(sqrt(3) * dims / 2.0);
    h_thresh[0] = 1;
    for (int b = 1; b <= nrbins; b++) {
        long long lo = 1, hi = k2max + 1;  // first k2 in [lo, hi) with bin >= b
        while (lo < hi) {
            const long long mid = (lo + hi) / 2;
            if (ref_bin(mid, bpu, nrbins) >= b) hi = mid; else lo = mid + 1;
        }
        h_thresh[b] = (int)lo;
    }
    // 1-D inverse window in float (powerspectrum.c:8-12)
    const int nz = dims / 2 + 1;
    for (int k = 0; k < nz; k++) h_w1[k] = k ? (float)(kPi * k / (dims * sin(kPi * k / (float)dims))) : 1.0f;
    // what must start at zero: the per-bin sums, |F(0)|^2 and the status word
    if (cudaMemsetAsync(S->sums, 0, sizeof(double) * (nrbins + 1), st) != cudaSuccess ||
        cudaMemsetAsync(&S->status, 0, sizeof(unsigned), st) != cudaSuccess ||
        cudaMemcpyAsync(S->thresh, h_thresh, sizeof(int) * (nrbins + 1), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(S->w1, h_w1, sizeof(float) * nz, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return KSPACE_ERR_CUDA;
    GridGeom g;
    memset(&g, 0, sizeof(g));
    g.N = dims;
    g.nrbins = nrbins;
    g.slab0 = startslab;
    g.nslab = nslab;
    g.nmodes = (long long)nslab * dims * nz;
    g.thresh = S->thresh;
    g.w1 = S->w1;
    g.cmap = nullptr;
    g.bin_c1 = (float)(bpu * 0.5 * log(2.0));
    if (g.nmodes > 0 &&
        launch_bin_power(g, reinterpret_cast<const float*>(grid), S->sums, S->sums + nrbins, &S->status, 5, 256, 2,
                         st) < 0)
        return KSPACE_ERR_CUDA;
    unsigned status = 0;
    if (cudaMemcpyAsync(bin_sums, S->sums, sizeof(double) * (nrbins + 1), cudaMemcpyDefault, st) != cudaSuccess ||
        cudaMemcpyAsync(&status, &S->status, sizeof(unsigned), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return KSPACE_ERR_CUDA;
    return status ? KSPACE_ERR_TIMEOUT : KSPACE_OK;
}
