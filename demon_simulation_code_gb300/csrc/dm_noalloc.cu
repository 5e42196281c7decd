// dm_noalloc.cu -- diagnostics entry point that allocates no memory.
//
// Some callers can't call cudaMalloc: a host application that manages every
// byte of device memory through its own fixed pool or budget, or code that
// must not trigger cudaMalloc's implicit device-wide synchronisation while
// its other streams run.  They already hold the particle state in their own
// device buffers and want the FP64 energies and momentum of it without
// creating a dm_cloud (which allocates ~200 bytes per particle) and without
// the temporary partial-sum buffer dm_cloud_diagnostics allocates.
//
// This file gives them dm_diagnostics_noalloc: the same diagnostics kernel,
// with its per-block partial sums in a fixed-size file-scope device array.
// Every GPU that loads this library holds that array (kMaxBlocks * 5
// doubles = 160 KiB) until the process exits.  Calls share the array, so
// calls that overlap on the GPU (different streams, or different host
// threads on the same device) race on it and must be serialised by the
// caller.  Each call overwrites every partial it later reads, so nothing has
// to start at zero.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "../../include/demon_gb300.h"
#include "dm_misc.cuh"

using namespace dm;

namespace {

constexpr int kDiagThreads = 128;       // same block size as dm_cloud_diagnostics
constexpr int kMaxBlocks = 4096;        // => at most 524,288 particles per call
constexpr int kMaxParticles = kDiagThreads * kMaxBlocks;

// The scratch: one row of 5 partial sums per block.
static __device__ __align__(256) double g_diag_scratch[kMaxBlocks * 5];

// In host code g_diag_scratch names a host-side stand-in, not device memory:
// the device address is looked up on every call, with the calling device
// current (see scratch_for_current_device).

// Sums the per-block partials into out[0..4] (one block, strided partial
// sums then a tree): a fixed order for a given block count.
__global__ void __launch_bounds__(256) diag_finish(const double *partial, int nblocks, double *out) {
    __shared__ double red[5][256];
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblocks; b += 256)
        for (int e = 0; e < 5; e++) v[e] += partial[b * 5 + e];
    for (int e = 0; e < 5; e++) red[e][threadIdx.x] = v[e];
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int e = 0; e < 5; e++) red[e][threadIdx.x] += red[e][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < 5) out[threadIdx.x] = red[threadIdx.x][0];
}

// The device address of the scratch on the current device.  Looked up on
// every call rather than cached: the lookup allocates nothing, and a cached
// address would dangle after the host application calls cudaDeviceReset
// (the module is loaded again and the array may move).  The first call on a
// device may load this library's module there, so make that first call
// before any stream capture.
int scratch_for_current_device(double **out) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_diag_scratch) != cudaSuccess || !p) return DM_ERR_CUDA;
    *out = static_cast<double *>(p);
    return DM_OK;
}

}  // namespace

extern "C" int dm_diagnostics_noalloc(int n, const double *d_x, const double *d_y,
                                      const double *d_vx, const double *d_vy,
                                      const double *d_q, const double *d_m,
                                      const dm_force_params *params, double *d_out,
                                      void *stream) {
    // Errors are reported by status code only (no message store is shared
    // with the rest of the library, and building one would allocate).
    if (n < 1 || n > kMaxParticles) return DM_ERR_ARG;  // the scratch holds kMaxBlocks blocks
    if (!d_x || !d_y || !d_vx || !d_vy || !d_q || !d_m || !d_out || !params) return DM_ERR_ARG;
    ForceParams f;
    static_assert(sizeof(ForceParams) == sizeof(dm_force_params), "layout");
    memcpy(&f, params, sizeof(f));
    const char *why = nullptr;
    if (const int st = check_force_params(f, &why)) return st;  // same rules as dm_cloud_set_forces
    double *scratch = nullptr;
    const int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;

    CloudDev c{};
    c.n = n;
    c.n_pad = n;
    c.x = const_cast<double *>(d_x);
    c.y = const_cast<double *>(d_y);
    c.vx = const_cast<double *>(d_vx);
    c.vy = const_cast<double *>(d_vy);
    c.q = const_cast<double *>(d_q);
    c.m = const_cast<double *>(d_m);
    const double coulomb = 1.0 / (4.0 * M_PI * 8.8541878E-12);
    const int blocks = (n + kDiagThreads - 1) / kDiagThreads;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    diagnostics_partial<kDiagThreads><<<blocks, kDiagThreads, 0, s>>>(c, f, coulomb, scratch);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        diag_finish<<<1, 256, 0, s>>>(scratch, blocks, d_out);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? DM_OK : DM_ERR_CUDA;
}
