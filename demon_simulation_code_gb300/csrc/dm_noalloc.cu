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
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/demon_gb300.h"
#include "dm_misc.cuh"

using namespace dm;

namespace {

constexpr int kDiagThreads = 128;       // same block size as dm_cloud_diagnostics
constexpr int kMaxBlocks = 4096;        // => at most 524,288 particles per call
constexpr int kMaxParticles = kDiagThreads * kMaxBlocks;

// The scratch: one row of 5 partial sums per block.
static __device__ __align__(256) double g_diag_scratch[kMaxBlocks * 5];

// In host code g_diag_scratch names a host-side stand-in, not device memory;
// the device address is looked up once per device (with that device current)
// and cached here.
constexpr int kMaxDevices = 64;
double *g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_setup_mutex;

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

// Errors are reported by status code only (no message store is shared with
// the rest of the library).
int fail(int code, const std::string &msg) {
    (void)msg;
    return code;
}

// Per-device set-up: runs on the first call on each device, with that
// device current.  It may load the module, so make that first call before
// any stream capture.
int scratch_for_current_device(double **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(DM_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(DM_ERR_UNSUPPORTED, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_diag_scratch);
        if (e != cudaSuccess || !p)
            return fail(DM_ERR_CUDA, std::string("cudaGetSymbolAddress(g_diag_scratch): ") +
                                         cudaGetErrorString(e));
        g_scratch_addr[dev] = static_cast<double *>(p);
    }
    *out = g_scratch_addr[dev];
    return DM_OK;
}

}  // namespace

extern "C" int dm_diagnostics_noalloc(int n, const double *d_x, const double *d_y,
                                      const double *d_vx, const double *d_vy,
                                      const double *d_q, const double *d_m,
                                      const dm_force_params *params, double *d_out,
                                      void *stream) {
    if (n < 1 || n > kMaxParticles)
        return fail(DM_ERR_ARG, "dm_diagnostics_noalloc: n = " + std::to_string(n) +
                                    " outside [1, " + std::to_string(kMaxParticles) +
                                    "] (the fixed scratch holds " + std::to_string(kMaxBlocks) +
                                    " blocks of " + std::to_string(kDiagThreads) + ")");
    if (!d_x || !d_y || !d_vx || !d_vy || !d_q || !d_m || !d_out || !params)
        return fail(DM_ERR_ARG, "dm_diagnostics_noalloc: NULL pointer");
    if ((params->flags & DM_SHIELDED_COULOMB_FORCE) && !(params->shielding > 0.0))
        return fail(DM_ERR_ARG, "dm_diagnostics_noalloc: shielding must be positive");
    double *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
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
    ForceParams f;
    static_assert(sizeof(ForceParams) == sizeof(dm_force_params), "layout");
    memcpy(&f, params, sizeof(f));
    const double coulomb = 1.0 / (4.0 * M_PI * 8.8541878E-12);
    const int blocks = (n + kDiagThreads - 1) / kDiagThreads;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    diagnostics_partial<kDiagThreads><<<blocks, kDiagThreads, 0, s>>>(c, f, coulomb, scratch);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        diag_finish<<<1, 256, 0, s>>>(scratch, blocks, d_out);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess)
        return fail(DM_ERR_CUDA, std::string("dm_diagnostics_noalloc launch: ") + cudaGetErrorString(e));
    return DM_OK;
}
