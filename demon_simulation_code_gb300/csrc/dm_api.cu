// dm_api.cu -- host side of the C ABI declared in include/demon_gb300.h.
//
// One dm_ctx = one GPU + one stream.  One dm_cloud = one device-resident
// particle cloud (layout in dm_device.cuh).  Per RK4 step the library issues
// four launches of the fused pair+stage kernel (dm_pair.cuh); fixed-dt step
// sequences are captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/demon_gb300.h"
#include "dm_misc.cuh"
#include "dm_pair.cuh"
#include "dm_sort.cuh"
#include "dm_batch.cuh"
#include "dm_adjoint.cuh"

using namespace dm;

static_assert(sizeof(dm_force_params) == sizeof(ForceParams), "force params layout");

namespace {

std::string g_create_error;

// FP64: 2 j-groups x 128 i-lanes, 2 particles per lane, 512-particle j tiles
constexpr int kNI64 = 128, kG64 = 2, kILP64 = 2, kJT64 = 512;
constexpr int kGraphSteps = 16;

}  // namespace

struct dm_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    int num_sms = 0;
    std::string err;
    bool prof = false;
    bool autotune = true;
    long long launches = 0;  // kernels this library has launched on the context
    std::map<long long, std::pair<int, int>> tune_cache;  // (n, precision) -> (variant, split)
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_events;
    size_t prof_used = 0;
    double prof_pairs = 0.0;
    long long prof_launches = 0;
    int *h_err = nullptr;  // pinned word for the device error flags (read with each download)
    int sort_ctas = 0;     // blocks of the one-cluster sort (0: not chosen yet)

    int fail(int code, const char *fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
};

struct GraphKey {
    int precision;
    int nsteps;
    double dt;
    bool operator<(const GraphKey &o) const {
        if (precision != o.precision) return precision < o.precision;
        if (nsteps != o.nsteps) return nsteps < o.nsteps;
        return dt < o.dt;
    }
};

struct dm_cloud {
    dm_ctx *ctx = nullptr;
    int n = 0, n_pad = 0;
    void *block = nullptr;
    CloudDev d{};
    ForceParams f{};
    double coulomb = 0.0;
    double *d_fx = nullptr, *d_fy = nullptr;
    double *d_dt = nullptr;
    unsigned int *d_min = nullptr;
    float *d_dmin = nullptr;
    int order = 4;               // integrator: 4 = Runge_Kutta4, 2 = Runge_Kutta2
    int eval_thermal_stage = 1;  // substep of the thermal kicks in force-only evaluations
    int fo_buf = 0;              // stage buffer force-only launches read (the autotuner's dense copy: 1)
    bool boxes_valid[2] = {false, false};  // group boxes (culling) match stage buffer b
    int split[2] = {0, 0};  // cluster size per precision (0 = not chosen yet)
    int tuned_variant[2] = {-1, -1};  // per precision: index into kVariants
    float2 *partial = nullptr;         // [partial_cap][2][n_pad] non-cluster partial sums (per rank, axis)
    int partial_cap = 0;
    SortScratch sort{};
    int sort_blocks = 0;
    int reorder_interval = 1;   // steps between Morton re-sorts (0 = never)
    bool order_dirty = true;    // re-sort before the next step
    unsigned long long host_steps = 0;  // RK4 steps enqueued so far
    long long graph_launches = 0;       // kernels in one replay of the step graph
    std::map<GraphKey, cudaGraphExec_t> graphs;
    cudaStream_t graph_stream = nullptr;  // stream the graphs were built for

    void drop_graphs() {
        for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
    }
    ~dm_cloud() {
        if (partial) cudaFree(partial);
    }
};

#define DM_CUDA(ctx, call)                                                                   \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return (ctx)->fail(DM_ERR_CUDA, "%s failed: %s (%s:%d)", #call,                 \
                               cudaGetErrorString(e_), __FILE__, __LINE__);                 \
    } while (0)

namespace {

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Status for device error flags h already read back (and clears them).
int device_error_status(dm_ctx *ctx, dm_cloud *c, int h) {
    if (h) {
        DM_CUDA(ctx, cudaMemsetAsync(c->d.err, 0, sizeof(int), ctx->stream));
        if (h & 2) return ctx->fail(DM_ERR_NUMERIC, "zero particle separation in the adaptive time step test");
        if (h & kErrSortPermutation)
            return ctx->fail(DM_ERR_CUDA, "internal error: the Morton sort produced an invalid permutation");
        return ctx->fail(DM_ERR_NUMERIC, "non-finite particle position after a stage (error bits 0x%x)", h);
    }
    return DM_OK;
}

int check_device_errors(dm_ctx *ctx, dm_cloud *c) {
    int h = 0;
    DM_CUDA(ctx, cudaMemcpyAsync(&h, c->d.err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return device_error_status(ctx, c, h);
}

// The FP32C sweep's threshold for evaluating a filtered chunk directly
// (StageParams::direct_min): at least this many of a slot's 128 (lane, j)
// pairs passed the filter.  DM_DIRECT_MIN_HITS overrides it (1..129; 129
// never evaluates directly).
int direct_min_hits() {
    static const int v = [] {
        const char *e = getenv("DM_DIRECT_MIN_HITS");
        const int k = e ? atoi(e) : 0;
        return (k >= 1 && k <= 129) ? k : 48;
    }();
    return v;
}

// StageParams::near_direct_f2: groups whose farthest separation from the
// tile is within F = 1.6 r_c are evaluated without the filter (measured on
// disk16k: the collapsed-state launch 154.8 -> 146.0 us, the densest step
// -7%, calm steps +1%; 1.3-2.5 within 1% of each other).
// DM_NEAR_DIRECT_F overrides F (0 turns the class off; at most 4).
float near_direct_f2() {
    static const float v = [] {
        const char *e = getenv("DM_NEAR_DIRECT_F");
        double f = e ? atof(e) : 1.6;
        if (!(f >= 0.0 && f <= 4.0)) f = 0.0;
        return (float)(f * f);
    }();
    return v;
}

// kappa*log2(e) as a float pair (hi + lo to ~2^-48 relative).
void kappa_log2e(double kappa, float &hi, float &lo) {
    const double k = kappa * 1.4426950408889634;
    hi = (float)k;
    lo = (float)(k - (double)hi);
}

StageParams make_stage_params(dm_cloud *c, int stage, int mode, double dt, const double *dt_dev) {
    StageParams P{};
    P.c = c->d;
    P.f = c->f;
    P.stage = stage;
    P.order = c->order;
    P.mode = mode;
    P.therm_stage = (mode == kModeForceOnly) ? c->eval_thermal_stage : stage;
    P.fo_buf = (mode == kModeForceOnly) ? c->fo_buf : 0;
    P.dt = dt;
    P.dt_dev = dt_dev;
    P.coulomb = c->coulomb;
    P.fx_out = c->d_fx;
    P.fy_out = c->d_fy;
    const double kappa = c->f.shielding;
    P.rc2 = (kappa > 0.0) ? (10.0 / kappa) * (10.0 / kappa) : INFINITY;
    // FP32 r^2 is within ~6 ulp of the FP64 value; outside this band the
    // FP32 decision cannot differ from the reference's FP64 one
    P.rc2_lo = (float)(P.rc2 * (1.0 - 4e-6));
    P.rc2_hi = (float)(P.rc2 * (1.0 + 4e-6));
    P.kappa_f = (float)kappa;
    P.nkl2e = (float)(-kappa * 1.4426950408889634);
    P.direct_min = direct_min_hits();
    P.near_direct_f2 = near_direct_f2();
    return P;
}

// ---------------------------------------------------------------------------
// Kernel variants and the autotuner
// ---------------------------------------------------------------------------
struct Variant {
    const char *name;
    int precision;
    bool cluster;  // reduce through a thread-block cluster (else global partials + stage_finish)
    bool cull;     // skip j groups whose box is beyond the cutoff from the tile's (group_bounds first)
    int nt;        // threads per CTA
    int tile;      // particles per i tile
    size_t smem;
    const void *fn;
    cudaError_t (*launch)(const cudaLaunchConfig_t *, const StageParams &);
};

template <int NW, int ILP, int TC, bool CL, bool CULL>
cudaError_t launch_fp32c(const cudaLaunchConfig_t *cfg, const StageParams &P) {
    return cudaLaunchKernelEx(cfg, pair_stage_fp32c<NW, ILP, TC, CL, CULL>, P);
}
template <int NI, int G, int ILP, int JT>
cudaError_t launch_fp64(const cudaLaunchConfig_t *cfg, const StageParams &P) {
    return cudaLaunchKernelEx(cfg, pair_stage_fp64<NI, G, ILP, JT>, P);
}

#define DM_FP32C_VARIANT(NW, ILP, TC, CL)                                                        \
    {"fp32c<" #NW "," #ILP "," #TC "," #CL ">", DM_FP32C, CL, false, NW * 32, 32 * ILP,           \
     Fp32cSmem<NW, ILP, TC>::bytes, (const void *)pair_stage_fp32c<NW, ILP, TC, CL, false>,       \
     launch_fp32c<NW, ILP, TC, CL, false>}
#define DM_FP32C_CULL_VARIANT(NW, ILP, TC, CL)                                                   \
    {"fp32c<" #NW "," #ILP "," #TC "," #CL ",cull>", DM_FP32C, CL, true, NW * 32, 32 * ILP,      \
     Fp32cSmem<NW, ILP, TC>::bytes, (const void *)pair_stage_fp32c<NW, ILP, TC, CL, true>,        \
     launch_fp32c<NW, ILP, TC, CL, true>}

const Variant kVariants[] = {
    DM_FP32C_VARIANT(8, 4, 256, true),
    DM_FP32C_VARIANT(8, 4, 256, false),
    DM_FP32C_VARIANT(4, 4, 256, true),
    DM_FP32C_VARIANT(4, 4, 256, false),
    DM_FP32C_VARIANT(16, 4, 256, false),
    DM_FP32C_VARIANT(8, 2, 256, false),
    DM_FP32C_CULL_VARIANT(8, 4, 256, false),
    DM_FP32C_CULL_VARIANT(4, 4, 256, false),
    DM_FP32C_CULL_VARIANT(8, 2, 256, false),
    DM_FP32C_CULL_VARIANT(4, 2, 128, false),
    DM_FP32C_CULL_VARIANT(8, 4, 256, true),
    {"fp64<128,2,2,512>", DM_FP64, true, false, kNI64 * kG64, kNI64 * kILP64,
     Fp64Smem<kNI64, kG64, kILP64>::bytes(kJT64),
     (const void *)pair_stage_fp64<kNI64, kG64, kILP64, kJT64>, launch_fp64<kNI64, kG64, kILP64, kJT64>},
};
constexpr int kNumVariants = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
constexpr int kDefaultVariant32 = 0;
constexpr int kDefaultVariant64 = kNumVariants - 1;
constexpr int kMaxSplitGlobal = 64;

int ensure_kernel_attrs(dm_ctx *ctx) {
    static bool done[64] = {false};
    int dev = ctx->device;
    if (dev < 0 || dev >= 64) dev = 0;
    if (done[dev]) return DM_OK;
    for (int v = 0; v < kNumVariants; v++) {
        const Variant &k = kVariants[v];
        if (k.cluster)
            DM_CUDA(ctx, cudaFuncSetAttribute(k.fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        DM_CUDA(ctx, cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem));
    }
    DM_CUDA(ctx, cudaFuncSetAttribute(sort_cluster<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sort_cluster_smem<8>()));
    DM_CUDA(ctx, cudaFuncSetAttribute(sort_cluster<16>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    DM_CUDA(ctx, cudaFuncSetAttribute(sort_cluster<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sort_cluster_smem<16>()));
    done[dev] = true;
    return DM_OK;
}

template <int CTAS>
cudaLaunchConfig_t sort_cluster_cfg(cudaStream_t s, cudaLaunchAttribute *attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(CTAS);
    cfg.blockDim = dim3(kSortClusterThreads);
    cfg.dynamicSmemBytes = sort_cluster_smem<CTAS>();
    cfg.stream = s;
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    attr[1].id = cudaLaunchAttributeClusterDimension;
    attr[1].val.clusterDim.x = CTAS;
    attr[1].val.clusterDim.y = 1;
    attr[1].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
    return cfg;
}

// Blocks of the one-cluster sort on this device: 16 (half the elements per
// SM of 8) when a 16-block cluster of it can be scheduled, else 8;
// DM_SORT_CLUSTER_CTAS=8 keeps 8.
int choose_sort_ctas(dm_ctx *ctx) {
    if (ctx->sort_ctas) return DM_OK;
    int rc = ensure_kernel_attrs(ctx);
    if (rc) return rc;
    const char *e = getenv("DM_SORT_CLUSTER_CTAS");
    int ctas = (e && atoi(e) == 8) ? 8 : 16;
    if (ctas == 16) {
        cudaLaunchAttribute attr[2];
        cudaLaunchConfig_t cfg = sort_cluster_cfg<16>(ctx->stream, attr);
        int nc = 0;
        if (cudaOccupancyMaxActiveClusters(&nc, sort_cluster<16>, &cfg) != cudaSuccess || nc < 1) {
            cudaGetLastError();
            ctas = 8;
        }
    }
    ctx->sort_ctas = ctas;
    return DM_OK;
}

// Launch of a kernel that starts with pdl_wait(): it may be scheduled while
// the previous kernel in the stream finishes.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                       Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

int variant_groups(const Variant &k) { return k.precision == DM_FP64 ? kG64 : k.nt / 32; }

// attr must hold 2 entries: programmatic serialization (see pdl_wait) and,
// for cluster variants, the cluster shape.
cudaLaunchConfig_t make_cfg(dm_ctx *ctx, const Variant &k, int ntiles, int S, cudaLaunchAttribute *attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ntiles * S, 1, 1);
    cfg.blockDim = dim3(k.nt, 1, 1);
    cfg.dynamicSmemBytes = k.smem;
    cfg.stream = ctx->stream;
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (k.cluster) {
        attr[1].id = cudaLaunchAttributeClusterDimension;
        attr[1].val.clusterDim.x = S;
        attr[1].val.clusterDim.y = 1;
        attr[1].val.clusterDim.z = 1;
        cfg.numAttrs = 2;
    }
    return cfg;
}

// j split S for a variant from a cost model: all CTAs do equal work (1/S of a
// tile), so a launch takes as long as its busiest SM.  With X co-resident
// clusters (or CTAs) the tiles run in ceil(ntiles / X) waves and within a
// wave the busiest SM holds ceil(CTAs_in_wave / num_sms) CTAs.  Cost = sum
// over waves of that count / S; on ties (within 2%) the larger S wins, since
// more co-resident CTAs hide latency better.
int model_split(dm_ctx *ctx, const Variant &k, int n, int n_pad) {
    const int ntiles = (n + k.tile - 1) / k.tile;
    const int smax = k.cluster ? 16 : kMaxSplitGlobal;
    int best_s = 1;
    double best_cost = 1e300;
    for (int S = 1; S <= smax; S++) {
        if (S > 1 && n_pad / S < 64 * variant_groups(k)) break;
        int slots = 0;
        if (k.cluster) {
            cudaLaunchAttribute attr[2];
            cudaLaunchConfig_t cfg = make_cfg(ctx, k, ntiles, S, attr);
            if (cudaOccupancyMaxActiveClusters(&slots, k.fn, &cfg) != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
        } else {
            int per_sm = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.fn, k.nt, k.smem) != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
            slots = per_sm * ctx->num_sms / S;  // co-resident "tiles"
        }
        if (slots <= 0) continue;
        double cost = 0.0;
        for (int left = ntiles; left > 0; left -= slots) {
            const int in_wave = std::min(left, slots) * S;
            cost += (double)((in_wave + ctx->num_sms - 1) / ctx->num_sms) / S;
        }
        if (cost <= best_cost * 1.02) {
            best_cost = std::min(best_cost, cost);
            best_s = S;
        }
    }
    return best_s;
}

int ensure_partial(dm_cloud *c, int S) {
    if (S <= c->partial_cap) return DM_OK;
    dm_ctx *ctx = c->ctx;
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (c->partial) cudaFree(c->partial);
    c->partial = nullptr;
    c->partial_cap = 0;
    cudaError_t e = cudaMalloc((void **)&c->partial, (size_t)S * 2 * c->n_pad * sizeof(float2));
    if (e != cudaSuccess)
        return ctx->fail(DM_ERR_NOMEM, "partial-sum buffer (%d x %d): %s", S, c->n_pad, cudaGetErrorString(e));
    c->partial_cap = S;
    c->drop_graphs();
    return DM_OK;
}

// One stage: the pair kernel (+ stage_finish for non-cluster variants).
int launch_variant(dm_cloud *c, int vi, int S, int stage, int mode, double dt, const double *dt_dev) {
    dm_ctx *ctx = c->ctx;
    const Variant &k = kVariants[vi];
    StageParams P = make_stage_params(c, stage, mode, dt, dt_dev);
    P.split = S;
    P.partial = c->partial;
    const int ntiles = (c->n + k.tile - 1) / k.tile;
    cudaLaunchAttribute attr[2];
    cudaLaunchConfig_t cfg = make_cfg(ctx, k, ntiles, S, attr);
    const int br = (mode == kModeForceOnly) ? c->fo_buf : (stage - 1) & 1;  // buffer read
    if (k.cull && !c->boxes_valid[br]) {  // boxes of the buffer this stage reads
        DM_CUDA(ctx, launch_pdl(group_bounds, dim3((c->n_pad + 255) / 256), dim3(256), 0, ctx->stream, c->d, br));
        ctx->launches++;
        c->boxes_valid[br] = true;
    }
    // profiling (dm_ctx_profile_enable): CUDA events around the pair launch
    // alone (a cluster variant's launch includes its epilogue)
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (ctx->prof) {
        if (ctx->prof_used == ctx->prof_events.size()) {
            cudaEvent_t a, b;
            DM_CUDA(ctx, cudaEventCreate(&a));
            DM_CUDA(ctx, cudaEventCreate(&b));
            ctx->prof_events.push_back({a, b});
        }
        e0 = ctx->prof_events[ctx->prof_used].first;
        e1 = ctx->prof_events[ctx->prof_used].second;
        ctx->prof_used++;
        DM_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
    }
    DM_CUDA(ctx, k.launch(&cfg, P));
    ctx->launches++;
    if (ctx->prof) {
        DM_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
        ctx->prof_launches++;
        ctx->prof_pairs += (double)c->n * (double)(c->n - 1);
    }
    if (!k.cluster) {
        // stage_finish also writes the group boxes of the buffer the stage writes
        P.box_out = (mode != kModeForceOnly) ? 1 : 0;
        if (P.f.flags & ~kBasicForces)
            DM_CUDA(ctx, launch_pdl(stage_finish, dim3((c->n + 63) / 64), dim3(64), 0, ctx->stream, P));
        else  // one thread per particle and axis, one block per 32-particle group
            DM_CUDA(ctx, launch_pdl(stage_finish_axes, dim3(2 * ((c->n + 63) / 64)), dim3(64), 0, ctx->stream, P));
        ctx->launches++;
    }
    if (mode != kModeForceOnly) c->boxes_valid[stage & 1] = !k.cluster;
    return DM_OK;
}

int tune_precision(dm_cloud *c, int precision);
int reorder(dm_cloud *c);

// One launch of the fused pair + stage kernel(s) with the cloud's tuned
// variant and split.
int launch_stage(dm_cloud *c, int precision, int stage, int mode, double dt, const double *dt_dev) {
    dm_ctx *ctx = c->ctx;
    int rc = ensure_kernel_attrs(ctx);
    if (rc) return rc;
    const int pi = precision == DM_FP32C ? 1 : 0;
    if (c->tuned_variant[pi] < 0) {
        rc = tune_precision(c, precision);
        if (rc) return rc;
    }
    const int vi = c->tuned_variant[pi];
    const int S = c->split[pi];
    return launch_variant(c, vi, S, stage, mode, dt, dt_dev);
}

// Autotuner: times every variant of this precision over a set of splits on
// THIS cloud (force-only launches: no state changes), keeps the fastest.
// Results are cached per (precision, n) in the context.  When disabled, the
// default variant and the cost-model split are used.
int tune_precision(dm_cloud *c, int precision) {
    dm_ctx *ctx = c->ctx;
    const int pi = precision == DM_FP32C ? 1 : 0;
    const long long key = ((long long)c->n << 1) | pi;
    auto hit = ctx->tune_cache.find(key);
    if (hit != ctx->tune_cache.end()) {
        c->tuned_variant[pi] = hit->second.first;
        c->split[pi] = hit->second.second;
        if (!kVariants[c->tuned_variant[pi]].cluster) return ensure_partial(c, c->split[pi]);
        return DM_OK;
    }
    const int defv = precision == DM_FP32C ? kDefaultVariant32 : kDefaultVariant64;
    int best_v = defv, best_s = model_split(ctx, kVariants[defv], c->n, c->n_pad);
    if (ctx->autotune) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        DM_CUDA(ctx, cudaStreamIsCapturing(ctx->stream, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            return ctx->fail(DM_ERR_STATE, "autotuning needs an uncaptured stream (run one step first)");
        if (c->order_dirty) {  // tune on the particle order the steps will see
            int rc = reorder(c);
            if (rc) return rc;
        }
        // Time every candidate on two states: the cloud as it is (buffer 0)
        // and, unless it is dense already, a copy squeezed about its centre
        // so that ~30% of the pairs are inside the cutoff (buffer 1).  A
        // trajectory passes through both kinds (a confined cloud collapses
        // and re-expands), and the best shape differs between them.
        const bool big = (double)c->n * c->n > 4e9;  // ~64k particles: keep tuning short
        int nstates = 1;
        if (!big && c->d.rc2 > 0.0 && std::isfinite(c->d.rc2)) {
            double v[4];  // bounding box min x, min y, max x, max y
            DM_CUDA(ctx, cudaMemcpyAsync(v, c->sort.box + 4, sizeof v, cudaMemcpyDeviceToHost, ctx->stream));
            DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            const double half = 0.5 * std::max(v[2] - v[0], v[3] - v[1]);
            const double lam = 1.8 * std::sqrt(c->d.rc2) / half;
            if (std::isfinite(half) && half > 0.0 && lam < 0.9) {
                c->boxes_valid[1] = false;
                tune_compress<<<(c->n + 255) / 256, 256, 0, ctx->stream>>>(c->d, 0.5 * (v[0] + v[2]),
                                                                            0.5 * (v[1] + v[3]), lam);
                DM_CUDA(ctx, cudaGetLastError());
                nstates = 2;
            }
        }
        cudaEvent_t a, b;
        DM_CUDA(ctx, cudaEventCreate(&a));
        DM_CUDA(ctx, cudaEventCreate(&b));
        float best_ms = 1e30f;
        const char *ev = getenv("DM_TUNE_VERBOSE");  // per-candidate timings on stderr
        const bool verbose = ev && ev[0] && ev[0] != '0';
        for (int vi = 0; vi < kNumVariants; vi++) {
            const Variant &k = kVariants[vi];
            if (k.precision != precision) continue;
            const int sm = model_split(ctx, k, c->n, c->n_pad);
            std::vector<int> cands = {sm};
            const int extra_c[] = {1, 2, 3, 4, 6, 8, 12, 16};
            const int extra_g[] = {1, 2, 4, 8, 12, 16, 24, 32, 48, 64};
            if (!big) {
                if (k.cluster) cands.insert(cands.end(), std::begin(extra_c), std::end(extra_c));
                else cands.insert(cands.end(), std::begin(extra_g), std::end(extra_g));
            }
            std::sort(cands.begin(), cands.end());
            cands.erase(std::unique(cands.begin(), cands.end()), cands.end());
            for (int S : cands) {
                if (S > 1 && c->n_pad / S < 64 * variant_groups(k)) continue;
                if (k.cluster) {
                    int nc = 0;
                    cudaLaunchAttribute attr[2];
                    cudaLaunchConfig_t cfg = make_cfg(ctx, k, (c->n + k.tile - 1) / k.tile, S, attr);
                    if (cudaOccupancyMaxActiveClusters(&nc, k.fn, &cfg) != cudaSuccess || nc <= 0) {
                        cudaGetLastError();
                        continue;
                    }
                } else {
                    int rc = ensure_partial(c, S);
                    if (rc) return rc;
                }
                const int reps = big ? 1 : 3;
                float ms = 0.0f, ms_state[2] = {0.0f, 0.0f};
                for (int st = 0; st < nstates; st++) {
                    c->fo_buf = st;
                    int rc = launch_variant(c, vi, S, 1, kModeForceOnly, 0.0, nullptr);  // warm-up
                    if (!rc) rc = cudaEventRecord(a, ctx->stream) == cudaSuccess ? DM_OK : DM_ERR_CUDA;
                    for (int r = 0; r < reps && !rc; r++) rc = launch_variant(c, vi, S, 1, kModeForceOnly, 0.0, nullptr);
                    if (!rc) rc = cudaEventRecord(b, ctx->stream) == cudaSuccess ? DM_OK : DM_ERR_CUDA;
                    if (!rc) rc = cudaEventSynchronize(b) == cudaSuccess ? DM_OK : DM_ERR_CUDA;
                    c->fo_buf = 0;
                    if (rc) return rc == DM_ERR_CUDA ? ctx->fail(rc, "autotuner timing failed") : rc;
                    float one = 0.0f;
                    DM_CUDA(ctx, cudaEventElapsedTime(&one, a, b));
                    ms += one;
                    ms_state[st] = one / reps;
                }
                ms /= reps;
                if (verbose)
                    fprintf(stderr, "dm autotune n=%d %s split %d: %.4f ms (state) %.4f ms (dense copy)\n", c->n,
                            k.name, S, ms_state[0], ms_state[1]);
                if (ms < best_ms) {
                    best_ms = ms;
                    best_v = vi;
                    best_s = S;
                }
            }
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    c->tuned_variant[pi] = best_v;
    c->split[pi] = best_s;
    ctx->tune_cache[key] = {best_v, best_s};
    if (!kVariants[best_v].cluster) return ensure_partial(c, best_s);
    return DM_OK;
}

// Puts the cloud in Morton order (dm_sort.cuh); graph-capturable.
int reorder(dm_cloud *c) {
    dm_ctx *ctx = c->ctx;
    cudaStream_t s = ctx->stream;
    const int n = c->n;
    const int grid = (n + 255) / 256;
    SortScratch &z = c->sort;
    int cur = 0;
    if (n <= kSmallSortMax) {  // one cluster launch sorts and rewrites the cloud in place
        int rc = choose_sort_ctas(ctx);
        if (rc) return rc;
        cudaLaunchAttribute attr[2];
        const float4 *pa0 = c->d.pa[0];
        if (ctx->sort_ctas == 16) {
            const cudaLaunchConfig_t cfg = sort_cluster_cfg<16>(s, attr);
            DM_CUDA(ctx, cudaLaunchKernelEx(&cfg, sort_cluster<16>, pa0, c->d, z));
        } else {
            const cudaLaunchConfig_t cfg = sort_cluster_cfg<8>(s, attr);
            DM_CUDA(ctx, cudaLaunchKernelEx(&cfg, sort_cluster<8>, pa0, c->d, z));
        }
        c->boxes_valid[0] = true;  // written by sort_cluster
        c->boxes_valid[1] = false;
        DM_CUDA(ctx, cudaGetLastError());
        ctx->launches += 1;
        c->order_dirty = false;
        return DM_OK;
    } else {
        const int mblocks = std::min(grid, kMomentBlocks);
        sort_moments<<<mblocks, 256, 0, s>>>(c->d.x, c->d.y, n, z.moments);
        sort_box<<<1, 32, 0, s>>>(z.moments, mblocks, c->d.x, c->d.y, z.box);
        sort_keys<<<grid, 256, 0, s>>>(c->d.x, c->d.y, n, z.box, z.keys[0], z.vals[0]);
        for (int shift = 0; shift < kSortBits; shift += kSortDigitBits) {
            radix_hist<<<c->sort_blocks, kSortThreads, 0, s>>>(z.keys[cur], n, shift, z.hist);
            radix_scan<<<1, 1024, 0, s>>>(z.hist, kSortBuckets * c->sort_blocks);
            radix_scatter<<<c->sort_blocks, kSortThreads, 0, s>>>(z.keys[cur], z.vals[cur], z.keys[cur ^ 1],
                                                                   z.vals[cur ^ 1], n, shift, z.hist);
            cur ^= 1;
        }
        ctx->launches += 3 + 3 * (kSortBits / kSortDigitBits);
    }
    permute_gather<<<grid, 256, 0, s>>>(c->d, z.vals[cur], z);
    permute_commit<<<grid, 256, 0, s>>>(c->d, z);
    init_positions<<<(c->n_pad + 255) / 256, 256, 0, s>>>(c->d);
    c->boxes_valid[0] = c->boxes_valid[1] = false;
    DM_CUDA(ctx, cudaGetLastError());
    ctx->launches += 3;
    c->order_dirty = false;
    return DM_OK;
}

int enqueue_steps(dm_cloud *c, int nsteps, double dt, int precision) {
    for (int s = 0; s < nsteps; s++) {
        if (c->order_dirty ||
            (c->reorder_interval > 0 && c->host_steps % (unsigned)c->reorder_interval == 0)) {
            int rc = reorder(c);
            if (rc) return rc;
        }
        for (int st = 1; st <= c->order; st++) {
            int rc = launch_stage(c, precision, st, kModeStep, dt, nullptr);
            if (rc) return rc;
        }
        c->host_steps++;
    }
    return DM_OK;
}

int run_steps(dm_cloud *c, int nsteps, double dt, int precision) {
    dm_ctx *ctx = c->ctx;
    if (ctx->prof || nsteps < kGraphSteps) return enqueue_steps(c, nsteps, dt, precision);
    if (c->graph_stream != ctx->stream) {
        c->drop_graphs();
        c->graph_stream = ctx->stream;
    }
    // the captured step sequence re-sorts at fixed positions: align the
    // host step counter and clear a pending re-sort first
    while (nsteps > 0 && (c->order_dirty ||
                          (c->reorder_interval > 0 && c->host_steps % kGraphSteps != 0))) {
        int rc = enqueue_steps(c, 1, dt, precision);
        if (rc) return rc;
        nsteps--;
    }
    if (nsteps < kGraphSteps) return enqueue_steps(c, nsteps, dt, precision);
    const GraphKey key{precision, kGraphSteps, dt};
    auto it = c->graphs.find(key);
    if (it == c->graphs.end()) {
        cudaGraph_t g = nullptr;
        const unsigned long long saved = c->host_steps;
        const long long saved_launches = ctx->launches;
        DM_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_steps(c, kGraphSteps, dt, precision);
        cudaError_t ec = cudaStreamEndCapture(ctx->stream, &g);
        c->host_steps = saved;  // capture recorded the steps, it did not run them
        c->graph_launches = ctx->launches - saved_launches;
        ctx->launches = saved_launches;
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (ec != cudaSuccess) return ctx->fail(DM_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ec));
        cudaGraphExec_t ge = nullptr;
        ec = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (ec != cudaSuccess) return ctx->fail(DM_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(ec));
        it = c->graphs.emplace(key, ge).first;
    }
    const int reps = nsteps / kGraphSteps;
    for (int r = 0; r < reps; r++) {
        DM_CUDA(ctx, cudaGraphLaunch(it->second, ctx->stream));
        c->host_steps += kGraphSteps;
        ctx->launches += c->graph_launches;
    }
    return enqueue_steps(c, nsteps - reps * kGraphSteps, dt, precision);
}

// The device's own address of a caller's host buffer when the device may
// dereference it (page-locked host memory: cudaHostAlloc, cudaMallocHost,
// cudaHostRegister, torch's pin_memory), else nullptr: then the buffer is
// copied by DMA.  On GB300 such buffers are read and written over
// NVLink-C2C by the copy kernel, one launch for all four arrays.
const void *device_view(const void *p) {
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (a.type == cudaMemoryTypeHost && a.devicePointer) ? a.devicePointer : nullptr;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int dm_version(void) { return DM_ABI_VERSION; }

int dm_ctx_create(int device, dm_ctx **out) {
    if (!out) {
        g_create_error = "dm_ctx_create: out is NULL";
        return DM_ERR_ARG;
    }
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || device < 0 || device >= count) {
        g_create_error = std::string("dm_ctx_create: no CUDA device ") + std::to_string(device) +
                         (e != cudaSuccess ? std::string(": ") + cudaGetErrorString(e) : std::string());
        return e != cudaSuccess ? DM_ERR_CUDA : DM_ERR_ARG;
    }
    dm_ctx *ctx = new dm_ctx();
    ctx->device = device;
    e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    int major = 0, minor = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
    if (e != cudaSuccess) {
        g_create_error = std::string("dm_ctx_create: ") + cudaGetErrorString(e);
        delete ctx;
        return DM_ERR_CUDA;
    }
    if (major * 10 + minor != 103) {
        g_create_error = "dm_ctx_create: this build targets sm_103a (GB300); device is sm_" +
                         std::to_string(major) + std::to_string(minor);
        cudaStreamDestroy(ctx->own_stream);
        delete ctx;
        return DM_ERR_UNSUPPORTED;
    }
    ctx->stream = ctx->own_stream;
    *out = ctx;
    return DM_OK;
}

int dm_ctx_destroy(dm_ctx *ctx) {
    if (!ctx) return DM_ERR_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto &p : ctx->prof_events) {
        cudaEventDestroy(p.first);
        cudaEventDestroy(p.second);
    }
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    if (ctx->h_err) cudaFreeHost(ctx->h_err);
    delete ctx;
    return DM_OK;
}

int dm_ctx_set_stream(dm_ctx *ctx, void *stream) {
    if (!ctx) return DM_ERR_ARG;
    ctx->stream = (cudaStream_t)stream;  // NULL: the CUDA default (legacy) stream
    return DM_OK;
}

int dm_ctx_reset_stream(dm_ctx *ctx) {
    if (!ctx) return DM_ERR_ARG;
    ctx->stream = ctx->own_stream;
    return DM_OK;
}

int dm_ctx_synchronize(dm_ctx *ctx) {
    if (!ctx) return DM_ERR_ARG;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return DM_OK;
}

int dm_last_error(const dm_ctx *ctx, char *buf, size_t len) {
    if (!buf || len == 0) return DM_ERR_ARG;
    const std::string &s = ctx ? ctx->err : g_create_error;
    snprintf(buf, len, "%s", s.c_str());
    return DM_OK;
}

int dm_ctx_launch_count(dm_ctx *ctx, long long *count) {
    if (!ctx || !count) return DM_ERR_ARG;
    *count = ctx->launches;
    return DM_OK;
}

int dm_ctx_profile_enable(dm_ctx *ctx, int enable) {
    if (!ctx) return DM_ERR_ARG;
    ctx->prof = enable != 0;
    ctx->prof_used = 0;
    ctx->prof_pairs = 0.0;
    ctx->prof_launches = 0;
    return DM_OK;
}

int dm_ctx_profile_read(dm_ctx *ctx, double *total_ms, long long *launches, double *pairs) {
    if (!ctx) return DM_ERR_ARG;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double tot = 0.0;
    for (size_t k = 0; k < ctx->prof_used; k++) {
        float ms = 0.0f;
        DM_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->prof_events[k].first, ctx->prof_events[k].second));
        tot += ms;
    }
    if (total_ms) *total_ms = tot;
    if (launches) *launches = ctx->prof_launches;
    if (pairs) *pairs = ctx->prof_pairs;
    ctx->prof_used = 0;
    ctx->prof_pairs = 0.0;
    ctx->prof_launches = 0;
    return DM_OK;
}

int dm_probe_peak(dm_ctx *ctx, int kind, double *tflops) {
    if (!ctx || !tflops || (kind != 0 && kind != 1)) return DM_ERR_ARG;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    void *out = nullptr;
    DM_CUDA(ctx, cudaMalloc(&out, 16));
    cudaEvent_t a, b;
    DM_CUDA(ctx, cudaEventCreate(&a));
    DM_CUDA(ctx, cudaEventCreate(&b));
    const int threads = 256, blocks = ctx->num_sms * 8;
    const int iters = (kind == 0) ? 8192 : 256;
    double best = 0.0;
    for (int rep = 0; rep < 4; rep++) {
        DM_CUDA(ctx, cudaEventRecord(a, ctx->stream));
        if (kind == 0)
            fma_probe<float><<<blocks, threads, 0, ctx->stream>>>((float *)out, iters, 0.999f, 0.001f);
        else
            fma_probe<double><<<blocks, threads, 0, ctx->stream>>>((double *)out, iters, 0.999, 0.001);
        DM_CUDA(ctx, cudaGetLastError());
        DM_CUDA(ctx, cudaEventRecord(b, ctx->stream));
        DM_CUDA(ctx, cudaEventSynchronize(b));
        float ms = 0.0f;
        DM_CUDA(ctx, cudaEventElapsedTime(&ms, a, b));
        const double flops = 2.0 * 16.0 * (double)iters * threads * (double)blocks;
        best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    *tflops = best;
    return DM_OK;
}

int dm_cloud_create(dm_ctx *ctx, int n, const double *x, const double *y, const double *vx,
                    const double *vy, const double *q, const double *m, dm_cloud **out) {
    if (!ctx || !out || n < 1 || !x || !y || !vx || !vy || !q || !m)
        return ctx ? ctx->fail(DM_ERR_ARG, "dm_cloud_create: bad argument") : DM_ERR_ARG;
    *out = nullptr;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    dm_cloud *c = new dm_cloud();
    c->ctx = ctx;
    c->n = n;
    c->n_pad = (n + 63) & ~63;
    // a re-sort costs less than the pair sweeps it saves every step (a confined
    // cloud's particles cross many cutoffs per step while it collapses, close
    // pairs of a random cloud are thrown out, and a stale order inflates
    // every group box)
    c->reorder_interval = 1;
    c->coulomb = 1.0 / (4.0 * M_PI * 8.8541878E-12);
    c->d.coulomb = c->coulomb;
    c->d.rc2 = (10.0 / 2e4) * (10.0 / 2e4);  // default kappa until set_forces
    const size_t nd = align256((size_t)c->n_pad * sizeof(double));
    const size_t nf4 = align256((size_t)c->n_pad * sizeof(float4));
    const size_t ni = align256((size_t)c->n_pad * sizeof(int));
    c->sort_blocks = (n + kSortPerBlock - 1) / kSortPerBlock;
    const size_t nh = align256((size_t)kSortBuckets * c->sort_blocks * sizeof(uint32_t));
    const size_t ngb = align256((size_t)(c->n_pad / 32) * sizeof(float4));
    const size_t total = nd * (6 + 2 + 8 + 4 + 2 + 6) + nf4 * 4 + ngb * 2 + ni * 6 + nh + 1024 + 512 +
                         align256(sizeof(double) * kMomentBlocks * kMomentFields);
    cudaError_t e = cudaMalloc(&c->block, total);
    if (e != cudaSuccess) {
        delete c;
        return ctx->fail(DM_ERR_NOMEM, "dm_cloud_create: cudaMalloc(%zu) failed: %s", total, cudaGetErrorString(e));
    }
    char *p = (char *)c->block;
    auto takeD = [&]() { double *r = (double *)p; p += nd; return r; };
    auto takeF4 = [&]() { float4 *r = (float4 *)p; p += nf4; return r; };
    c->d.n = n;
    c->d.n_pad = c->n_pad;
    c->d.x = takeD(); c->d.y = takeD(); c->d.vx = takeD(); c->d.vy = takeD();
    c->d.q = takeD(); c->d.m = takeD();
    c->d.vxc = takeD(); c->d.vyc = takeD();
    for (int k = 0; k < 4; k++) c->d.a1[k] = takeD();
    for (int k = 0; k < 4; k++) c->d.a23[k] = takeD();
    for (int b = 0; b < 2; b++) { c->d.px[b] = takeD(); c->d.py[b] = takeD(); }
    c->d_fx = takeD();
    c->d_fy = takeD();
    for (int b = 0; b < 2; b++) { c->d.pa[b] = takeF4(); c->d.pb[b] = takeF4(); }
    for (int b = 0; b < 2; b++) { c->d.gbox[b] = (float4 *)p; p += ngb; }
    c->d.eval_pairs = (unsigned long long *)p; p += 256;
    c->d.step_ctr = (unsigned long long *)p; p += 256;
    c->d.time = (double *)(c->d.step_ctr + 4);  // same 256-byte slot, bytes 32-47
    c->d.err = (int *)p; p += 256;
    c->d_dt = (double *)p; p += 256;
    c->d_min = (unsigned int *)p; c->d_dmin = (float *)(p + 64); p += 256;
    auto takeI = [&]() { int *r = (int *)p; p += ni; return r; };
    c->d.orig = takeI();
    c->sort.keys[0] = (uint32_t *)takeI();
    c->sort.keys[1] = (uint32_t *)takeI();
    c->sort.vals[0] = takeI();
    c->sort.vals[1] = takeI();
    c->sort.orig_stage = takeI();
    for (int k = 0; k < 6; k++) c->sort.stage[k] = takeD();
    c->sort.hist = (uint32_t *)p; p += nh;
    c->sort.box = (double *)p; p += 256;
    c->sort.moments = (double *)p; p += align256(sizeof(double) * kMomentBlocks * kMomentFields);
    cudaStream_t s = ctx->stream;
    const size_t bytes = (size_t)n * sizeof(double);
    e = cudaMemsetAsync(c->block, 0, total, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->d.x, x, bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->d.y, y, bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->d.vx, vx, bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->d.vy, vy, bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->d.q, q, bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->d.m, m, bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        set_identity<<<(n + 255) / 256, 256, 0, s>>>(c->d.orig, n);
        init_positions<<<(c->n_pad + 255) / 256, 256, 0, s>>>(c->d);
        c->boxes_valid[0] = c->boxes_valid[1] = false;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaFree(c->block);
        delete c;
        return ctx->fail(DM_ERR_CUDA, "dm_cloud_create: %s", cudaGetErrorString(e));
    }
    c->f.flags = kConfinement | kDrag | kShieldedCoulomb;
    c->f.shielding = 2e4;
    c->f.confine = 100;
    c->f.gamma = 10.0;
    *out = c;
    return DM_OK;
}

int dm_cloud_destroy(dm_cloud *c) {
    if (!c) return DM_ERR_ARG;
    cudaSetDevice(c->ctx->device);
    cudaStreamSynchronize(c->ctx->stream);
    c->drop_graphs();
    cudaFree(c->block);
    delete c;
    return DM_OK;
}

int dm_cloud_size(const dm_cloud *c, int *n) {
    if (!c || !n) return DM_ERR_ARG;
    *n = c->n;
    return DM_OK;
}

int dm_cloud_upload(dm_cloud *c, const double *x, const double *y, const double *vx, const double *vy) {
    if (!c) return DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    if (!x || !y || !vx || !vy) return ctx->fail(DM_ERR_ARG, "dm_cloud_upload: NULL array");
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t bytes = (size_t)c->n * sizeof(double);
    // caller order -> staging -> the cloud's current internal order (charges,
    // masses and the order stay; stage buffer 0 and its boxes are rewritten)
    double **st = c->sort.stage;
    const void *dv[4] = {device_view(x), device_view(y), device_view(vx), device_view(vy)};
    if (dv[0] && dv[1] && dv[2] && dv[3]) {
        copy4<<<(c->n + 255) / 256, 256, 0, ctx->stream>>>(c->n, (const double *)dv[0], (const double *)dv[1],
                                                           (const double *)dv[2], (const double *)dv[3], st[0],
                                                           st[1], st[2], st[3], nullptr, nullptr);
        DM_CUDA(ctx, cudaGetLastError());
        ctx->launches += 1;
    } else {
        DM_CUDA(ctx, cudaMemcpyAsync(st[0], x, bytes, cudaMemcpyHostToDevice, ctx->stream));
        DM_CUDA(ctx, cudaMemcpyAsync(st[1], y, bytes, cudaMemcpyHostToDevice, ctx->stream));
        DM_CUDA(ctx, cudaMemcpyAsync(st[2], vx, bytes, cudaMemcpyHostToDevice, ctx->stream));
        DM_CUDA(ctx, cudaMemcpyAsync(st[3], vy, bytes, cudaMemcpyHostToDevice, ctx->stream));
    }
    upload_internal_order<<<(c->n_pad + 255) / 256, 256, 0, ctx->stream>>>(c->d, c->sort);
    c->boxes_valid[0] = true;
    c->boxes_valid[1] = false;
    DM_CUDA(ctx, cudaGetLastError());
    ctx->launches += 1;
    c->order_dirty = true;  // the uploaded positions may be far from the old order
    return DM_OK;
}

int dm_cloud_download(dm_cloud *c, double *x, double *y, double *vx, double *vy) {
    if (!c) return DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t bytes = (size_t)c->n * sizeof(double);
    double **st = c->sort.stage;
    scatter_to_caller<<<(c->n + 255) / 256, 256, 0, ctx->stream>>>(
        c->d.orig, c->n, c->d.x, c->d.y, c->d.vx, c->d.vy, st[0], st[1], st[2], st[3]);
    DM_CUDA(ctx, cudaGetLastError());
    ctx->launches++;
    // the error flags come back with the state: one synchronisation
    if (!ctx->h_err) DM_CUDA(ctx, cudaMallocHost((void **)&ctx->h_err, sizeof(int)));
    const void *dv[4] = {device_view(x), device_view(y), device_view(vx), device_view(vy)};
    int *err_dv = (int *)device_view(ctx->h_err);
    if (dv[0] && dv[1] && dv[2] && dv[3] && err_dv) {
        copy4<<<(c->n + 255) / 256, 256, 0, ctx->stream>>>(c->n, st[0], st[1], st[2], st[3], (double *)dv[0],
                                                           (double *)dv[1], (double *)dv[2], (double *)dv[3],
                                                           c->d.err, err_dv);
        DM_CUDA(ctx, cudaGetLastError());
        ctx->launches++;
    } else {
        if (x) DM_CUDA(ctx, cudaMemcpyAsync(x, st[0], bytes, cudaMemcpyDeviceToHost, ctx->stream));
        if (y) DM_CUDA(ctx, cudaMemcpyAsync(y, st[1], bytes, cudaMemcpyDeviceToHost, ctx->stream));
        if (vx) DM_CUDA(ctx, cudaMemcpyAsync(vx, st[2], bytes, cudaMemcpyDeviceToHost, ctx->stream));
        if (vy) DM_CUDA(ctx, cudaMemcpyAsync(vy, st[3], bytes, cudaMemcpyDeviceToHost, ctx->stream));
        DM_CUDA(ctx, cudaMemcpyAsync(ctx->h_err, c->d.err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    }
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return device_error_status(ctx, c, *ctx->h_err);
}

int dm_cloud_set_charge_mass(dm_cloud *c, const double *q, const double *m) {
    if (!c) return DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t bytes = (size_t)c->n * sizeof(double);
    double **st = c->sort.stage;
    // caller order -> staging -> internal order
    if (q) DM_CUDA(ctx, cudaMemcpyAsync(st[4], q, bytes, cudaMemcpyHostToDevice, ctx->stream));
    if (m) DM_CUDA(ctx, cudaMemcpyAsync(st[5], m, bytes, cudaMemcpyHostToDevice, ctx->stream));
    gather_from_caller<<<(c->n + 255) / 256, 256, 0, ctx->stream>>>(
        c->d.orig, c->n, q ? st[4] : nullptr, m ? st[5] : nullptr, c->d.q, c->d.m);
    // the float charge copy lives in the stage buffers: refresh buffer 0
    init_positions<<<(c->n_pad + 255) / 256, 256, 0, ctx->stream>>>(c->d);
    c->boxes_valid[0] = c->boxes_valid[1] = false;
    DM_CUDA(ctx, cudaGetLastError());
    return DM_OK;
}

int dm_cloud_set_forces(dm_cloud *c, const dm_force_params *p) {
    if (!c || !p) return DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    ForceParams fp;
    std::memcpy(&fp, p, sizeof(ForceParams));
    const char *why = nullptr;
    if (const int st = check_force_params(fp, &why))
        return ctx->fail(st, "dm_cloud_set_forces: %s (flags 0x%llx)", why, (unsigned long long)p->flags);
    c->f = fp;
    c->d.rc2 = (p->shielding > 0.0) ? (10.0 / p->shielding) * (10.0 / p->shielding) : 0.0;
    c->drop_graphs();
    // the stage buffers carry a per-particle filter bound that depends on kappa
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    init_positions<<<(c->n_pad + 255) / 256, 256, 0, ctx->stream>>>(c->d);
    c->boxes_valid[0] = c->boxes_valid[1] = false;
    DM_CUDA(ctx, cudaGetLastError());
    return DM_OK;
}

int dm_cloud_eval_forces_device(dm_cloud *c, int precision, double *d_fx, double *d_fy) {
    if (!c) return DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    if (precision != DM_FP64 && precision != DM_FP32C)
        return ctx->fail(DM_ERR_ARG, "bad precision %d", precision);
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    if (c->order_dirty) {  // spatial order first (internal only: outputs are in the caller's order)
        const int rc = reorder(c);
        if (rc) return rc;
    }
    int rc = launch_stage(c, precision, 1, kModeForceOnly, 0.0, nullptr);
    if (rc) return rc;
    const size_t bytes = (size_t)c->n * sizeof(double);
    if (d_fx && d_fx != c->d_fx) DM_CUDA(ctx, cudaMemcpyAsync(d_fx, c->d_fx, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    if (d_fy && d_fy != c->d_fy) DM_CUDA(ctx, cudaMemcpyAsync(d_fy, c->d_fy, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    return DM_OK;
}

int dm_cloud_eval_forces(dm_cloud *c, int precision, double *fx, double *fy) {
    if (!c) return DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    if (!fx || !fy) return ctx->fail(DM_ERR_ARG, "dm_cloud_eval_forces: NULL output");
    int rc = dm_cloud_eval_forces_device(c, precision, nullptr, nullptr);
    if (rc) return rc;
    const size_t bytes = (size_t)c->n * sizeof(double);
    DM_CUDA(ctx, cudaMemcpyAsync(fx, c->d_fx, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    DM_CUDA(ctx, cudaMemcpyAsync(fy, c->d_fy, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return DM_OK;
}

int dm_cloud_evaluated_pairs(dm_cloud *c, unsigned long long *pairs) {
    if (!c || !pairs) return c ? c->ctx->fail(DM_ERR_ARG, "dm_cloud_evaluated_pairs: NULL") : DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    DM_CUDA(ctx, cudaMemcpyAsync(pairs, c->d.eval_pairs, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return DM_OK;
}

int dm_cloud_eval_forces_stage(dm_cloud *c, int precision, int stage, double *fx, double *fy) {
    if (!c) return DM_ERR_ARG;
    if (stage < 1 || stage > 4) return c->ctx->fail(DM_ERR_ARG, "dm_cloud_eval_forces_stage: stage must be 1..4");
    c->eval_thermal_stage = stage;
    const int rc = dm_cloud_eval_forces(c, precision, fx, fy);
    c->eval_thermal_stage = 1;
    return rc;
}

int dm_cloud_step(dm_cloud *c, int nsteps, double dt, int precision, double *t_inout) {
    if (!c) return DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    if (nsteps < 0 || !std::isfinite(dt)) return ctx->fail(DM_ERR_ARG, "dm_cloud_step: bad nsteps/dt");
    if (precision != DM_FP64 && precision != DM_FP32C)
        return ctx->fail(DM_ERR_ARG, "bad precision %d", precision);
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    if (t_inout) {  // the force time of the first step is the caller's time
        set_time_slots<<<1, 1, 0, ctx->stream>>>(c->d.time, *t_inout);
        DM_CUDA(ctx, cudaGetLastError());
    }
    int rc = run_steps(c, nsteps, dt, precision);
    if (rc) return rc;
    if (t_inout)
        for (int s = 0; s < nsteps; s++) *t_inout += dt;
    return DM_OK;
}

int dm_cloud_modify_timestep(dm_cloud *c, double init_dt, float *min_dist, double *dt_out) {
    if (!c) return DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    if (c->n % 4 != 0 || c->n < 4)
        return ctx->fail(DM_ERR_ARG, "adaptive time step needs n %% 4 == 0 (Integrator.cpp:87-107)");
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    DM_CUDA(ctx, cudaMemsetAsync(c->d_min, 0x7f, sizeof(unsigned int), ctx->stream));
    const int nb = c->n / 4;
    const long long total = (long long)nb * (nb + 1) / 2;
    const int blocks = (int)std::min<long long>((total + 255) / 256, (long long)ctx->num_sms * 16);
    // the checked pair pattern is defined on the caller's order
    double **st = c->sort.stage;
    scatter_to_caller<<<(c->n + 255) / 256, 256, 0, ctx->stream>>>(
        c->d.orig, c->n, c->d.x, c->d.y, nullptr, nullptr, st[0], st[1], nullptr, nullptr);
    DM_CUDA(ctx, cudaGetLastError());
    checked_min_dist2<<<std::max(blocks, 1), 256, 0, ctx->stream>>>(st[0], st[1], nb, c->d_min);
    DM_CUDA(ctx, cudaGetLastError());
    adaptive_dt<<<1, 1, 0, ctx->stream>>>(c->d_min, init_dt, c->d_dt, c->d_dmin, c->d.err);
    DM_CUDA(ctx, cudaGetLastError());
    if (min_dist) DM_CUDA(ctx, cudaMemcpyAsync(min_dist, c->d_dmin, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    if (dt_out) DM_CUDA(ctx, cudaMemcpyAsync(dt_out, c->d_dt, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return check_device_errors(ctx, c);
}

int dm_cloud_move_particles(dm_cloud *c, double end_time, double dt, int precision, int adaptive,
                            double *t_inout, int *steps) {
    if (!c || !t_inout) return c ? c->ctx->fail(DM_ERR_ARG, "t_inout is NULL") : DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    if (!(dt > 0.0)) return ctx->fail(DM_ERR_ARG, "dt must be positive");
    double t = *t_inout;
    int count = 0;
    // the force time of the first step is the caller's time
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    set_time_slots<<<1, 1, 0, ctx->stream>>>(c->d.time, t);
    DM_CUDA(ctx, cudaGetLastError());
    if (!adaptive) {
        // same accumulation as `while (currentTime < endTime) currentTime += dt`
        while (t < end_time) {
            t += dt;
            count++;
        }
        int rc = dm_cloud_step(c, count, dt, precision, nullptr);
        if (rc) return rc;
    } else {
        while (t < end_time) {
            double step_dt = 0.0;
            int rc = dm_cloud_modify_timestep(c, dt, nullptr, &step_dt);
            if (rc) return rc;
            for (int st = 1; st <= c->order; st++) {
                rc = launch_stage(c, precision, st, kModeStep, 0.0, c->d_dt);
                if (rc) return rc;
            }
            t += step_dt;
            count++;
        }
    }
    *t_inout = t;
    if (steps) *steps = count;
    return DM_OK;
}

int dm_cloud_diagnostics(dm_cloud *c, double out[5]) {
    if (!c || !out) return DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    const int nt = 128;
    const int blocks = (c->n + nt - 1) / nt;
    double *partial = nullptr;
    DM_CUDA(ctx, cudaMallocAsync((void **)&partial, sizeof(double) * 5 * blocks, ctx->stream));
    diagnostics_partial<nt><<<blocks, nt, 0, ctx->stream>>>(c->d, c->f, c->coulomb, partial);
    cudaError_t e = cudaGetLastError();
    std::vector<double> h((size_t)5 * blocks);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h.data(), partial, sizeof(double) * 5 * blocks, cudaMemcpyDeviceToHost, ctx->stream);
    cudaFreeAsync(partial, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->fail(DM_ERR_CUDA, "dm_cloud_diagnostics: %s", cudaGetErrorString(e));
    for (int k = 0; k < 5; k++) out[k] = 0.0;
    for (int b = 0; b < blocks; b++)
        for (int k = 0; k < 5; k++) out[k] += h[(size_t)b * 5 + k];
    return DM_OK;
}

int dm_ctx_set_autotune(dm_ctx *ctx, int enable) {
    if (!ctx) return DM_ERR_ARG;
    ctx->autotune = enable != 0;
    ctx->tune_cache.clear();
    return DM_OK;
}

int dm_cloud_autotune(dm_cloud *c, int precision, char *variant, size_t len, int *split) {
    if (!c) return DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    if (precision != DM_FP64 && precision != DM_FP32C) return ctx->fail(DM_ERR_ARG, "bad precision %d", precision);
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    int rc = ensure_kernel_attrs(ctx);
    if (rc) return rc;
    const int pi = precision == DM_FP32C ? 1 : 0;
    if (c->tuned_variant[pi] < 0) {
        rc = tune_precision(c, precision);
        if (rc) return rc;
    }
    if (variant && len) snprintf(variant, len, "%s", kVariants[c->tuned_variant[pi]].name);
    if (split) *split = c->split[pi];
    return DM_OK;
}

int dm_kernel_variants(char *buf, size_t len) {
    if (!buf || len == 0) return DM_ERR_ARG;
    std::string out;
    for (int v = 0; v < kNumVariants; v++) {
        if (v) out += ";";
        out += kVariants[v].name;
    }
    snprintf(buf, len, "%s", out.c_str());
    return DM_OK;
}

int dm_cloud_set_kernel(dm_cloud *c, const char *variant, int split) {
    if (!c || !variant) return DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    int vi = -1;
    for (int v = 0; v < kNumVariants; v++)
        if (std::strcmp(kVariants[v].name, variant) == 0) vi = v;
    if (vi < 0) return ctx->fail(DM_ERR_ARG, "unknown kernel variant '%s'", variant);
    const Variant &k = kVariants[vi];
    const int smax = k.cluster ? 16 : kMaxSplitGlobal;
    if (split < 0 || split > smax) return ctx->fail(DM_ERR_ARG, "split %d outside [0, %d]", split, smax);
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    int rc = ensure_kernel_attrs(ctx);
    if (rc) return rc;
    if (split == 0) split = model_split(ctx, k, c->n, c->n_pad);
    if (k.cluster) {
        int nc = 0;
        cudaLaunchAttribute attr[2];
        cudaLaunchConfig_t cfg = make_cfg(ctx, k, (c->n + k.tile - 1) / k.tile, split, attr);
        if (cudaOccupancyMaxActiveClusters(&nc, k.fn, &cfg) != cudaSuccess || nc <= 0) {
            cudaGetLastError();
            return ctx->fail(DM_ERR_UNSUPPORTED, "cluster of %d CTAs of %s cannot be scheduled", split, k.name);
        }
    } else {
        rc = ensure_partial(c, split);
        if (rc) return rc;
    }
    const int pi = k.precision == DM_FP32C ? 1 : 0;
    c->tuned_variant[pi] = vi;
    c->split[pi] = split;
    c->drop_graphs();
    return DM_OK;
}

int dm_cloud_set_reorder_interval(dm_cloud *c, int steps) {
    if (!c) return DM_ERR_ARG;
    if (steps < 0 || steps > kGraphSteps || (steps & (steps - 1)) != 0)
        return c->ctx->fail(DM_ERR_ARG, "reorder interval must be 0 or a power of two <= %d", kGraphSteps);
    c->reorder_interval = steps;
    c->drop_graphs();
    return DM_OK;
}

int dm_cloud_set_step_counter(dm_cloud *c, uint64_t step) {
    if (!c) return DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    unsigned long long v[2] = {step, step};
    DM_CUDA(ctx, cudaMemcpyAsync(c->d.step_ctr, v, sizeof(v), cudaMemcpyHostToDevice, ctx->stream));
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return DM_OK;
}

int dm_cloud_set_integrator(dm_cloud *c, int order) {
    if (!c) return DM_ERR_ARG;
    if (order != 2 && order != 4) return c->ctx->fail(DM_ERR_ARG, "integrator order must be 2 or 4");
    if (order != c->order) c->drop_graphs();
    c->order = order;
    return DM_OK;
}

int dm_cloud_set_time(dm_cloud *c, double t) {
    if (!c) return DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    set_time_slots<<<1, 1, 0, ctx->stream>>>(c->d.time, t);
    DM_CUDA(ctx, cudaGetLastError());
    return DM_OK;
}

int dm_cloud_get_time(dm_cloud *c, double *t) {
    if (!c || !t) return DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    double v = 0.0;
    DM_CUDA(ctx, cudaMemcpyAsync(&v, c->d.time, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream));
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *t = v;
    return DM_OK;
}

int dm_cloud_get_step_counter(dm_cloud *c, uint64_t *step) {
    if (!c || !step) return DM_ERR_ARG;
    dm_ctx *ctx = c->ctx;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    unsigned long long v = 0;
    DM_CUDA(ctx, cudaMemcpyAsync(&v, c->d.step_ctr, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream));
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *step = v;
    return DM_OK;
}


// ===========================================================================
// Batched clouds
// ===========================================================================
}  // extern "C"

namespace {

struct BatchVariant {
    const char *name;
    bool cull;
    int nt, tile;
    size_t smem;
    const void *fn;
    cudaError_t (*launch)(dim3, dim3, size_t, cudaStream_t, const StageParams &, const BatchCloud *,
                          const int2 *, int, unsigned int *);
};

template <int NW, int ILP, int TC, bool CULL>
cudaError_t launch_batch(dim3 g, dim3 b, size_t smem, cudaStream_t s, const StageParams &P,
                         const BatchCloud *desc, const int2 *items, int nitems, unsigned int *ctr) {
    return launch_pdl(batch_stage_fp32c<NW, ILP, TC, CULL>, g, b, smem, s, P, desc, items, nitems, ctr);
}

#define DM_BATCH_VARIANT(NW, ILP, TC, CULL, SUFFIX)                                                \
    {"batch_fp32c<" #NW "," #ILP "," #TC SUFFIX ">", CULL, NW * 32, 32 * ILP,                      \
     Fp32cSmem<NW, ILP, TC>::bytes, (const void *)batch_stage_fp32c<NW, ILP, TC, CULL>,            \
     launch_batch<NW, ILP, TC, CULL>}

const BatchVariant kBatchVariants[] = {
    DM_BATCH_VARIANT(8, 4, 256, false, ""),
    DM_BATCH_VARIANT(4, 4, 256, false, ""),
    DM_BATCH_VARIANT(8, 2, 256, false, ""),
    DM_BATCH_VARIANT(4, 2, 128, false, ""),
    DM_BATCH_VARIANT(8, 4, 256, true, ",cull"),
    DM_BATCH_VARIANT(4, 2, 128, true, ",cull"),
    DM_BATCH_VARIANT(8, 2, 256, true, ",cull"),
};
constexpr int kNumBatchVariants = (int)(sizeof(kBatchVariants) / sizeof(kBatchVariants[0]));

}  // namespace

struct dm_batch {
    dm_ctx *ctx = nullptr;
    int nclouds = 0, total = 0, total_pad = 0;
    void *block = nullptr;
    CloudDev d{};
    std::vector<BatchCloud> hdesc;
    std::vector<int> hn;
    BatchCloud *ddesc = nullptr;
    int *dseg = nullptr;
    unsigned int *dcounter = nullptr;  // [4] work-item counters, one per stage
    int2 *ditems[kNumBatchVariants] = {nullptr};
    int nitems[kNumBatchVariants] = {0};
    int grid[kNumBatchVariants] = {0};
    double *dbox = nullptr;  // [nclouds][8] key box and bounding box (batch_boxes)
    SortScratch sort{};
    int sort_blocks = 0;
    int mbits = 24;
    double *d_fx = nullptr, *d_fy = nullptr;
    int ngroups = 0;            // 32-particle groups over all clouds
    int *dgseg = nullptr;       // [ngroups] cloud of each group
    int variant = -1;
    int reorder_interval = 4;  // 1 when every cloud fits batch_sort_clouds
    int max_n = 0;             // largest cloud
    int order = 4;  // integrator: 4 = Runge_Kutta4, 2 = Runge_Kutta2
    bool order_dirty = true;
    unsigned long long host_steps = 0;
    std::map<GraphKey, cudaGraphExec_t> graphs;
    cudaStream_t graph_stream = nullptr;
    std::vector<void *> extra;

    void drop_graphs() {
        for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
    }
    ~dm_batch() {
        drop_graphs();
        for (void *p : extra) cudaFree(p);
        if (block) cudaFree(block);
    }
};

namespace {

int batch_launch_stage(dm_batch *B, int stage, int mode, double dt, int fo_buf = 0) {
    dm_ctx *ctx = B->ctx;
    const BatchVariant &k = kBatchVariants[B->variant];
    StageParams P{};
    P.c = B->d;
    P.stage = stage;
    P.order = B->order;
    P.mode = mode;
    P.therm_stage = (mode == kModeForceOnly) ? 1 : stage;
    P.fo_buf = (mode == kModeForceOnly) ? fo_buf : 0;
    P.dt = dt;
    P.coulomb = B->d.coulomb;
    P.fx_out = B->d_fx;
    P.fy_out = B->d_fy;
    P.direct_min = direct_min_hits();
    P.near_direct_f2 = near_direct_f2();
    const int slot = (mode == kModeForceOnly) ? 0 : stage - 1;
    if (k.cull) {  // group boxes of the buffer this stage reads
        const int br = (mode == kModeForceOnly) ? fo_buf : (stage - 1) & 1;
        DM_CUDA(ctx, launch_pdl(batch_group_bounds, dim3((B->ngroups * 32 + 255) / 256), dim3(256), 0, ctx->stream,
                                B->d, (const BatchCloud *)B->ddesc, (const int *)B->dgseg, B->ngroups, br));
        ctx->launches++;
    }
    DM_CUDA(ctx, k.launch(dim3(B->grid[B->variant]), dim3(k.nt), k.smem, ctx->stream, P, B->ddesc,
                          B->ditems[B->variant], B->nitems[B->variant], B->dcounter + slot));
    ctx->launches++;
    return DM_OK;
}

int batch_reorder(dm_batch *B) {
    dm_ctx *ctx = B->ctx;
    cudaStream_t s = ctx->stream;
    const int n = B->total;
    const int grid = (n + 255) / 256;
    SortScratch &z = B->sort;
    if (B->max_n <= kBatchSortMax) {  // one block per cloud sorts and gathers; two more commit
        DM_CUDA(ctx, cudaFuncSetAttribute(batch_sort_clouds, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)kBatchSortSmem));
        DM_CUDA(ctx, launch_pdl(batch_sort_clouds, dim3(B->nclouds), dim3(kBatchSortThreads), kBatchSortSmem, s,
                                B->d, (const BatchCloud *)B->ddesc, B->dbox, z));
        DM_CUDA(ctx, launch_pdl(permute_commit, dim3(grid), dim3(256), 0, s, B->d, z));
        DM_CUDA(ctx, launch_pdl(batch_init_positions, dim3((B->total_pad + 255) / 256), dim3(256), 0, s, B->d,
                                (const BatchCloud *)B->ddesc, (const int *)B->dseg));
        ctx->launches += 3;
        B->order_dirty = false;
        return DM_OK;
    }
    batch_boxes<<<B->nclouds, 256, 0, s>>>(B->d.x, B->d.y, B->ddesc, B->dbox);
    batch_keys<<<grid, 256, 0, s>>>(B->d.x, B->d.y, n, B->dseg, B->dbox, B->mbits, z.keys[0], z.vals[0]);
    int cur = 0;
    int passes = 0;
    const int bits = B->mbits + 32 - __builtin_clz((unsigned)std::max(B->nclouds - 1, 1));
    for (int shift = 0; shift < bits; shift += kSortDigitBits) {
        radix_hist<<<B->sort_blocks, kSortThreads, 0, s>>>(z.keys[cur], n, shift, z.hist);
        radix_scan<<<1, 1024, 0, s>>>(z.hist, kSortBuckets * B->sort_blocks);
        radix_scatter<<<B->sort_blocks, kSortThreads, 0, s>>>(z.keys[cur], z.vals[cur], z.keys[cur ^ 1],
                                                               z.vals[cur ^ 1], n, shift, z.hist);
        cur ^= 1;
        passes++;
    }
    permute_gather<<<grid, 256, 0, s>>>(B->d, z.vals[cur], z);
    permute_commit<<<grid, 256, 0, s>>>(B->d, z);
    batch_init_positions<<<(B->total_pad + 255) / 256, 256, 0, s>>>(B->d, B->ddesc, B->dseg);
    DM_CUDA(ctx, cudaGetLastError());
    ctx->launches += 5 + 3 * passes;
    B->order_dirty = false;
    return DM_OK;
}

int batch_enqueue_steps(dm_batch *B, int nsteps, double dt) {
    dm_ctx *ctx = B->ctx;
    for (int s = 0; s < nsteps; s++) {
        if (B->order_dirty || (B->reorder_interval > 0 && B->host_steps % (unsigned)B->reorder_interval == 0)) {
            int rc = batch_reorder(B);
            if (rc) return rc;
        }
        DM_CUDA(ctx, cudaMemsetAsync(B->dcounter, 0, 4 * sizeof(unsigned int), ctx->stream));
        for (int st = 1; st <= B->order; st++) {
            int rc = batch_launch_stage(B, st, kModeStep, dt);
            if (rc) return rc;
        }
        B->host_steps++;
    }
    return DM_OK;
}

int batch_tune(dm_batch *B) {
    dm_ctx *ctx = B->ctx;
    int rc = DM_OK;
    for (int v = 0; v < kNumBatchVariants; v++) {
        const BatchVariant &k = kBatchVariants[v];
        DM_CUDA(ctx, cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem));
        int per_sm = 0;
        DM_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k.fn, k.nt, k.smem));
        B->grid[v] = std::max(1, per_sm) * ctx->num_sms;
        // work items (cloud, tile), largest clouds first
        std::vector<int2> items;
        std::vector<int> order(B->nclouds);
        for (int c = 0; c < B->nclouds; c++) order[c] = c;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return B->hn[a] > B->hn[b]; });
        for (int c : order)
            for (int t = 0; t * k.tile < B->hn[c]; t++) items.push_back(make_int2(c, t));
        B->nitems[v] = (int)items.size();
        if (!B->ditems[v]) {
            DM_CUDA(ctx, cudaMalloc((void **)&B->ditems[v], items.size() * sizeof(int2)));
            B->extra.push_back(B->ditems[v]);
        }
        DM_CUDA(ctx, cudaMemcpyAsync(B->ditems[v], items.data(), items.size() * sizeof(int2),
                                     cudaMemcpyHostToDevice, ctx->stream));
    }
    int best = 0;
    if (ctx->autotune) {
        if (B->order_dirty) {  // tune on the particle order the steps will see
            rc = batch_reorder(B);
            if (rc) return rc;
        }
        // two states, as for one cloud: the batch as it is (buffer 0) and
        // every cloud squeezed to ~30% in-cutoff pairs (buffer 1)
        batch_tune_compress<<<(B->total + 255) / 256, 256, 0, ctx->stream>>>(B->d, B->ddesc, B->dseg, B->dbox);
        DM_CUDA(ctx, cudaGetLastError());
        cudaEvent_t a, b;
        DM_CUDA(ctx, cudaEventCreate(&a));
        DM_CUDA(ctx, cudaEventCreate(&b));
        float best_ms = 1e30f;
        for (int v = 0; v < kNumBatchVariants; v++) {
            B->variant = v;
            float total = 0.0f;
            for (int st = 0; st < 2; st++) {
                DM_CUDA(ctx, cudaMemsetAsync(B->dcounter, 0, sizeof(unsigned int), ctx->stream));
                rc = batch_launch_stage(B, 1, kModeForceOnly, 0.0, st);  // warm-up
                if (rc) return rc;
                float one = 1e30f;
                for (int r = 0; r < 3; r++) {  // best of three
                    DM_CUDA(ctx, cudaMemsetAsync(B->dcounter, 0, sizeof(unsigned int), ctx->stream));
                    DM_CUDA(ctx, cudaEventRecord(a, ctx->stream));
                    rc = batch_launch_stage(B, 1, kModeForceOnly, 0.0, st);
                    if (rc) return rc;
                    DM_CUDA(ctx, cudaEventRecord(b, ctx->stream));
                    DM_CUDA(ctx, cudaEventSynchronize(b));
                    float ms = 0.0f;
                    DM_CUDA(ctx, cudaEventElapsedTime(&ms, a, b));
                    one = std::min(one, ms);
                }
                total += one;
            }
            if (total < best_ms) {
                best_ms = total;
                best = v;
            }
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    B->variant = best;
    return DM_OK;
}

}  // namespace

extern "C" {

int dm_batch_create(dm_ctx *ctx, int nclouds, const int *n, const double *x, const double *y,
                    const double *vx, const double *vy, const double *q, const double *m,
                    const dm_force_params *params, dm_batch **out) {
    if (!ctx || !out || nclouds < 1 || !n || !x || !y || !vx || !vy || !q || !m || !params)
        return ctx ? ctx->fail(DM_ERR_ARG, "dm_batch_create: bad argument") : DM_ERR_ARG;
    if (nclouds > 65536) return ctx->fail(DM_ERR_ARG, "dm_batch_create: at most 65536 clouds");
    *out = nullptr;
    long long total = 0;
    for (int c = 0; c < nclouds; c++) {
        if (n[c] < 1) return ctx->fail(DM_ERR_ARG, "dm_batch_create: cloud %d has n = %d", c, n[c]);
        ForceParams fp;
        std::memcpy(&fp, &params[c], sizeof(ForceParams));
        const char *why = nullptr;
        if (const int st = check_force_params(fp, &why))
            return ctx->fail(st, "dm_batch_create: cloud %d: %s", c, why);
        total += n[c];
    }
    if (total > (1LL << 30)) return ctx->fail(DM_ERR_ARG, "dm_batch_create: too many particles");
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    dm_batch *B = new dm_batch();
    B->ctx = ctx;
    B->nclouds = nclouds;
    B->total = (int)total;
    B->total_pad = ((int)total + 63) & ~63;
    B->hn.assign(n, n + nclouds);
    B->max_n = *std::max_element(n, n + nclouds);
    // per-cloud sort in one launch: cheap enough to keep every cloud's order
    // fresh each step (confined clouds collapse and their groups spread)
    B->reorder_interval = (B->max_n <= kBatchSortMax) ? 1 : 4;
    const int cbits = 32 - __builtin_clz((unsigned)std::max(nclouds - 1, 1));
    B->mbits = std::min(24, (32 - cbits) & ~1);
    const double coulomb = 1.0 / (4.0 * M_PI * 8.8541878E-12);
    const int np = B->total_pad;
    const size_t nd = align256((size_t)np * sizeof(double));
    const size_t nf4 = align256((size_t)np * sizeof(float4));
    const size_t ni = align256((size_t)np * sizeof(int));
    B->sort_blocks = (B->total + kSortPerBlock - 1) / kSortPerBlock;
    const size_t nh = align256((size_t)kSortBuckets * B->sort_blocks * sizeof(uint32_t));
    const size_t ndesc = align256((size_t)nclouds * sizeof(BatchCloud));
    const size_t nbb = align256((size_t)nclouds * 8 * sizeof(double));
    const size_t bytes_total = nd * (6 + 2 + 8 + 4 + 2 + 6) + nf4 * 4 + ni * 7 + nh + ndesc + nbb + 1024;
    cudaError_t e = cudaMalloc(&B->block, bytes_total);
    if (e != cudaSuccess) {
        delete B;
        return ctx->fail(DM_ERR_NOMEM, "dm_batch_create: cudaMalloc(%zu): %s", bytes_total, cudaGetErrorString(e));
    }
    char *p = (char *)B->block;
    auto takeD = [&]() { double *r = (double *)p; p += nd; return r; };
    auto takeF4 = [&]() { float4 *r = (float4 *)p; p += nf4; return r; };
    auto takeI = [&]() { int *r = (int *)p; p += ni; return r; };
    CloudDev &d = B->d;
    d.n = B->total;
    d.n_pad = np;
    d.coulomb = coulomb;
    d.x = takeD(); d.y = takeD(); d.vx = takeD(); d.vy = takeD(); d.q = takeD(); d.m = takeD();
    d.vxc = takeD(); d.vyc = takeD();
    for (int k = 0; k < 4; k++) d.a1[k] = takeD();
    for (int k = 0; k < 4; k++) d.a23[k] = takeD();
    for (int b = 0; b < 2; b++) { d.px[b] = takeD(); d.py[b] = takeD(); }
    B->d_fx = takeD();
    B->d_fy = takeD();
    for (int k = 0; k < 6; k++) B->sort.stage[k] = takeD();
    for (int b = 0; b < 2; b++) { d.pa[b] = takeF4(); d.pb[b] = takeF4(); }
    d.orig = takeI();
    B->dseg = takeI();
    B->sort.keys[0] = (uint32_t *)takeI();
    B->sort.keys[1] = (uint32_t *)takeI();
    B->sort.vals[0] = takeI();
    B->sort.vals[1] = takeI();
    B->sort.orig_stage = takeI();
    B->sort.hist = (uint32_t *)p; p += nh;
    B->ddesc = (BatchCloud *)p; p += ndesc;
    B->dbox = (double *)p; p += nbb;
    d.step_ctr = (unsigned long long *)p; p += 256;
    d.time = (double *)(d.step_ctr + 4);  // same 256-byte slot, bytes 32-47
    d.err = (int *)p; p += 256;
    B->dcounter = (unsigned int *)p; p += 256;
    // host descriptors
    B->hdesc.resize(nclouds);
    std::vector<int> seg((size_t)B->total), orig((size_t)B->total), gseg;
    int off = 0;
    for (int c = 0; c < nclouds; c++) {
        BatchCloud &bc = B->hdesc[c];
        bc.off = off;
        bc.n = n[c];
        bc.goff = B->ngroups;
        for (int g = 0; g < (n[c] + 31) / 32; g++) gseg.push_back(c);
        B->ngroups += (n[c] + 31) / 32;
        std::memcpy(&bc.f, &params[c], sizeof(ForceParams));
        const double kappa = params[c].shielding;
        bc.rc2 = (kappa > 0.0) ? (10.0 / kappa) * (10.0 / kappa) : 0.0;
        bc.rc2_lo = (float)(bc.rc2 * (1.0 - 4e-6));
        bc.rc2_hi = (float)(bc.rc2 * (1.0 + 4e-6));
        bc.kappa_f = (float)kappa;
        bc.nkl2e = (float)(-kappa * 1.4426950408889634);
        for (int i = 0; i < n[c]; i++) {
            seg[off + i] = c;
            orig[off + i] = off + i;
        }
        off += n[c];
    }
    cudaStream_t s = ctx->stream;
    // group boxes (culling kernels), the group -> cloud map, the swept-pair counter
    for (int b = 0; b < 2 && e == cudaSuccess; b++) {
        e = cudaMalloc((void **)&d.gbox[b], (size_t)B->ngroups * sizeof(float4));
        if (e == cudaSuccess) B->extra.push_back(d.gbox[b]);
    }
    if (e == cudaSuccess) e = cudaMalloc((void **)&B->dgseg, gseg.size() * sizeof(int));
    if (e == cudaSuccess) B->extra.push_back(B->dgseg);
    if (e == cudaSuccess) e = cudaMalloc((void **)&d.eval_pairs, sizeof(unsigned long long));
    if (e == cudaSuccess) B->extra.push_back(d.eval_pairs);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.eval_pairs, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(B->dgseg, gseg.data(), gseg.size() * sizeof(int), cudaMemcpyHostToDevice, s);
    const size_t bt = (size_t)B->total * sizeof(double);
    if (e == cudaSuccess) e = cudaMemsetAsync(B->block, 0, bytes_total, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.x, x, bt, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.y, y, bt, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.vx, vx, bt, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.vy, vy, bt, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.q, q, bt, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.m, m, bt, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(B->dseg, seg.data(), seg.size() * sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.orig, orig.data(), orig.size() * sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(B->ddesc, B->hdesc.data(), nclouds * sizeof(BatchCloud), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        batch_init_positions<<<(np + 255) / 256, 256, 0, s>>>(d, B->ddesc, B->dseg);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        delete B;
        return ctx->fail(DM_ERR_CUDA, "dm_batch_create: %s", cudaGetErrorString(e));
    }
    int rc = batch_tune(B);
    if (rc) {
        delete B;
        return rc;
    }
    *out = B;
    return DM_OK;
}

int dm_batch_destroy(dm_batch *B) {
    if (!B) return DM_ERR_ARG;
    cudaSetDevice(B->ctx->device);
    cudaStreamSynchronize(B->ctx->stream);
    delete B;
    return DM_OK;
}

int dm_batch_step(dm_batch *B, int nsteps, double dt, int precision) {
    if (!B) return DM_ERR_ARG;
    dm_ctx *ctx = B->ctx;
    if (precision != DM_FP32C)
        return ctx->fail(DM_ERR_UNSUPPORTED, "batched clouds run the FP32C kernel; step FP64 clouds singly");
    if (nsteps < 0 || !std::isfinite(dt)) return ctx->fail(DM_ERR_ARG, "dm_batch_step: bad nsteps/dt");
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    if (ctx->prof || nsteps < kGraphSteps) return batch_enqueue_steps(B, nsteps, dt);
    if (B->graph_stream != ctx->stream) {
        B->drop_graphs();
        B->graph_stream = ctx->stream;
    }
    while (nsteps > 0 && (B->order_dirty || (B->reorder_interval > 0 && B->host_steps % kGraphSteps != 0))) {
        int rc = batch_enqueue_steps(B, 1, dt);
        if (rc) return rc;
        nsteps--;
    }
    if (nsteps < kGraphSteps) return batch_enqueue_steps(B, nsteps, dt);
    const GraphKey key{DM_FP32C, kGraphSteps, dt};
    auto it = B->graphs.find(key);
    static long long graph_launches_cache = 0;
    if (it == B->graphs.end()) {
        cudaGraph_t g = nullptr;
        const unsigned long long saved = B->host_steps;
        const long long sl = ctx->launches;
        DM_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        int rc = batch_enqueue_steps(B, kGraphSteps, dt);
        cudaError_t ec = cudaStreamEndCapture(ctx->stream, &g);
        B->host_steps = saved;
        graph_launches_cache = ctx->launches - sl;
        ctx->launches = sl;
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (ec != cudaSuccess) return ctx->fail(DM_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ec));
        cudaGraphExec_t ge = nullptr;
        ec = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (ec != cudaSuccess) return ctx->fail(DM_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(ec));
        it = B->graphs.emplace(key, ge).first;
    }
    const int reps = nsteps / kGraphSteps;
    for (int r = 0; r < reps; r++) {
        DM_CUDA(ctx, cudaGraphLaunch(it->second, ctx->stream));
        B->host_steps += kGraphSteps;
        ctx->launches += graph_launches_cache;
    }
    return batch_enqueue_steps(B, nsteps - reps * kGraphSteps, dt);
}

int dm_batch_eval_forces(dm_batch *B, int precision, double *fx, double *fy) {
    if (!B || !fx || !fy) return B ? B->ctx->fail(DM_ERR_ARG, "NULL output") : DM_ERR_ARG;
    dm_ctx *ctx = B->ctx;
    if (precision != DM_FP32C)
        return ctx->fail(DM_ERR_UNSUPPORTED, "batched clouds run the FP32C kernel");
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    DM_CUDA(ctx, cudaMemsetAsync(B->dcounter, 0, sizeof(unsigned int), ctx->stream));
    int rc = batch_launch_stage(B, 1, kModeForceOnly, 0.0);
    if (rc) return rc;
    const size_t bt = (size_t)B->total * sizeof(double);
    DM_CUDA(ctx, cudaMemcpyAsync(fx, B->d_fx, bt, cudaMemcpyDeviceToHost, ctx->stream));
    DM_CUDA(ctx, cudaMemcpyAsync(fy, B->d_fy, bt, cudaMemcpyDeviceToHost, ctx->stream));
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return DM_OK;
}

int dm_batch_download(dm_batch *B, double *x, double *y, double *vx, double *vy) {
    if (!B) return DM_ERR_ARG;
    dm_ctx *ctx = B->ctx;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t bt = (size_t)B->total * sizeof(double);
    double **st = B->sort.stage;
    scatter_to_caller<<<(B->total + 255) / 256, 256, 0, ctx->stream>>>(
        B->d.orig, B->total, B->d.x, B->d.y, B->d.vx, B->d.vy, st[0], st[1], st[2], st[3]);
    DM_CUDA(ctx, cudaGetLastError());
    ctx->launches++;
    if (x) DM_CUDA(ctx, cudaMemcpyAsync(x, st[0], bt, cudaMemcpyDeviceToHost, ctx->stream));
    if (y) DM_CUDA(ctx, cudaMemcpyAsync(y, st[1], bt, cudaMemcpyDeviceToHost, ctx->stream));
    if (vx) DM_CUDA(ctx, cudaMemcpyAsync(vx, st[2], bt, cudaMemcpyDeviceToHost, ctx->stream));
    if (vy) DM_CUDA(ctx, cudaMemcpyAsync(vy, st[3], bt, cudaMemcpyDeviceToHost, ctx->stream));
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int h = 0;
    DM_CUDA(ctx, cudaMemcpy(&h, B->d.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        cudaMemset(B->d.err, 0, sizeof(int));
        return ctx->fail(DM_ERR_NUMERIC, "non-finite particle position in the batch");
    }
    return DM_OK;
}

int dm_batch_variants(char *buf, size_t len) {
    if (!buf || len == 0) return DM_ERR_ARG;
    std::string out;
    for (int v = 0; v < kNumBatchVariants; v++) {
        if (v) out += ";";
        out += kBatchVariants[v].name;
    }
    snprintf(buf, len, "%s", out.c_str());
    return out.size() < len ? DM_OK : DM_ERR_ARG;
}

int dm_batch_set_kernel(dm_batch *B, const char *variant) {
    if (!B || !variant) return B ? B->ctx->fail(DM_ERR_ARG, "dm_batch_set_kernel: NULL") : DM_ERR_ARG;
    for (int v = 0; v < kNumBatchVariants; v++)
        if (std::strcmp(kBatchVariants[v].name, variant) == 0) {
            B->variant = v;
            B->drop_graphs();
            return DM_OK;
        }
    return B->ctx->fail(DM_ERR_ARG, "dm_batch_set_kernel: unknown variant '%s'", variant);
}

int dm_batch_evaluated_pairs(dm_batch *B, unsigned long long *pairs) {
    if (!B || !pairs) return B ? B->ctx->fail(DM_ERR_ARG, "dm_batch_evaluated_pairs: NULL") : DM_ERR_ARG;
    dm_ctx *ctx = B->ctx;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    DM_CUDA(ctx, cudaMemcpyAsync(pairs, B->d.eval_pairs, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return DM_OK;
}

int dm_batch_info(dm_batch *B, char *variant, size_t len, int *nitems, int *grid) {
    if (!B) return DM_ERR_ARG;
    if (variant && len) snprintf(variant, len, "%s", kBatchVariants[B->variant].name);
    if (nitems) *nitems = B->nitems[B->variant];
    if (grid) *grid = B->grid[B->variant];
    return DM_OK;
}

int dm_batch_set_integrator(dm_batch *B, int order) {
    if (!B) return DM_ERR_ARG;
    if (order != 2 && order != 4) return B->ctx->fail(DM_ERR_ARG, "integrator order must be 2 or 4");
    if (order != B->order) B->drop_graphs();
    B->order = order;
    return DM_OK;
}

int dm_batch_set_time(dm_batch *B, double t) {
    if (!B) return DM_ERR_ARG;
    dm_ctx *ctx = B->ctx;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    set_time_slots<<<1, 1, 0, ctx->stream>>>(B->d.time, t);
    DM_CUDA(ctx, cudaGetLastError());
    return DM_OK;
}

int dm_batch_get_time(dm_batch *B, double *t) {
    if (!B || !t) return DM_ERR_ARG;
    dm_ctx *ctx = B->ctx;
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    double v = 0.0;
    DM_CUDA(ctx, cudaMemcpyAsync(&v, B->d.time, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream));
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *t = v;
    return DM_OK;
}

int dm_batch_set_step_counter(dm_batch *B, uint64_t step) {
    if (!B) return DM_ERR_ARG;
    dm_ctx *ctx = B->ctx;
    unsigned long long v[2] = {step, step};
    DM_CUDA(ctx, cudaMemcpy(B->d.step_ctr, v, sizeof(v), cudaMemcpyHostToDevice));
    return DM_OK;
}


// ===========================================================================
// Differentiable rollout support: FP64 forces and their VJP on device arrays
// ===========================================================================
}  // extern "C"

struct dm_adjoint {
    dm_ctx *ctx = nullptr;
    int nclouds = 0, total = 0, nblocks = 0;
    std::vector<AdjCloud> hdesc;
    AdjCloud *ddesc = nullptr;
    int *dcloud = nullptr, *dtile = nullptr;
    double coulomb = 0.0;
    // fused RK4 step and adjoint: one block of total-length arrays
    void *work = nullptr;
    double *k1[4], *k23[4], *pbuf[2][4], *dk[2][4], *mu[3][4], *axd, *ayd;
    float *axf, *ayf;
    ~dm_adjoint() {
        if (ddesc) cudaFree(ddesc);
        if (dcloud) cudaFree(dcloud);
        if (dtile) cudaFree(dtile);
        if (work) cudaFree(work);
    }
};

namespace {
void adj_fill(dm_adjoint *A, const dm_force_params *params) {
    for (int c = 0; c < A->nclouds; c++) {
        AdjCloud &d = A->hdesc[c];
        d.flags = params[c].flags;
        d.kappa = params[c].shielding;
        d.confine = params[c].confine;
        d.confine_x = params[c].confine_x;
        d.confine_y = params[c].confine_y;
        d.gamma = params[c].gamma;
        d.rc2 = (d.kappa > 0.0) ? (10.0 / d.kappa) * (10.0 / d.kappa) : 0.0;
        d.rc2_lo = (float)(d.rc2 * (1.0 - 4e-6));
        d.rc2_hi = (float)(d.rc2 * (1.0 + 4e-6));
        d.kappa_f = (float)d.kappa;
        d.kappa2_f = (float)(d.kappa * d.kappa);
        kappa_log2e(d.kappa, d.kl2e_hi, d.kl2e_lo);
        d.nkl2e = (float)(-d.kappa * 1.4426950408889634);
    }
}

template <int MODE>
void adj_launch(dm_adjoint *A, int precision, const double *x, const double *y, const double *vx,
                const double *vy, const double *q, const double *m, const double *ax, const double *ay,
                double *o0, double *o1, double *o2, double *o3, double *o4, double *o5, double *o6) {
    cudaStream_t st = A->ctx->stream;
    if (precision == DM_FP32C)
        adjoint_kernel<MODE, true><<<A->nblocks, kAdjThreads, 0, st>>>(
            A->ddesc, A->dcloud, A->dtile, x, y, vx, vy, q, m, ax, ay, o0, o1, o2, o3, o4, o5, o6, A->coulomb);
    else
        adjoint_kernel<MODE, false><<<A->nblocks, kAdjThreads, 0, st>>>(
            A->ddesc, A->dcloud, A->dtile, x, y, vx, vy, q, m, ax, ay, o0, o1, o2, o3, o4, o5, o6, A->coulomb);
}
}  // namespace

extern "C" {

int dm_adjoint_create(dm_ctx *ctx, int nclouds, const int *n, const dm_force_params *params,
                      dm_adjoint **out) {
    if (!ctx || !out || nclouds < 1 || !n || !params) return ctx ? ctx->fail(DM_ERR_ARG, "dm_adjoint_create: bad argument") : DM_ERR_ARG;
    const long long known = kConfinement | kDrag | kShieldedCoulomb | kRectConfinement;
    for (int c = 0; c < nclouds; c++) {
        if (n[c] < 1) return ctx->fail(DM_ERR_ARG, "dm_adjoint_create: cloud %d is empty", c);
        if (params[c].flags & ~known)
            return ctx->fail(DM_ERR_UNSUPPORTED, "dm_adjoint_create: only confinement, drag and shielded "
                                                 "Coulomb forces are differentiated");
        ForceParams fp;
        std::memcpy(&fp, &params[c], sizeof(ForceParams));
        const char *why = nullptr;
        if (const int st = check_force_params(fp, &why))
            return ctx->fail(st, "dm_adjoint_create: cloud %d: %s", c, why);
    }
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    dm_adjoint *A = new dm_adjoint();
    A->ctx = ctx;
    A->nclouds = nclouds;
    A->coulomb = 1.0 / (4.0 * M_PI * 8.8541878E-12);
    A->hdesc.resize(nclouds);
    std::vector<int> bc, bt;
    int off = 0;
    for (int c = 0; c < nclouds; c++) {
        A->hdesc[c].off = off;
        A->hdesc[c].n = n[c];
        for (int t = 0; t * kAdjThreads < n[c]; t++) {
            bc.push_back(c);
            bt.push_back(t);
        }
        off += n[c];
    }
    A->total = off;
    A->nblocks = (int)bc.size();
    adj_fill(A, params);
    cudaError_t e = cudaMalloc((void **)&A->ddesc, nclouds * sizeof(AdjCloud));
    if (e == cudaSuccess) e = cudaMalloc((void **)&A->dcloud, bc.size() * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc((void **)&A->dtile, bt.size() * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(A->ddesc, A->hdesc.data(), nclouds * sizeof(AdjCloud), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(A->dcloud, bc.data(), bc.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(A->dtile, bt.data(), bt.size() * sizeof(int), cudaMemcpyHostToDevice);
    // scratch of the fused RK4 step and its adjoint: 38 arrays of total doubles, 2 of floats
    const size_t nd = align256((size_t)A->total * sizeof(double));
    const size_t nf = align256((size_t)A->total * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&A->work, 38 * nd + 2 * nf);
    if (e == cudaSuccess) {
        char *p = (char *)A->work;
        auto take = [&]() { double *r = (double *)p; p += nd; return r; };
        for (int c = 0; c < 4; c++) A->k1[c] = take();
        for (int c = 0; c < 4; c++) A->k23[c] = take();
        for (int b = 0; b < 2; b++)
            for (int c = 0; c < 4; c++) A->pbuf[b][c] = take();
        for (int b = 0; b < 2; b++)
            for (int c = 0; c < 4; c++) A->dk[b][c] = take();
        for (int b = 0; b < 3; b++)
            for (int c = 0; c < 4; c++) A->mu[b][c] = take();
        A->axd = take();
        A->ayd = take();
        A->axf = (float *)p;
        p += nf;
        A->ayf = (float *)p;
    }
    if (e != cudaSuccess) {
        delete A;
        return ctx->fail(DM_ERR_CUDA, "dm_adjoint_create: %s", cudaGetErrorString(e));
    }
    *out = A;
    return DM_OK;
}

int dm_adjoint_destroy(dm_adjoint *A) {
    if (!A) return DM_ERR_ARG;
    cudaSetDevice(A->ctx->device);
    cudaStreamSynchronize(A->ctx->stream);
    delete A;
    return DM_OK;
}

int dm_adjoint_set_params(dm_adjoint *A, const dm_force_params *params) {
    if (!A || !params) return DM_ERR_ARG;
    dm_ctx *ctx = A->ctx;
    adj_fill(A, params);
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    DM_CUDA(ctx, cudaMemcpyAsync(A->ddesc, A->hdesc.data(), A->nclouds * sizeof(AdjCloud),
                                 cudaMemcpyHostToDevice, ctx->stream));
    DM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // the host copy may be reused at once
    return DM_OK;
}

int dm_adjoint_forces(dm_adjoint *A, int precision, const double *x, const double *y, const double *vx,
                      const double *vy, const double *q, const double *m, double *fx, double *fy,
                      double *fpx, double *fpy) {
    if (!A || !x || !y || !vx || !vy || !q || !m || !fx || !fy) return A ? A->ctx->fail(DM_ERR_ARG, "NULL pointer") : DM_ERR_ARG;
    dm_ctx *ctx = A->ctx;
    if (precision != DM_FP64 && precision != DM_FP32C)
        return ctx->fail(DM_ERR_ARG, "dm_adjoint_forces: unknown precision %d", precision);
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    adj_launch<0>(A, precision, x, y, vx, vy, q, m, nullptr, nullptr, fx, fy, fpx, fpy, nullptr, nullptr,
                  nullptr);
    DM_CUDA(ctx, cudaGetLastError());
    ctx->launches++;
    return DM_OK;
}

int dm_adjoint_rk4_step(dm_adjoint *A, int precision, double dt, double *x, double *y, double *vx, double *vy,
                        const double *q, const double *m, double *stages) {
    if (!A || !x || !y || !vx || !vy || !q || !m) return A ? A->ctx->fail(DM_ERR_ARG, "NULL pointer") : DM_ERR_ARG;
    dm_ctx *ctx = A->ctx;
    if (precision != DM_FP64 && precision != DM_FP32C)
        return ctx->fail(DM_ERR_ARG, "dm_adjoint_rk4_step: unknown precision %d", precision);
    if (!std::isfinite(dt)) return ctx->fail(DM_ERR_ARG, "dm_adjoint_rk4_step: dt must be finite");
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t n = (size_t)A->total;
    double *base[4] = {x, y, vx, vy};
    if (stages)
        for (int c = 0; c < 4; c++)
            DM_CUDA(ctx, cudaMemcpyAsync(stages + c * n, base[c], n * sizeof(double), cudaMemcpyDeviceToDevice,
                                         ctx->stream));
    for (int st = 1; st <= 4; st++) {
        AdjStepIO io{};
        double *in[4], *nx[4];
        for (int c = 0; c < 4; c++) {
            in[c] = (st == 1) ? base[c] : stages ? stages + (4 * (st - 1) + c) * n : A->pbuf[st & 1][c];
            nx[c] = (st == 4) ? nullptr : stages ? stages + (4 * st + c) * n : A->pbuf[(st + 1) & 1][c];
            io.k1[c] = A->k1[c];
            io.k23[c] = A->k23[c];
        }
        io.x = in[0]; io.y = in[1]; io.vx = in[2]; io.vy = in[3];
        io.sx = x; io.sy = y; io.svx = vx; io.svy = vy;
        io.nx = nx[0]; io.ny = nx[1]; io.nvx = nx[2]; io.nvy = nx[3];
        io.q = q;
        io.m = m;
        io.dt = dt;
        io.stage = st;
        if (precision == DM_FP32C)
            adj_step_forces<true><<<A->nblocks, kAdjThreads, 0, ctx->stream>>>(A->ddesc, A->dcloud, A->dtile, io,
                                                                              A->coulomb);
        else
            adj_step_forces<false><<<A->nblocks, kAdjThreads, 0, ctx->stream>>>(A->ddesc, A->dcloud, A->dtile, io,
                                                                               A->coulomb);
        DM_CUDA(ctx, cudaGetLastError());
        ctx->launches++;
    }
    return DM_OK;
}

int dm_adjoint_rk4_step_vjp(dm_adjoint *A, int precision, double dt, const double *stages, const double *q,
                            const double *m, double *lx, double *ly, double *lvx, double *lvy, double *gq,
                            double *gkappa, double *gkc) {
    if (!A || !stages || !q || !m || !lx || !ly || !lvx || !lvy || !gq || !gkappa || !gkc)
        return A ? A->ctx->fail(DM_ERR_ARG, "NULL pointer") : DM_ERR_ARG;
    dm_ctx *ctx = A->ctx;
    if (precision != DM_FP64 && precision != DM_FP32C)
        return ctx->fail(DM_ERR_ARG, "dm_adjoint_rk4_step_vjp: unknown precision %d", precision);
    if (!std::isfinite(dt)) return ctx->fail(DM_ERR_ARG, "dm_adjoint_rk4_step_vjp: dt must be finite");
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t n = (size_t)A->total;
    for (int st = 4; st >= 1; st--) {
        AdjVjpIO V{};
        V.x = stages + (4 * (st - 1) + 0) * n;
        V.y = stages + (4 * (st - 1) + 1) * n;
        V.vx = stages + (4 * (st - 1) + 2) * n;
        V.vy = stages + (4 * (st - 1) + 3) * n;
        // dk_3 in dk[0], dk_2 in dk[1], dk_1 in dk[0]; dk_4 = lam / 6
        const int rd = (st == 3 || st == 1) ? 0 : 1, wr = (st == 4 || st == 2) ? 0 : 1;
        double *lam[4] = {lx, ly, lvx, lvy};
        for (int c = 0; c < 4; c++) {
            V.dk[c] = A->dk[rd][c];
            V.dkn[c] = A->dk[wr][c];
            V.lam[c] = lam[c];
            for (int b = 0; b < 3; b++) V.mu[b][c] = A->mu[b][c];
        }
        V.gq = gq;
        V.gkappa = gkappa;
        V.gkc = gkc;
        V.q = q;
        V.m = m;
        V.dt = dt;
        V.stage = st;
        adj_force_adjoint<<<(A->total + 255) / 256, 256, 0, ctx->stream>>>(V, A->total, A->axf, A->ayf, A->axd,
                                                                         A->ayd);
        DM_CUDA(ctx, cudaGetLastError());
        if (precision == DM_FP32C)
            adj_step_vjp<true><<<A->nblocks, kAdjThreads, 0, ctx->stream>>>(A->ddesc, A->dcloud, A->dtile, V, A->axf,
                                                                           A->ayf, A->axd, A->ayd, A->coulomb);
        else
            adj_step_vjp<false><<<A->nblocks, kAdjThreads, 0, ctx->stream>>>(A->ddesc, A->dcloud, A->dtile, V, A->axf,
                                                                            A->ayf, A->axd, A->ayd, A->coulomb);
        DM_CUDA(ctx, cudaGetLastError());
        ctx->launches += 2;
    }
    return DM_OK;
}

int dm_adjoint_vjp(dm_adjoint *A, int precision, const double *x, const double *y, const double *vx,
                   const double *vy, const double *q, const double *m, const double *ax, const double *ay,
                   double *gx, double *gy, double *gvx, double *gvy, double *gq, double *gkappa, double *gkc) {
    if (!A || !x || !y || !vx || !vy || !q || !m || !ax || !ay || !gx || !gy || !gvx || !gvy || !gq ||
        !gkappa || !gkc)
        return A ? A->ctx->fail(DM_ERR_ARG, "NULL pointer") : DM_ERR_ARG;
    dm_ctx *ctx = A->ctx;
    if (precision != DM_FP64 && precision != DM_FP32C)
        return ctx->fail(DM_ERR_ARG, "dm_adjoint_vjp: unknown precision %d", precision);
    DM_CUDA(ctx, cudaSetDevice(ctx->device));
    adj_launch<1>(A, precision, x, y, vx, vy, q, m, ax, ay, gx, gy, gvx, gvy, gq, gkappa, gkc);
    DM_CUDA(ctx, cudaGetLastError());
    ctx->launches++;
    return DM_OK;
}

}  // extern "C"
