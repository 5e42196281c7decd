// dm_batch.cuh -- many independent clouds of uneven size in one launch.
//
// The clouds are concatenated (caller order: cloud 0's particles, then cloud
// 1's, ...) into one set of device arrays with no per-cloud padding; each
// cloud keeps its own force parameters (kappa, charge, confinement, ...).
// A stage is ONE persistent launch: every CTA repeatedly takes the next work
// item -- (cloud, i-tile) -- from a global counter and runs the same FP32C
// sweep as the single-cloud kernel over that cloud's j, then the stage
// epilogue for the tile's particles.  Items are ordered by cost (largest
// clouds first), so the dynamic hand-out is a longest-processing-time
// schedule; since an item is computed entirely by one CTA, the result does
// not depend on which CTA takes it (deterministic, no atomics on forces).
#pragma once

#include "dm_pair.cuh"
#include "dm_sort.cuh"

namespace dm {

struct BatchCloud {
    int off;        // first particle in the concatenated arrays
    int n;
    int goff;       // first of the cloud's 32-particle groups in the batch's group boxes
    ForceParams f;
    double rc2;
    float rc2_lo, rc2_hi, kappa_f;
    float nkl2e;    // -kappa*log2(e)
};

// A StageParams view of one cloud: pointers offset to the cloud's particles.
__device__ __forceinline__ void batch_view(StageParams &V, const StageParams &P0, const BatchCloud &d) {
    V = P0;
    const int o = d.off;
    CloudDev &c = V.c;
    c.x += o; c.y += o; c.vx += o; c.vy += o; c.q += o; c.m += o;
    c.vxc += o; c.vyc += o;
    for (int k = 0; k < 4; k++) { c.a1[k] += o; c.a23[k] += o; }
    for (int b = 0; b < 2; b++) {
        c.px[b] += o; c.py[b] += o; c.pa[b] += o; c.pb[b] += o;
        c.gbox[b] += d.goff;  // group boxes numbered within the cloud
    }
    c.orig += o;  // values stay global caller indices (thermal counter, outputs)
    c.n = d.n;
    c.n_pad = d.n;
    c.rc2 = d.rc2;
    V.f = d.f;
    V.rc2 = d.rc2;
    V.rc2_lo = d.rc2_lo;
    V.rc2_hi = d.rc2_hi;
    V.kappa_f = d.kappa_f;
    V.nkl2e = d.nkl2e;
}

template <int NW, int ILP, int TC, bool CULL = false>
__global__ void __launch_bounds__(NW * 32, (24 / NW > 0 ? 24 / NW : 1))
    batch_stage_fp32c(const StageParams P0, const BatchCloud *__restrict__ desc,
                      const int2 *__restrict__ items, int nitems, unsigned int *counter) {
    constexpr int TILE = 32 * ILP;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ StageParams sV;
    __shared__ int s_item;
    float4 *s_red = reinterpret_cast<float4 *>(smem_raw) + Fp32cSmem<NW, ILP, TC>::red_offset;
    const int tid = threadIdx.x;
    pdl_wait();
    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int it = s_item;
        if (it >= nitems) break;
        const int2 w = items[it];
        if (tid == 0) batch_view(sV, P0, desc[w.x]);
        __syncthreads();
        const int tile = w.y;
        fp32c_sweep<NW, ILP, TC, CULL>(sV, tile, 0, 1, smem_raw);
        if (tid < TILE) {
            const int i = tile * TILE + tid;
            if (i < sV.c.n) {
                const float4 v = s_red[tid];
                const double cq = pair_scale(sV, i);
                stage_epilogue(sV, i, __dmul_rn(cq, (double)v.x - (double)v.z),
                               __dmul_rn(cq, (double)v.y - (double)v.w), stage_thermal(sV, i));
            }
        }
        __syncthreads();  // before the next item reuses shared memory
    }
    stage_step_advance(P0);
}

// Box of every cloud's 32-particle groups in stage buffer b (one warp per
// group; gseg[w] is group w's cloud; a cloud's last group may be partial).
static __global__ void batch_group_bounds(CloudDev c, const BatchCloud *__restrict__ desc,
                                          const int *__restrict__ gseg, int ngroups, int b) {
    pdl_wait();
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= ngroups) return;  // whole warp
    const BatchCloud d = desc[gseg[w]];
    const int li = 32 * (w - d.goff) + lane;
    float x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
    if (li < d.n) {
        const float4 A = c.pa[b][d.off + li];
        x0 = x1 = A.x;
        y0 = y1 = A.y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
        y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
        x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
        y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
    }
    if (lane == 0) c.gbox[b][w] = make_float4(x0, y0, x1, y1);
}

// --- per-cloud Morton order ------------------------------------------------

// bbox rows are (min x, min y, max x, max y) in ordered bits: the min
// entries start at all-ones (memset), the max entries at zero.
// One block per cloud: the cloud's key box (the bounding box clipped to
// mean +- 4 sigma per axis) and bounding box, box[8 * cloud ...] as in
// moments_to_box.  Deterministic (fixed partition and order).
static __global__ void __launch_bounds__(256) batch_boxes(const double *__restrict__ x,
                                                          const double *__restrict__ y,
                                                          const BatchCloud *__restrict__ desc, double *box) {
    const BatchCloud &d = desc[blockIdx.x];
    const double ox = finite_or_zero(x[d.off]), oy = finite_or_zero(y[d.off]);
    const Moments m = block_moments(x, y, d.off, d.off + d.n, blockDim.x, ox, oy);
    if (threadIdx.x == 0) moments_to_box(m, ox, oy, box + 8 * blockIdx.x);
}

// key = cloud index (high bits) | the top `mbits` bits of the 24-bit Morton
// code within the cloud's box, so a stable sort keeps every cloud in its own
// contiguous range.
static __global__ void batch_keys(const double *__restrict__ x, const double *__restrict__ y, int n,
                                  const int *__restrict__ seg, const double *__restrict__ box,
                                  int mbits, uint32_t *keys, int *vals) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int sg = seg[i];
    const double *bb = box + 8 * sg;
    const double x0 = bb[0], y0 = bb[1], ext = bb[2];
    const double scale = (ext > 0.0 && isfinite(ext)) ? 4095.0 / ext : 0.0;
    const double fx = (x[i] - x0) * scale, fy = (y[i] - y0) * scale;
    const uint32_t qx = (fx > 0.0) ? (uint32_t)fmin(fx, 4095.0) : 0u;
    const uint32_t qy = (fy > 0.0) ? (uint32_t)fmin(fy, 4095.0) : 0u;
    const uint32_t morton = spread_bits12(qx) | (spread_bits12(qy) << 1);
    keys[i] = ((uint32_t)sg << mbits) | (morton >> (24 - mbits));
    vals[i] = i;
}

// ---------------------------------------------------------------------------
// Per-cloud sort for batches whose clouds all hold at most kBatchSortMax
// particles: block b sorts cloud b on its own -- key box, 24-bit Morton keys,
// three stable 8-bit LSD passes in shared memory -- and gathers the cloud's
// state in the new order into the staging arrays (permute_commit copies it
// back).  One launch replaces the batch-wide path (per-cloud boxes, keys with
// the cloud index in the high bits, four radix passes over every particle of
// every cloud, gather: fifteen dependent launches).  As in sort_cluster the
// key box and keys are FP32 functions of the positions' hi parts (stage
// buffer 0), lanes with equal digits are found by match_digit8, and the
// element order (warp, round, lane) makes every pass stable.
// ---------------------------------------------------------------------------
constexpr int kBatchSortMax = 4096;
constexpr int kBatchSortThreads = 1024;
constexpr int kBatchSortWarps = kBatchSortThreads / 32;
constexpr int kBatchSortRounds = kBatchSortMax / kBatchSortThreads;  // 4 per thread

struct BatchSortSmem {
    uint32_t keys[2][kBatchSortMax];
    uint16_t slot[2][kBatchSortMax];
    uint32_t wcnt[kBatchSortWarps][kSortBuckets];  // per-warp digit counts, then offsets
    uint32_t dbase[kSortBuckets];
    uint32_t part[kSortBuckets / 32];
    float wmom[kBatchSortWarps][kMomentFields];
    float box[3];
};
constexpr size_t kBatchSortSmem = sizeof(BatchSortSmem);

// box_out[8 * cloud]: key box x0, y0, extent, 0, bounding box min x, min y,
// max x, max y (as batch_boxes writes them; the batch autotuner reads it).
static __global__ void __launch_bounds__(kBatchSortThreads, 1)
    batch_sort_clouds(CloudDev c, const BatchCloud *__restrict__ desc, double *box_out, SortScratch z) {
    pdl_wait();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    BatchSortSmem &S = *reinterpret_cast<BatchSortSmem *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const BatchCloud d = desc[blockIdx.x];
    const int off = d.off, n = d.n;
    const float4 *__restrict__ pa0 = c.pa[0] + off;

    float4 pos[kBatchSortRounds];
#pragma unroll
    for (int k = 0; k < kBatchSortRounds; k++) {
        const int e = k * kBatchSortThreads + tid;
        pos[k] = (e < n) ? pa0[e] : make_float4(NAN, NAN, 0.0f, 0.0f);
    }
    const float4 p0 = pa0[0];
    const float ox = isfinite(p0.x) ? p0.x : 0.0f, oy = isfinite(p0.y) ? p0.y : 0.0f;
    {
        float v[kMomentFields] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, INFINITY, INFINITY, -INFINITY, -INFINITY};
#pragma unroll
        for (int k = 0; k < kBatchSortRounds; k++) moments_f32_add(v, pos[k], ox, oy);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            float w[kMomentFields];
#pragma unroll
            for (int k = 0; k < kMomentFields; k++) w[k] = __shfl_xor_sync(0xffffffffu, v[k], o);
            moments_f32_merge(v, w);
        }
        if (lane == 0)
            for (int k = 0; k < kMomentFields; k++) S.wmom[warp][k] = v[k];
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < kBatchSortWarps; w++) moments_f32_merge(v, S.wmom[w]);
            float lo[2] = {0.0f, 0.0f}, hi[2] = {0.0f, 0.0f};
            if (v[0] > 0.0f) {
                const float org[2] = {ox, oy};
                for (int a = 0; a < 2; a++) {
                    const float mean = v[1 + a] / v[0];
                    const float sd = sqrtf(fmaxf(v[3 + a] / v[0] - mean * mean, 0.0f));
                    lo[a] = fmaxf(v[5 + a], org[a] + mean - 4.0f * sd);
                    hi[a] = fminf(v[7 + a], org[a] + mean + 4.0f * sd);
                    if (!(lo[a] <= hi[a])) {
                        lo[a] = v[5 + a];
                        hi[a] = v[7 + a];
                    }
                }
            }
            S.box[0] = lo[0];
            S.box[1] = lo[1];
            S.box[2] = fmaxf(hi[0] - lo[0], hi[1] - lo[1]);
            double *bo = box_out + 8 * blockIdx.x;
            bo[0] = S.box[0];
            bo[1] = S.box[1];
            bo[2] = S.box[2];
            bo[3] = 0.0;
            for (int k = 0; k < 4; k++) bo[4 + k] = (v[0] > 0.0f) ? (double)v[5 + k] : 0.0;
        }
        __syncthreads();
    }
    {
        const float x0 = S.box[0], y0 = S.box[1], ext = S.box[2];
        const float scale = (ext > 0.0f && isfinite(ext)) ? 4095.0f / ext : 0.0f;
#pragma unroll
        for (int k = 0; k < kBatchSortRounds; k++) {
            const int li = k * kBatchSortThreads + tid;
            uint32_t key = 0u;
            if (li < n) {
                const float fx = (pos[k].x - x0) * scale, fy = (pos[k].y - y0) * scale;
                const uint32_t qx = (fx > 0.0f) ? (uint32_t)fminf(fx, 4095.0f) : 0u;  // NaN: 0
                const uint32_t qy = (fy > 0.0f) ? (uint32_t)fminf(fy, 4095.0f) : 0u;
                key = spread_bits12(qx) | (spread_bits12(qy) << 1);
            }
            S.keys[0][li] = key;
            S.slot[0][li] = (uint16_t)li;
        }
    }
    __syncthreads();

    const uint32_t lower = (1u << lane) - 1u;
    int cur = 0;
    for (int shift = 0; shift < kSortBits; shift += kSortDigitBits) {
        for (int dg = lane; dg < kSortBuckets; dg += 32) S.wcnt[warp][dg] = 0u;
        __syncwarp();
        uint32_t dk[kBatchSortRounds], rk[kBatchSortRounds];
#pragma unroll
        for (int k = 0; k < kBatchSortRounds; k++) {
            const int li = warp * (32 * kBatchSortRounds) + k * 32 + lane;
            const bool valid = li < n;
            const uint32_t dg = (S.keys[cur][li] >> shift) & (kSortBuckets - 1);
            const uint32_t peers = match_digit8(dg, valid);
            rk[k] = S.wcnt[warp][dg] + __popc(peers & lower);
            dk[k] = valid ? dg : kSortBuckets;
            __syncwarp();
            if (valid && (peers & lower) == 0u) S.wcnt[warp][dg] += __popc(peers);
            __syncwarp();
        }
        __syncthreads();
        uint32_t tot = 0u, inc = 0u;
        if (tid < kSortBuckets) {  // per digit: offsets of the warps, block total, scan over digits
            for (int w = 0; w < kBatchSortWarps; w++) {
                const uint32_t v = S.wcnt[w][tid];
                S.wcnt[w][tid] = tot;
                tot += v;
            }
            inc = tot;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += v;
            }
            if (lane == 31) S.part[warp] = inc;
        }
        __syncthreads();
        if (tid < kSortBuckets) {
            uint32_t wb = 0u;
            for (int w = 0; w < warp; w++) wb += S.part[w];
            S.dbase[tid] = wb + inc - tot;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kBatchSortRounds; k++) {
            if (dk[k] < (uint32_t)kSortBuckets) {
                const int li = warp * (32 * kBatchSortRounds) + k * 32 + lane;
                const uint32_t p = S.dbase[dk[k]] + S.wcnt[warp][dk[k]] + rk[k];
                if (p >= (uint32_t)n) {  // cannot happen for a consistent count; never store out of range
                    atomicOr(c.err, kErrSortPermutation);
                    continue;
                }
                S.keys[cur ^ 1][p] = S.keys[cur][li];
                S.slot[cur ^ 1][p] = S.slot[cur][li];
            }
        }
        __syncthreads();
        cur ^= 1;
    }

    // gather the cloud's state in the new order (all loads before the stores)
    int src[kBatchSortRounds];
#pragma unroll
    for (int k = 0; k < kBatchSortRounds; k++) {
        const int li = k * kBatchSortThreads + tid;
        int o = (li < n) ? (int)S.slot[cur][li] : 0;
        if (li < n && o >= n) {
            atomicOr(c.err, kErrSortPermutation);
            o = li;
        }
        src[k] = off + o;
    }
    const double *__restrict__ in[6] = {c.x, c.y, c.vx, c.vy, c.q, c.m};
    double val[6][kBatchSortRounds];
    int ov[kBatchSortRounds];
#pragma unroll
    for (int k = 0; k < kBatchSortRounds; k++) {
        const bool ok = k * kBatchSortThreads + tid < n;
#pragma unroll
        for (int a = 0; a < 6; a++) val[a][k] = ok ? __ldg(in[a] + src[k]) : 0.0;
        ov[k] = ok ? __ldg(c.orig + src[k]) : 0;
    }
#pragma unroll
    for (int k = 0; k < kBatchSortRounds; k++) {
        const int li = k * kBatchSortThreads + tid;
        if (li < n) {
#pragma unroll
            for (int a = 0; a < 6; a++) z.stage[a][off + li] = val[a][k];
            z.orig_stage[off + li] = ov[k];
        }
    }
}

// For the batch autotuner: every cloud squeezed about its own box centre
// so that ~30% of its pairs are inside its cutoff (clouds already that dense
// are copied as they are), written as stage buffer 1 (nothing live there
// between steps).
static __global__ void batch_tune_compress(CloudDev c, const BatchCloud *__restrict__ desc,
                                           const int *__restrict__ seg, const double *__restrict__ box) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int sg = seg[i];
    const double *bb = box + 8 * sg;  // bounding box in bb[4..7]
    const double x0 = bb[4], y0 = bb[5], x1 = bb[6], y1 = bb[7];
    const double half = 0.5 * fmax(x1 - x0, y1 - y0);
    double lam = 1.8 * sqrt(desc[sg].rc2) / half;
    if (!(isfinite(lam) && lam > 0.0 && lam < 1.0)) lam = 1.0;
    const double cx = 0.5 * (x0 + x1), cy = 0.5 * (y0 + y1);
    CloudDev v = c;
    v.rc2 = desc[sg].rc2;
    write_stage_position(v, 1, i, cx + lam * (c.x[i] - cx), cy + lam * (c.y[i] - cy));
}

// Stage buffer 0 from the base positions, with each particle's own cloud's
// filter bound.
static __global__ void batch_init_positions(CloudDev c, const BatchCloud *__restrict__ desc,
                                            const int *__restrict__ seg) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < c.n) {
        CloudDev v = c;
        v.rc2 = desc[seg[i]].rc2;
        write_stage_position(v, 0, i, c.x[i], c.y[i]);
    } else if (i < c.n_pad) {
        for (int b = 0; b < 2; b++) {
            c.px[b][i] = (double)kPadPosition;
            c.py[b][i] = (double)kPadPosition;
            c.pa[b][i] = make_float4(kPadPosition, kPadPosition, kPadPosition * kPadPosition, 0.0f);
            c.pb[b][i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
}

}  // namespace dm
