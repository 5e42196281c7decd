// dm_sort.cuh -- spatial (Morton) ordering of a device-resident cloud.
//
// The all-pairs kernels test every pair, but their cost is decided per warp:
// a warp runs the precise path for a group of j as soon as ONE of its lanes'
// particles is within the cutoff.  With particles in input order a warp's
// particles are spread over the whole cloud and nearly every j group wakes
// it; in Morton order a warp's particles are a compact patch and only the j
// near that patch do.  The cloud therefore lives in Morton order on the
// device; `orig[s]` maps internal slot s back to the caller's particle index
// (used for the thermal RNG counter, for downloads and for the adaptive-dt
// pair pattern, all of which are defined on the caller's order).
//
// Sort: 24-bit Morton keys (12 bits per axis) and a deterministic, stable
// LSD radix sort with 8-bit digits (per-block digit histograms, one scan,
// stable scatter ranked by a ballot-based digit match).  No atomics decide any
// order; the result depends only on the positions.
//
// The key box is the bounding box clipped to mean +- 4 standard deviations
// per axis.  A confined cloud that collapses and re-expands throws a few
// particles metres out while the rest stay within centimetres; over the
// plain bounding box a 12-bit cell is then wider than the cutoff and
// thousands of core particles share one key, so 32-particle groups are no
// longer compact.  Particles outside the clipped box take the edge cells.
#pragma once

#include <cooperative_groups.h>

#include "dm_device.cuh"

namespace dm {
namespace cg = cooperative_groups;

constexpr int kSortThreads = 256;
constexpr int kSortPerBlock = 4 * kSortThreads;  // keys per block
constexpr int kSortBits = 24;
constexpr int kSortDigitBits = 8;  // 24-bit keys: 3 passes
constexpr int kSortBuckets = 1 << kSortDigitBits;

constexpr int kMomentBlocks = 64;  // fixed partition of the moment reduction
constexpr int kMomentFields = 9;   // count, sum dx, sum dy, sum dx^2, sum dy^2, min x, min y, max x, max y

struct SortScratch {
    double *moments;           // [kMomentBlocks][kMomentFields] per-block partials
    double *box;               // [8]: key box x0, y0, extent; -; bounding box min x, min y, max x, max y
    uint32_t *keys[2];
    int *vals[2];
    uint32_t *hist;            // [kSortBuckets * nblocks]
    double *stage[6];          // gather staging for x, y, vx, vy, q, m
    int *orig_stage;
};

// Moments of finite positions: count, sums of the offsets (dx, dy) from an
// origin and of their squares (the origin keeps the second moments well
// conditioned), and the bounding box.
struct Moments {
    double v[kMomentFields];
    __device__ __forceinline__ void clear() {
        for (int k = 0; k < 5; k++) v[k] = 0.0;
        v[5] = v[6] = INFINITY;
        v[7] = v[8] = -INFINITY;
    }
    __device__ __forceinline__ void add(double a, double b, double ox, double oy) {
        if (!(isfinite(a) && isfinite(b))) return;
        const double da = a - ox, db = b - oy;
        v[0] += 1.0;
        v[1] += da;
        v[2] += db;
        v[3] += da * da;
        v[4] += db * db;
        v[5] = fmin(v[5], a);
        v[6] = fmin(v[6], b);
        v[7] = fmax(v[7], a);
        v[8] = fmax(v[8], b);
    }
    __device__ __forceinline__ void merge(const double *o) {
        for (int k = 0; k < 5; k++) v[k] += o[k];
        v[5] = fmin(v[5], o[5]);
        v[6] = fmin(v[6], o[6]);
        v[7] = fmax(v[7], o[7]);
        v[8] = fmax(v[8], o[8]);
    }
    // butterfly over the warp; lane 0's result has a fixed evaluation order
    __device__ __forceinline__ void warp_reduce() {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            double o[kMomentFields];
#pragma unroll
            for (int k = 0; k < kMomentFields; k++) o[k] = __shfl_xor_sync(0xffffffffu, v[k], off);
            merge(o);
        }
    }
};

// Block-wide moments of positions i0, i0 + stride, ... < i1 (fixed
// partition and order: deterministic); the result is valid in thread 0.
__device__ __forceinline__ Moments block_moments(const double *__restrict__ x, const double *__restrict__ y,
                                                 int i0, int i1, int stride, double ox, double oy) {
    __shared__ double s[32][kMomentFields];
    Moments m;
    m.clear();
    for (int i = i0 + (int)threadIdx.x; i < i1; i += stride) m.add(x[i], y[i], ox, oy);
    m.warp_reduce();
    const int warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < kMomentFields; k++) s[warp][k] = m.v[k];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int w = 1; w < nw; w++) m.merge(s[w]);
    __syncthreads();  // s is reused by the next call
    return m;
}

// Key box of a cloud from its moments: the bounding box clipped to mean +-
// 4 standard deviations per axis, as (x0, y0, extent); then the bounding
// box itself.  box[8]: x0, y0, extent, 0, min x, min y, max x, max y.
__device__ __forceinline__ void moments_to_box(const Moments &m, double ox, double oy, double *box) {
    double lo[2] = {0.0, 0.0}, hi[2] = {0.0, 0.0};
    const double n = m.v[0];
    if (n > 0.0) {
        const double org[2] = {ox, oy};
        for (int a = 0; a < 2; a++) {
            const double mean = m.v[1 + a] / n;
            const double sd = sqrt(fmax(m.v[3 + a] / n - mean * mean, 0.0));
            lo[a] = fmax(m.v[5 + a], org[a] + mean - 4.0 * sd);
            hi[a] = fmin(m.v[7 + a], org[a] + mean + 4.0 * sd);
            if (!(lo[a] <= hi[a])) {  // degenerate: fall back to the bounding box
                lo[a] = m.v[5 + a];
                hi[a] = m.v[7 + a];
            }
        }
    }
    box[0] = lo[0];
    box[1] = lo[1];
    box[2] = fmax(hi[0] - lo[0], hi[1] - lo[1]);
    box[3] = 0.0;
    for (int k = 0; k < 4; k++) box[4 + k] = (n > 0.0) ? m.v[5 + k] : 0.0;
}

__device__ __forceinline__ double finite_or_zero(double v) { return isfinite(v) ? v : 0.0; }

// Per-block moments of one cloud's positions (origin: its first particle).
static __global__ void __launch_bounds__(256) sort_moments(const double *__restrict__ x,
                                                           const double *__restrict__ y, int n, double *part) {
    const double ox = finite_or_zero(x[0]), oy = finite_or_zero(y[0]);
    const Moments m = block_moments(x, y, blockIdx.x * blockDim.x, n, gridDim.x * blockDim.x, ox, oy);
    if (threadIdx.x == 0)
        for (int k = 0; k < kMomentFields; k++) part[blockIdx.x * kMomentFields + k] = m.v[k];
}

// One warp: the per-block moments summed in fixed order, then the key box.
static __global__ void sort_box(const double *__restrict__ part, int nparts, const double *__restrict__ x,
                                const double *__restrict__ y, double *box) {
    Moments m;
    m.clear();
    for (int b = (int)threadIdx.x; b < nparts; b += 32) m.merge(part + b * kMomentFields);
    m.warp_reduce();
    if (threadIdx.x == 0) moments_to_box(m, finite_or_zero(x[0]), finite_or_zero(y[0]), box);
}

// Spreads the low 12 bits of v to the even bit positions.
__device__ __forceinline__ uint32_t spread_bits12(uint32_t v) {
    v &= 0x00000FFFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

// Lanes of the warp holding the same 8-bit digit as this one, among the
// lanes with `valid` set: one ballot per digit bit.  Eight ballots cost far
// less than __match_any_sync when 32 warps of one block issue them (the
// match unit's throughput, not the ballots', bounds a one-block sort).
__device__ __forceinline__ uint32_t match_digit8(uint32_t d, bool valid) {
    uint32_t m = __ballot_sync(0xffffffffu, valid);
#pragma unroll
    for (int b = 0; b < kSortDigitBits; b++) {
        const bool bit = (d >> b) & 1u;
        const uint32_t bal = __ballot_sync(0xffffffffu, bit);
        m &= bit ? bal : ~bal;
    }
    return m;
}

static __global__ void sort_keys(const double *__restrict__ x, const double *__restrict__ y, int n,
                                 const double *__restrict__ box, uint32_t *keys, int *vals) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x0 = box[0], y0 = box[1], ext = box[2];
    const double scale = (ext > 0.0 && isfinite(ext)) ? 4095.0 / ext : 0.0;
    const double fx = (x[i] - x0) * scale, fy = (y[i] - y0) * scale;
    const uint32_t qx = (fx > 0.0) ? (uint32_t)fmin(fx, 4095.0) : 0u;
    const uint32_t qy = (fy > 0.0) ? (uint32_t)fmin(fy, 4095.0) : 0u;
    keys[i] = spread_bits12(qx) | (spread_bits12(qy) << 1);
    vals[i] = i;
}

static __global__ void __launch_bounds__(kSortThreads) radix_hist(const uint32_t *__restrict__ keys, int n,
                                                                  int shift, uint32_t *hist) {
    __shared__ uint32_t h[kSortBuckets];
    if (threadIdx.x < kSortBuckets) h[threadIdx.x] = 0u;
    __syncthreads();
    for (int k = 0; k < 4; k++) {
        const int e = blockIdx.x * kSortPerBlock + k * kSortThreads + threadIdx.x;
        if (e < n) atomicAdd(&h[(keys[e] >> shift) & (kSortBuckets - 1)], 1u);
    }
    __syncthreads();
    if (threadIdx.x < kSortBuckets) hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of len entries in one block of 1024 threads.  Warp w owns
// the w-th of 32 consecutive segments and reads it 32 entries at a time
// (lane l takes entry 32 r + l of the segment, so every load is one
// coalesced row): first the segment's total, then, after a scan of the 32
// totals, the segment again, row by row, each row scanned by shuffles on top
// of the carried prefix.  (A thread per contiguous run of entries made every
// warp load touch 32 cache lines: 110 us for the 65,536 entries of a
// 262,144-particle sort.)
static __global__ void __launch_bounds__(1024) radix_scan(uint32_t *hist, int len) {
    __shared__ uint32_t wsum[32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int seg = (len + 31) / 32;
    const int lo = min(len, warp * seg), hi = min(len, lo + seg);
    uint32_t s = 0;
    for (int e = lo + lane; e < hi; e += 32) s += hist[e];
    s = __reduce_add_sync(0xffffffffu, s);
    if (lane == 0) wsum[warp] = s;
    __syncthreads();
    if (warp == 0) {  // exclusive prefix of the 32 segment totals
        const uint32_t v = wsum[lane];
        uint32_t inc = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, inc, off);
            if (lane >= off) inc += t;
        }
        wsum[lane] = inc - v;
    }
    __syncthreads();
    uint32_t carry = wsum[warp];
    for (int r = lo; r < hi; r += 32) {
        const int e = r + lane;
        const uint32_t v = (e < hi) ? hist[e] : 0u;
        uint32_t inc = v;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, inc, off);
            if (lane >= off) inc += t;
        }
        if (e < hi) hist[e] = carry + inc - v;
        carry += __shfl_sync(0xffffffffu, inc, 31);
    }
}

// Stable scatter: elements are ranked in index order (chunk, warp, lane).
static __global__ void __launch_bounds__(kSortThreads) radix_scatter(
    const uint32_t *__restrict__ kin, const int *__restrict__ vin, uint32_t *kout, int *vout, int n,
    int shift, const uint32_t *__restrict__ hist) {
    constexpr int NWARP = kSortThreads / 32;
    __shared__ uint32_t base[kSortBuckets];
    __shared__ uint32_t wcnt[NWARP][kSortBuckets];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x < kSortBuckets) base[threadIdx.x] = hist[threadIdx.x * gridDim.x + blockIdx.x];
    for (int k = 0; k < 4; k++) {
        for (int e = threadIdx.x; e < NWARP * kSortBuckets; e += kSortThreads) (&wcnt[0][0])[e] = 0u;
        __syncthreads();
        const int e = blockIdx.x * kSortPerBlock + k * kSortThreads + threadIdx.x;
        const bool valid = e < n;
        const uint32_t key = valid ? kin[e] : 0u;
        const int d = (int)((key >> shift) & (kSortBuckets - 1));
        const uint32_t peers = match_digit8((uint32_t)d, valid);
        const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t pos = base[d] + rank;
            for (int w = 0; w < warp; w++) pos += wcnt[w][d];
            kout[pos] = key;
            vout[pos] = vin[e];
        }
        __syncthreads();
        if (threadIdx.x < kSortBuckets) {
            uint32_t add = 0;
            for (int w = 0; w < NWARP; w++) add += wcnt[w][threadIdx.x];
            base[threadIdx.x] += add;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// One-launch sort for clouds of up to kSmallSortMax particles: a cluster of
// CTAS blocks, block r owning sorted positions [r*P, (r+1)*P),
// P = kSmallSortMax / CTAS.  Key box, keys, the three 8-bit LSD
// passes and the gather of the cloud's arrays in the new order run in one
// launch: per pass each block counts its digits per warp, the blocks'
// digit totals meet through distributed shared memory, and every element is
// stored straight into the shared memory of the block owning its new
// position.  The multi-kernel path above needs fifteen dependent launches
// (~0.1 ms at n = 16384); a single block was no better (one SM's issue rate).
//
// Element order: block r, warp w, round k, lane l is element
// r*P + w*32*R + k*32 + l (R = P / threads).  Digits are ranked in that order
// (lanes with equal digits found by match_digit8) and bases are laid out
// digit-major over (digit, block, warp), so the sort is stable and depends
// only on the positions.  The key
// box and keys are FP32 functions of the positions' hi parts: GB300's FP64
// rate (~2 FMA per clock per SM) would dominate a pass over 16384 doubles,
// and any order is correct (the permutation moves every array together).
// ---------------------------------------------------------------------------
constexpr int kSmallSortMax = 16384;
constexpr int kErrSortPermutation = 8;  // error bit: the cluster sort's ranks were inconsistent
constexpr int kSortClusterThreads = 512;
constexpr int kSortClusterWarps = kSortClusterThreads / 32;

// CTAS blocks of PER elements, ROUNDS per thread: 8 (a portable cluster) or
// 16 (non-portable; half the elements per SM)
template <int CTAS>
struct SortClusterShape {
    static constexpr int per = kSmallSortMax / CTAS;
    static constexpr int rounds = per / kSortClusterThreads;
    static_assert(rounds * kSortClusterThreads == per, "whole rounds per thread");
};

template <int CTAS>
struct SortClusterSmem {
    static constexpr int kPer = SortClusterShape<CTAS>::per;
    uint32_t keys[2][kPer];
    uint16_t slot[2][kPer];
    uint32_t wcnt[kSortClusterWarps][kSortBuckets];  // per-warp digit counts, then offsets within the block
    uint32_t ctot[kSortBuckets];      // this block's digit totals (read by the whole cluster)
    uint32_t dbase[kSortBuckets];     // first sorted position of (digit, this block)
    uint32_t part[kSortBuckets / 32];
    float wmom[kSortClusterWarps][kMomentFields];
    float mom[kMomentFields];  // this block's moments (read by the whole cluster)
    float box[3];
};
template <int CTAS>
constexpr size_t sort_cluster_smem() { return sizeof(SortClusterSmem<CTAS>); }

__device__ __forceinline__ void moments_f32_add(float *v, float4 a, float ox, float oy) {
    if (!(isfinite(a.x) && isfinite(a.y))) return;
    const float dx = a.x - ox, dy = a.y - oy;
    v[0] += 1.0f;
    v[1] += dx;
    v[2] += dy;
    v[3] = fmaf(dx, dx, v[3]);
    v[4] = fmaf(dy, dy, v[4]);
    v[5] = fminf(v[5], a.x);
    v[6] = fminf(v[6], a.y);
    v[7] = fmaxf(v[7], a.x);
    v[8] = fmaxf(v[8], a.y);
}

__device__ __forceinline__ void moments_f32_merge(float *v, const float *o) {
    for (int k = 0; k < 5; k++) v[k] += o[k];
    v[5] = fminf(v[5], o[5]);
    v[6] = fminf(v[6], o[6]);
    v[7] = fmaxf(v[7], o[7]);
    v[8] = fmaxf(v[8], o[8]);
}

// pa0: the FP32 hi parts of the current positions (stage buffer 0 holds them
// at every step boundary).  The cloud's x, y, vx, vy, q, m and orig end up in
// the new order, with stage buffer 0 and the group boxes rewritten.
// Launched as one cluster of CTAS blocks.
template <int CTAS>
static __global__ void __launch_bounds__(kSortClusterThreads, 1)
    sort_cluster(const float4 *__restrict__ pa0, CloudDev c, SortScratch z) {
    constexpr int kSortClusterCtas = CTAS;
    constexpr int kSortClusterPer = SortClusterShape<CTAS>::per;
    constexpr int kSortClusterRounds = SortClusterShape<CTAS>::rounds;
    pdl_wait();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    SortClusterSmem<CTAS> &S = *reinterpret_cast<SortClusterSmem<CTAS> *>(smem_raw);
    cg::cluster_group cl = cg::this_cluster();
    const int r = (int)cl.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int n = c.n;
    const int e0 = r * kSortClusterPer;

    // this block's positions, loaded once (moments, then keys)
    float4 pos[kSortClusterRounds];
#pragma unroll
    for (int k = 0; k < kSortClusterRounds; k++) {
        const int e = e0 + k * kSortClusterThreads + tid;
        pos[k] = (e < n) ? pa0[e] : make_float4(NAN, NAN, 0.0f, 0.0f);
    }
    // moments of this block's slice, then of the cloud: lanes 0..CTAS-1 of warp 0
    // fetch the cluster's blocks' moments and merge them in a fixed butterfly
    // (commutative steps), so every block derives the same key box
    const float4 p0 = pa0[0];
    const float ox = isfinite(p0.x) ? p0.x : 0.0f, oy = isfinite(p0.y) ? p0.y : 0.0f;
    {
        float v[kMomentFields] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, INFINITY, INFINITY, -INFINITY, -INFINITY};
#pragma unroll
        for (int k = 0; k < kSortClusterRounds; k++) moments_f32_add(v, pos[k], ox, oy);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            float o[kMomentFields];
#pragma unroll
            for (int k = 0; k < kMomentFields; k++) o[k] = __shfl_xor_sync(0xffffffffu, v[k], off);
            moments_f32_merge(v, o);
        }
        if (lane == 0)
            for (int k = 0; k < kMomentFields; k++) S.wmom[warp][k] = v[k];
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < kSortClusterWarps; w++) moments_f32_merge(v, S.wmom[w]);
            for (int k = 0; k < kMomentFields; k++) S.mom[k] = v[k];
        }
    }
    cl.sync();
    if (warp == 0) {
        float v[kMomentFields];
        const float *mb = cl.map_shared_rank(S.mom, lane & (kSortClusterCtas - 1));
#pragma unroll
        for (int k = 0; k < kMomentFields; k++) v[k] = mb[k];
#pragma unroll
        for (int off = 1; off < kSortClusterCtas; off <<= 1) {
            float o[kMomentFields];
#pragma unroll
            for (int k = 0; k < kMomentFields; k++) o[k] = __shfl_xor_sync(0xffffffffu, v[k], off);
            moments_f32_merge(v, o);
        }
        if (lane == 0) {
            // bounding box clipped to mean +- 4 sd per axis
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
            if (r == 0) {  // the key box and the bounding box, as the multi-kernel path writes them
                z.box[0] = S.box[0];
                z.box[1] = S.box[1];
                z.box[2] = S.box[2];
                z.box[3] = 0.0;
                for (int k = 0; k < 4; k++) z.box[4 + k] = (v[0] > 0.0f) ? (double)v[5 + k] : 0.0;
            }
        }
    }
    __syncthreads();
    {
        const float x0 = S.box[0], y0 = S.box[1], ext = S.box[2];
        const float scale = (ext > 0.0f && isfinite(ext)) ? 4095.0f / ext : 0.0f;
#pragma unroll
        for (int k = 0; k < kSortClusterRounds; k++) {
            const int li = k * kSortClusterThreads + tid, e = e0 + li;
            uint32_t key = 0u;
            if (e < n) {
                const float fx = (pos[k].x - x0) * scale, fy = (pos[k].y - y0) * scale;
                const uint32_t qx = (fx > 0.0f) ? (uint32_t)fminf(fx, 4095.0f) : 0u;  // NaN: 0
                const uint32_t qy = (fy > 0.0f) ? (uint32_t)fminf(fy, 4095.0f) : 0u;
                key = spread_bits12(qx) | (spread_bits12(qy) << 1);
            }
            S.keys[0][li] = key;
            S.slot[0][li] = (uint16_t)e;
        }
    }
    __syncthreads();

    const uint32_t lower = (1u << lane) - 1u;
    int cur = 0;
    for (int shift = 0; shift < kSortBits; shift += kSortDigitBits) {
        for (int d = lane; d < kSortBuckets; d += 32) S.wcnt[warp][d] = 0u;
        __syncwarp();
        uint32_t dk[kSortClusterRounds], rk[kSortClusterRounds];
#pragma unroll
        for (int k = 0; k < kSortClusterRounds; k++) {
            const int li = warp * (32 * kSortClusterRounds) + k * 32 + lane;
            const bool valid = e0 + li < n;
            const uint32_t d = (S.keys[cur][li] >> shift) & (kSortBuckets - 1);
            const uint32_t peers = match_digit8(d, valid);
            rk[k] = S.wcnt[warp][d] + __popc(peers & lower);  // rank within the warp
            dk[k] = valid ? d : kSortBuckets;
            __syncwarp();
            if (valid && (peers & lower) == 0u) S.wcnt[warp][d] += __popc(peers);
            __syncwarp();
        }
        __syncthreads();
        if (tid < kSortBuckets) {  // per digit: offsets of the warps, block total
            uint32_t run = 0u;
            for (int w = 0; w < kSortClusterWarps; w++) {
                const uint32_t v = S.wcnt[w][tid];
                S.wcnt[w][tid] = run;
                run += v;
            }
            S.ctot[tid] = run;
        }
        cl.sync();  // every block's totals are complete
        uint32_t tot = 0u, pre = 0u, inc = 0u;
        if (tid < kSortBuckets) {
            for (int b = 0; b < kSortClusterCtas; b++) {
                const uint32_t v = *cl.map_shared_rank(&S.ctot[tid], b);
                tot += v;
                pre += (b < r) ? v : 0u;
            }
            inc = tot;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, inc, off);
                if (lane >= off) inc += v;
            }
            if (lane == 31) S.part[warp] = inc;
        }
        __syncthreads();
        if (tid < kSortBuckets) {
            uint32_t wb = 0u;
            for (int w = 0; w < warp; w++) wb += S.part[w];
            S.dbase[tid] = wb + inc - tot + pre;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kSortClusterRounds; k++) {
            if (dk[k] < (uint32_t)kSortBuckets) {
                const int li = warp * (32 * kSortClusterRounds) + k * 32 + lane;
                const uint32_t pos = S.dbase[dk[k]] + S.wcnt[warp][dk[k]] + rk[k];
                if (pos >= (uint32_t)n) {  // cannot happen for a consistent count; never store out of range
                    atomicOr(c.err, kErrSortPermutation);
                    continue;
                }
                const int dst = (int)(pos / kSortClusterPer), off = (int)(pos % kSortClusterPer);
                *cl.map_shared_rank(&S.keys[cur ^ 1][off], dst) = S.keys[cur][li];
                *cl.map_shared_rank(&S.slot[cur ^ 1][off], dst) = S.slot[cur][li];
            }
        }
        cl.sync();  // all elements placed; all remote reads of this pass done
        cur ^= 1;
    }

    // gather: new slot s takes old slot S.slot[cur][s - e0]; plain loads (the
    // arrays are overwritten in place below), all issued before any store
    int src[kSortClusterRounds];
#pragma unroll
    for (int k = 0; k < kSortClusterRounds; k++) {
        const int li = k * kSortClusterThreads + tid, s = e0 + li;
        int o = (s < n) ? (int)S.slot[cur][li] : 0;
        if (s < n && o >= n) {  // as above: flag and keep the slot rather than read out of range
            atomicOr(c.err, kErrSortPermutation);
            o = s;
        }
        src[k] = o;
    }
    const double *in[6] = {c.x, c.y, c.vx, c.vy, c.q, c.m};
    double val[6][kSortClusterRounds];
    int ov[kSortClusterRounds];
#pragma unroll
    for (int k = 0; k < kSortClusterRounds; k++) {
        const bool ok = e0 + k * kSortClusterThreads + tid < n;
#pragma unroll
        for (int a = 0; a < 6; a++) val[a][k] = ok ? in[a][src[k]] : 0.0;
        ov[k] = ok ? c.orig[src[k]] : 0;
    }
    // Every block of the cluster holds its sources in registers, and the
    // cluster barrier orders those loads before any block's stores.  The
    // cluster covers every slot of the cloud, so the cloud's arrays are
    // rewritten in place in the new order, with stage buffer 0 (the first
    // stage's inputs), the padding slots and the 32-particle group boxes.
    cl.sync();
#pragma unroll
    for (int k = 0; k < kSortClusterRounds; k++) {
        const int s = e0 + k * kSortClusterThreads + tid;  // a warp holds 32 consecutive slots
        float x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
        if (s < n) {
            const double x = val[0][k], y = val[1][k];
            c.x[s] = x;
            c.y[s] = y;
            c.vx[s] = val[2][k];
            c.vy[s] = val[3][k];
            c.q[s] = val[4][k];
            c.m[s] = val[5][k];
            c.orig[s] = ov[k];
            write_stage_position(c, 0, s, x, y);
            x0 = x1 = __double2float_rn(x);  // the hi parts write_stage_position stored
            y0 = y1 = __double2float_rn(y);
        } else if (s < c.n_pad) {
            for (int b = 0; b < 2; b++) {
                c.px[b][s] = (double)kPadPosition;
                c.py[b][s] = (double)kPadPosition;
                c.pa[b][s] = make_float4(kPadPosition, kPadPosition, kPadPosition * kPadPosition, 0.0f);
                c.pb[b][s] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
            c.q[s] = 0.0;
            c.m[s] = 1.0;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
            y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
            x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
            y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
        }
        if (lane == 0 && s < c.n_pad) c.gbox[0][s >> 5] = make_float4(x0, y0, x1, y1);
    }
}

// new slot s takes old slot perm[s]: gather into staging ...
static __global__ void permute_gather(CloudDev c, const int *__restrict__ perm, SortScratch z) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= c.n) return;
    const int o = perm[s];
    z.stage[0][s] = c.x[o];
    z.stage[1][s] = c.y[o];
    z.stage[2][s] = c.vx[o];
    z.stage[3][s] = c.vy[o];
    z.stage[4][s] = c.q[o];
    z.stage[5][s] = c.m[o];
    z.orig_stage[s] = c.orig[o];
}

// ... and copy back (the cloud's array addresses never change, so captured
// CUDA graphs stay valid)
static __global__ void permute_commit(CloudDev c, SortScratch z) {
    pdl_wait();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= c.n) return;
    c.x[s] = z.stage[0][s];
    c.y[s] = z.stage[1][s];
    c.vx[s] = z.stage[2][s];
    c.vy[s] = z.stage[3][s];
    c.q[s] = z.stage[4][s];
    c.m[s] = z.stage[5][s];
    c.orig[s] = z.orig_stage[s];
}

// An upload in the caller's order (staging arrays 0..3: x, y, vx, vy) put
// straight into the cloud's current internal order, with stage buffer 0 and
// the boxes of its 32-particle groups: charges, masses and the order itself
// stay where they are (the next re-sort starts from them).
static __global__ void upload_internal_order(CloudDev c, SortScratch z) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= c.n_pad) return;  // whole warps: n_pad is a multiple of 64
    float x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
    if (s < c.n) {
        const int o = c.orig[s];
        const double x = z.stage[0][o], y = z.stage[1][o];
        c.x[s] = x;
        c.y[s] = y;
        c.vx[s] = z.stage[2][o];
        c.vy[s] = z.stage[3][o];
        write_stage_position(c, 0, s, x, y);
        const float4 A = c.pa[0][s];
        x0 = x1 = A.x;
        y0 = y1 = A.y;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, off));
        y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, off));
        x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, off));
        y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, off));
    }
    if ((threadIdx.x & 31) == 0) c.gbox[0][s >> 5] = make_float4(x0, y0, x1, y1);
}

static __global__ void set_identity(int *orig, int n) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) orig[s] = s;
}

// out[orig[s]] = in[s] for up to four arrays (internal -> caller order).
static __global__ void scatter_to_caller(const int *__restrict__ orig, int n, const double *a0,
                                         const double *a1, const double *a2, const double *a3,
                                         double *o0, double *o1, double *o2, double *o3) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int o = orig[s];
    if (a0) o0[o] = a0[s];
    if (a1) o1[o] = a1[s];
    if (a2) o2[o] = a2[s];
    if (a3) o3[o] = a3[s];
}

// Four arrays of n doubles copied element for element (coalesced on both
// sides): caller buffers in page-locked host memory read or written by the
// device itself over the host link, in place of four DMA copies.  err_src /
// err_dst (optional): the device error word copied along with them.
static __global__ void copy4(int n, const double *__restrict__ i0, const double *__restrict__ i1,
                             const double *__restrict__ i2, const double *__restrict__ i3, double *o0,
                             double *o1, double *o2, double *o3, const int *err_src, int *err_dst) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (err_dst && s == 0) *err_dst = *err_src;
    if (s >= n) return;
    o0[s] = i0[s];
    o1[s] = i1[s];
    o2[s] = i2[s];
    o3[s] = i3[s];
}

// out[s] = in[orig[s]] for up to two arrays (caller -> internal order).
static __global__ void gather_from_caller(const int *__restrict__ orig, int n, const double *i0,
                                          const double *i1, double *o0, double *o1) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int o = orig[s];
    if (i0) o0[s] = i0[o];
    if (i1) o1[s] = i1[o];
}

}  // namespace dm
