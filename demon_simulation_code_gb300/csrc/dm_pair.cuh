// dm_pair.cuh -- tiled all-pairs shielded-Coulomb (Yukawa) kernels with the
// RK4 stage epilogue fused in, for sm_103a.
//
// Replaces ShieldedCoulombForce::force1..4 (ShieldedCoulombForce.cpp:37-237)
// plus, in the epilogue, the per-particle forces, CacheOperator and the RK4
// stage/combine loops (see dm_device.cuh).
//
// Work decomposition (owner computes, no atomics on forces):
//   * an i-tile of NT*ILP particles belongs to one thread-block CLUSTER of S
//     CTAs; thread t of every CTA owns particles i = tile*NT*ILP + k*NT + t,
//     k < ILP, kept in registers;
//   * CTA rank r of the cluster sweeps the r-th of S contiguous j ranges,
//     staging JT j particles at a time in shared memory;
//   * each pair is first filtered with the expanded distance
//       |p_i|^2 + |p_j|^2 - 2 p_i.p_j < (r_c + margin)^2
//     (2 FMAs per pair with |p_j|^2 precomputed), and only surviving pairs
//     run the precise force arithmetic -- the GPU form of the reference's
//     early exit for kappa*r >= 10 (ShieldedCoulombForce.cpp:178-180);
//   * the S partial sums of a particle are combined through distributed
//     shared memory (DSMEM) inside the cluster, in rank order, and the
//     stage epilogue runs once per particle.
#pragma once

#include <cooperative_groups.h>

#include <type_traits>

#include "dm_device.cuh"

namespace dm {
namespace cg = cooperative_groups;

// log2(e) as a float pair, and Taylor coefficients c_k = (-ln 2)^k / k! of
// 2^-f on |f| <= 1/2 (degree 7: truncation error < 6e-9 relative).
struct ExpConsts {
    float l2e_hi, l2e_lo;
    float c[8];
};

// e^{-a} for a >= 0 in FP32 with the argument carried as a float pair:
// t = a*log2(e) = t_hi + t_lo exactly to ~2^-48, n = rint(t_hi),
// f = (t_hi - n) + t_lo, e^{-a} = 2^-n * poly(f) (Cody-Waite style range
// reduction; the 2^-n scale is exact).
__device__ __forceinline__ float exp_neg(float a, const ExpConsts &E) {
    const float t_hi = a * E.l2e_hi;
    const float t_lo = fmaf(a, E.l2e_hi, -t_hi) + a * E.l2e_lo;
    const float n = rintf(t_hi);
    const float f = (t_hi - n) + t_lo;
    float p = E.c[7];
#pragma unroll
    for (int k = 6; k >= 0; k--) p = fmaf(p, f, E.c[k]);
    const int e = 127 - (int)n;
    const float scale = __int_as_float((e > 0 ? e : 0) << 23);
    return p * scale;
}

// e^{-kappa r} on the SFU with kappa*log2(e) = k_hi + k_lo given as a float
// pair: t = k_hi r rounded to FP32 (absolute error up to ~1e-6 at kappa r =
// 10), and its residue t_lo (exact to ~2^-48) put back to first order,
// 2^{-(t + t_lo)} = 2^{-t} (1 - t_lo ln 2).  Relative error: the hardware
// ex2.approx (a few ulp) plus (t_lo ln 2)^2 / 2 < 1e-12, for the FP32 r given.
__device__ __forceinline__ float exp_neg_kr(float r, float k_hi, float k_lo) {
    const float t = k_hi * r;
    const float t_lo = fmaf(k_lo, r, fmaf(k_hi, r, -t));
    float e;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(-t));
    return e * fmaf(-t_lo, 0.693147182f, 1.0f);
}

// Sum kept as an unevaluated pair hi + lo: Knuth's TwoSum gives the exact
// rounding error of each addition, accumulated in lo (error ~ n eps^2 of the
// sum of magnitudes).
struct TwoFloatSum {
    float hi = 0.0f, lo = 0.0f;
    __device__ __forceinline__ void add(float v) {
        const float t = hi + v;
        const float bp = t - hi;
        lo += (hi - (t - bp)) + (v - bp);
        hi = t;
    }
};

// Kahan (compensated) accumulation: true sum ~= s - c.
__device__ __forceinline__ void kahan_add(float &s, float &c, float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

struct PairTuning {
    int nt, ilp, jt, s;
};

// ---------------------------------------------------------------------------
// FP32-compensated kernel.
//
// CTA = G j-groups x NI i-lanes.  Lane t of every group owns the ILP
// particles i = tile*NI*ILP + k*NI + t; group g sweeps every G-th j of each
// shared-memory tile, so all G groups reuse one tile.  Hot registers per
// particle: -2*xh, -2*yh (packed in pairs for the f32x2 FMA), the filter
// threshold and the Kahan sums; the rest of the particle's data lives in
// shared memory.
//
// Filter hits are not evaluated where they are found.  Per j the warp takes
// one uniform branch (vote over lanes and slots); when some lane's filter
// fired, the warp ballots each slot and queues (j, ballot) in shared memory.
// Every 32 queued entries of a slot (and at the end of a tile) a 32x32
// bit-matrix transpose gives each lane the set of queued j it hit, and all
// lanes run the precise path on their own hits together.  Each lane
// accumulates only into its own sums, so the result is deterministic and no
// atomics are needed; SIMD utilisation of the precise path goes from ~1/32
// (sparse) or the hit fraction (dense) to mean/max of the per-lane hit count.
// ---------------------------------------------------------------------------
template <int NW, int ILP, int TC>
struct Fp32cSmem {
    // j tile: TC 4-j chunks as structure of arrays (x, y, |p|^2) + precise data
    static constexpr size_t tile = (size_t)TC * (3 * sizeof(float4) + 4 * sizeof(float4));
    static constexpr size_t cold = (size_t)ILP * 32 * sizeof(float4);
    static constexpr size_t acc = (size_t)NW * ILP * 32 * sizeof(float4);
    static constexpr size_t red = (size_t)ILP * 32 * sizeof(float4);
    // culling: near and inside group lists (NT each) and their per-warp counts
    static constexpr size_t glist = 2 * ((size_t)NW * 32 * sizeof(int) + NW * sizeof(int));
    static constexpr size_t bytes = tile + cold + acc + red + glist;
    // s_red, in float4 units from the start of shared memory
    static constexpr size_t red_offset = (tile + cold + acc) / sizeof(float4);
};

// Conservative FP32 test: can any point of box a come within the cutoff of
// any point of box b?  Boxes are (x0, y0, x1, y1) of FP32 hi parts; the true
// positions lie within an ulp of them and the box arithmetic rounds, so the
// gaps are shrunk by 2^-20 of the largest coordinate before comparing with
// r_c^2 (already rounded up, rc2_hi).
__device__ __forceinline__ bool boxes_near(const float4 &a, const float4 &b, float rc2_hi) {
    const float gx = fmaxf(a.x - b.z, b.x - a.z);
    const float gy = fmaxf(a.y - b.w, b.y - a.w);
    const float big = fmaxf(fmaxf(fmaxf(fabsf(a.x), fabsf(a.z)), fmaxf(fabsf(b.x), fabsf(b.z))),
                            fmaxf(fmaxf(fabsf(a.y), fabsf(a.w)), fmaxf(fabsf(b.y), fabsf(b.w))));
    const float m = 9.5367431640625e-7f * big;  // 2^-20
    const float dx = fmaxf(0.0f, gx - m), dy = fmaxf(0.0f, gy - m);
    return !(fmaf(dx, dx, dy * dy) >= rc2_hi);  // NaN: near (never drops a pair)
}

// Conservative FP32 test: is every point of box a within the cutoff of every
// point of box b?  The farthest separations are widened by 2^-20 of the
// largest coordinate and the squared distance must stay below 0.999 r_c^2,
// so for every pair of the two groups the reference's FP64 test
// kappa*sqrt(dx*dx + dy*dy) < 10 holds (NaN: false).
__device__ __forceinline__ bool boxes_inside(const float4 &a, const float4 &b, float rc2_lo) {
    const float gx = fmaxf(a.z - b.x, b.z - a.x);
    const float gy = fmaxf(a.w - b.y, b.w - a.y);
    const float big = fmaxf(fmaxf(fmaxf(fabsf(a.x), fabsf(a.z)), fmaxf(fabsf(b.x), fabsf(b.z))),
                            fmaxf(fmaxf(fabsf(a.y), fabsf(a.w)), fmaxf(fabsf(b.y), fabsf(b.w))));
    const float m = 9.5367431640625e-7f * big;  // 2^-20
    const float dx = gx + m, dy = gy + m;
    return fmaf(dx, dx, dy * dy) < 0.999f * rc2_lo;
}

// 32x32 bit-matrix transpose across a warp: lane r holds row r on entry and
// column r (bit c = bit r of row c) on exit.
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x) {
    const int lane = threadIdx.x & 31;
    const uint32_t masks[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
    for (int st = 0; st < 5; st++) {
        const int j = 16 >> st;
        const uint32_t m = masks[st];
        const uint32_t y = __shfl_xor_sync(0xffffffffu, x, j);
        // lanes with bit j clear keep their low half-blocks and take the
        // partner's; lanes with it set the reverse
        if (lane & j) x = (x & ~m) | ((y & ~m) >> j);
        else x = (x & m) | ((y & m) << j);
    }
    return x;
}

// Calls f(std::integral_constant<int, k>) for k = 0 .. K-1 (compile-time k).
template <int K, typename F>
__device__ __forceinline__ void static_for(F &&f) {
    if constexpr (K > 0) {
        static_for<K - 1>(f);
        f(std::integral_constant<int, K - 1>{});
    }
}

struct PairCtx {
    float xl, yl, qc;
    int ii;
};

// The pair force on i from j (added into px, py; nothing for j == i or a
// pair outside the cutoff).
__device__ __forceinline__ void precise_pair(const StageParams &P, int b,
                                             float xh_i, float yh_i, const PairCtx &ic,
                                             const float4 &A, const float4 &Bj, int jg, float &px,
                                             float &py) {
    if (jg == ic.ii) return;
    const float dx = (xh_i - A.x) + (ic.xl - Bj.x);
    const float dy = (yh_i - A.y) + (ic.yl - Bj.y);
    const float r2 = fmaf(dx, dx, dy * dy);
    bool in = r2 < P.rc2_hi;
    if (in && !(r2 < P.rc2_lo)) {
        // borderline: decide exactly as the reference does
        double r, a;
        in = ref_in_cutoff(P.c.px[b][ic.ii] - P.c.px[b][jg], P.c.py[b][ic.ii] - P.c.py[b][jg],
                           P.f.shielding, r, a);
    }
    if (!in) return;
    // 1/r: hardware rsqrt + one Newton step
    float y = rsqrtf(r2);
    const float h = r2 * y;
    const float ee = fmaf(-h, y, 1.0f);
    y = fmaf(0.5f * ee, y, y);
    const float ex = exp_neg_kr(r2 * y, P.kl2e_hi, P.kl2e_lo);
    // C q_i q_j (1 + kappa r) e^{-kappa r} / r^3 = C q_i q_j e^{-kappa r} y^2 (y + kappa), y = 1/r
    const float s = ((ic.qc * A.w) * ex) * ((y * y) * (y + P.kappa_f));
    px = fmaf(s, dx, px);
    py = fmaf(s, dy, py);
}

// The pair force on i from j for a pair known to be inside the cutoff (a
// j group entirely within reach of the i tile, never one of the tile's own
// groups, so j != i): the precise arithmetic with no cutoff test.
__device__ __forceinline__ void inside_pair(const StageParams &P, float xh_i, float yh_i, const PairCtx &ic,
                                            float xj, float yj, const float4 &Bj, float &px, float &py) {
    const float dx = (xh_i - xj) + (ic.xl - Bj.x);
    const float dy = (yh_i - yj) + (ic.yl - Bj.y);
    const float r2 = fmaf(dx, dx, dy * dy);
    float y = rsqrtf(r2);
    const float h = r2 * y;
    const float ee = fmaf(-h, y, 1.0f);
    y = fmaf(0.5f * ee, y, y);
    const float ex = exp_neg_kr(r2 * y, P.kl2e_hi, P.kl2e_lo);
    const float s = ((ic.qc * Bj.z) * ex) * ((y * y) * (y + P.kappa_f));
    px = fmaf(s, dx, px);
    py = fmaf(s, dy, py);
}

// The FP32C sweep of one i tile against rank `rank` of S of the j chunks:
// i-side setup, filtered j loop with the compaction queue, and the combine
// of the NW warps' Kahan sums into s_red[TILE] = (sx, sy, cx, cy).  Ends with
// the block synchronised.  `P` may live in shared memory (batched kernel).
// Particles are those of P.c (n = P.c.n); j at or beyond n read as padding,
// so a cloud needs no padding of its own.
template <int NW, int ILP, int TC, bool CULL = false>
__device__ __forceinline__ void fp32c_sweep(const StageParams &P, const ExpConsts &E, int tile,
                                            int rank, int S, unsigned char *smem_raw) {
    constexpr int NT = NW * 32;
    constexpr int TILE = 32 * ILP;  // particles per i tile
    static_assert(ILP <= 4, "the i slots of a lane are selected with unrolled compares");
    float4 *s_x4 = reinterpret_cast<float4 *>(smem_raw);  // [TC] xh of 4 j
    float4 *s_y4 = s_x4 + TC;                              // [TC] yh
    float4 *s_b4 = s_y4 + TC;                              // [TC] xh^2 + yh^2
    float4 *s_pb = s_b4 + TC;                              // [4*TC] (xl, yl, q, j)
    float4 *s_cold = s_pb + 4 * TC;                        // [ILP][32]
    float4 *s_acc = s_cold + ILP * 32;                     // [NW][ILP][32]
    float4 *s_red = s_acc + NW * ILP * 32;                                 // [TILE]
    int *s_glist = reinterpret_cast<int *>(s_red + TILE);                  // [NT] surviving groups
    int *s_wcount = s_glist + NT;                                          // [NW]

    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int n = P.c.n;
    const int b = (P.mode == kModeForceOnly) ? P.fo_buf : (P.stage - 1) & 1;
    const float4 *__restrict__ pa = P.c.pa[b];
    const float4 *__restrict__ pb = P.c.pb[b];
    float4 *my_acc = s_acc + warp * ILP * 32;

    // every warp owns the same TILE particles: lane l, slot k -> i = tile*TILE + k*32 + l.
    // i side duplicated into both halves of a packed pair: the packed FMAs
    // evaluate two consecutive j against one i
    float2 mx2[ILP], my2[ILP], nu2[ILP];
#pragma unroll
    for (int k = 0; k < ILP; k++) {
        const int i = tile * TILE + k * 32 + lane;
        float ax = 0.0f, ay = 0.0f, nu = INFINITY;
        float4 cold = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
        if (i < n) {
            const float4 A = pa[i];
            const float4 B = pb[i];
            ax = A.x;
            ay = A.y;
            nu = B.z;
            cold = make_float4(B.x, B.y, B.w, __int_as_float(i));
        }
        mx2[k] = make_float2(-2.0f * ax, -2.0f * ax);
        my2[k] = make_float2(-2.0f * ay, -2.0f * ay);
        nu2[k] = make_float2(nu, nu);
        if (warp == 0) s_cold[k * 32 + lane] = cold;
        my_acc[k * 32 + lane] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }

    // Filter hits are recorded per lane: bit 4*g + u of hits[k] is the pair
    // (slot k's i, j = 4*(cbase + g*NW) + u of the staged tile), for the
    // last (up to 8) chunks this warp swept.  The flush runs the precise
    // path on every lane's own hits, slot by slot (the slot is a runtime
    // value, so the precise path exists once in the kernel's code).
    uint32_t hits[ILP];
#pragma unroll
    for (int k = 0; k < ILP; k++) hits[k] = 0u;
    const float *s_xf = reinterpret_cast<const float *>(s_x4);
    const float *s_yf = reinterpret_cast<const float *>(s_y4);
    auto flush_hits = [&](int cbase) {
#pragma unroll 1
        for (int k = 0; k < ILP; k++) {
            uint32_t m = hits[0];
            float xh = -0.5f * mx2[0].x, yh = -0.5f * my2[0].x;
#pragma unroll
            for (int t = 1; t < ILP; t++) {
                m = (k == t) ? hits[t] : m;
                xh = (k == t) ? -0.5f * mx2[t].x : xh;
                yh = (k == t) ? -0.5f * my2[t].x : yh;
            }
            if (!__any_sync(0xffffffffu, m != 0u)) continue;
            const float4 c4 = s_cold[k * 32 + lane];
            PairCtx ic;
            ic.xl = c4.x;
            ic.yl = c4.y;
            ic.qc = c4.z;
            ic.ii = __float_as_int(c4.w);
            float4 acc = my_acc[k * 32 + lane];
            const int jbase = 4 * cbase;  // j of bit 0
            // up to 4 pair terms are summed plainly, each group then added to
            // the compensated sums (the group's rounding is that of one pair term)
            while (m) {
                float px = 0.0f, py = 0.0f;
#pragma unroll 1
                for (int g = 0; g < 4 && m; g++) {
                    const int e = __ffs(m) - 1;
                    m &= m - 1u;
                    const int jj = jbase + (e >> 2) * (4 * NW) + (e & 3);  // index into the tile's j
                    const float4 Bj = s_pb[jj];
                    precise_pair(P, b, xh, yh, ic, make_float4(s_xf[jj], s_yf[jj], 0.0f, Bj.z), Bj,
                                 __float_as_int(Bj.w), px, py);
                }
                kahan_add(acc.x, acc.z, px);
                kahan_add(acc.y, acc.w, py);
            }
            my_acc[k * 32 + lane] = acc;
        }
#pragma unroll
        for (int k = 0; k < ILP; k++) hits[k] = 0u;
    };

    // Chunk c of the staged tile against the i slots in `full` (bit k: slot
    // k), every lane evaluating the same 4 j; pair terms summed plainly and
    // added to the slot's compensated sums.  The slot is a runtime value, so
    // the precise path appears once here, as in flush_hits.
    auto direct_chunk = [&](int c, uint32_t full) {
#pragma unroll 1
        for (int k = 0; k < ILP; k++) {
            if (!((full >> k) & 1u)) continue;
            float xh = -0.5f * mx2[0].x, yh = -0.5f * my2[0].x;
#pragma unroll
            for (int t = 1; t < ILP; t++) {
                xh = (k == t) ? -0.5f * mx2[t].x : xh;
                yh = (k == t) ? -0.5f * my2[t].x : yh;
            }
            const float4 c4 = s_cold[k * 32 + lane];
            PairCtx ic;
            ic.xl = c4.x;
            ic.yl = c4.y;
            ic.qc = c4.z;
            ic.ii = __float_as_int(c4.w);
            float px = 0.0f, py = 0.0f;
#pragma unroll 1
            for (int u = 0; u < 4; u++) {
                const int jj = 4 * c + u;
                const float4 Bj = s_pb[jj];
                precise_pair(P, b, xh, yh, ic, make_float4(s_xf[jj], s_yf[jj], 0.0f, Bj.z), Bj,
                             __float_as_int(Bj.w), px, py);
            }
            float4 acc = my_acc[k * 32 + lane];
            kahan_add(acc.x, acc.z, px);
            kahan_add(acc.y, acc.w, py);
            my_acc[k * 32 + lane] = acc;
        }
    };

    // Sweeps the `count` chunks (4 consecutive j) of this CTA's list through
    // shared-memory tiles; chunk_of(q) is the cloud chunk index of entry q.
    // Within a tile, chunk c goes to warp c % NW.
    auto sweep = [&](int count, auto chunk_of, auto dense_tag) {
    constexpr bool DENSE = decltype(dense_tag)::value;
    for (int q0 = 0; q0 < count; q0 += TC) {
        const int tcn = min(TC, count - q0);
        __syncthreads();
        for (int e = tid; e < tcn; e += NT) {
            const int jb = 4 * chunk_of(q0 + e);  // first j of the chunk
            float xs[4], ys[4], bs[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                if (jb + u < n) {
                    const float4 A = pa[jb + u];
                    const float4 B = pb[jb + u];
                    xs[u] = A.x;
                    ys[u] = A.y;
                    bs[u] = A.z;
                    s_pb[4 * e + u] = make_float4(B.x, B.y, A.w, __int_as_float(jb + u));
                } else {  // padding: never passes the filter
                    xs[u] = kPadPosition;
                    ys[u] = kPadPosition;
                    bs[u] = INFINITY;
                    s_pb[4 * e + u] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
                }
            }
            s_x4[e] = make_float4(xs[0], xs[1], xs[2], xs[3]);
            s_y4[e] = make_float4(ys[0], ys[1], ys[2], ys[3]);
            s_b4[e] = make_float4(bs[0], bs[1], bs[2], bs[3]);
        }
        __syncthreads();
        if constexpr (DENSE) {
            // every pair of these groups is inside the cutoff: no filter, no
            // queue; each lane evaluates its own i against the chunk's 4 j,
            // with its i data and Kahan sums in registers for the whole tile
            PairCtx ic[ILP];
            float xhk[ILP], yhk[ILP];
            float4 acc[ILP];
#pragma unroll
            for (int k = 0; k < ILP; k++) {
                const float4 c4 = s_cold[k * 32 + lane];
                ic[k].xl = c4.x;
                ic[k].yl = c4.y;
                ic[k].qc = c4.z;
                ic[k].ii = __float_as_int(c4.w);
                xhk[k] = -0.5f * mx2[k].x;
                yhk[k] = -0.5f * my2[k].x;
                acc[k] = my_acc[k * 32 + lane];
            }
            for (int c = warp; c < tcn; c += NW) {
                const float4 X = s_x4[c], Y = s_y4[c];
                const float xs[4] = {X.x, X.y, X.z, X.w};
                const float ys[4] = {Y.x, Y.y, Y.z, Y.w};
#pragma unroll
                for (int k = 0; k < ILP; k++) {
                    float px = 0.0f, py = 0.0f;
#pragma unroll 1
                    for (int u = 0; u < 4; u++)
                        inside_pair(P, xhk[k], yhk[k], ic[k], xs[u], ys[u], s_pb[4 * c + u], px, py);
                    kahan_add(acc[k].x, acc[k].z, px);
                    kahan_add(acc[k].y, acc[k].w, py);
                }
            }
#pragma unroll
            for (int k = 0; k < ILP; k++) my_acc[k * 32 + lane] = acc[k];
        } else {
        // one flush site: the loop runs one step past the tile's last chunk
        int nb = 0, cbase = warp;  // chunks recorded in hits, chunk of bit group 0
        bool any_hit = false;      // warp-uniform
        for (int c = warp;; c += NW) {
            const bool live = c < tcn;  // warp-uniform
            if (live) {
                const float4 X = s_x4[c], Y = s_y4[c], Bq = s_b4[c];
                const float2 X01 = make_float2(X.x, X.y), X23 = make_float2(X.z, X.w);
                const float2 Y01 = make_float2(Y.x, Y.y), Y23 = make_float2(Y.z, Y.w);
                const float2 B01 = make_float2(Bq.x, Bq.y), B23 = make_float2(Bq.z, Bq.w);
                // d = |p_j|^2 - 2 p_i.p_j - threshold_i: pair (i, j) passes iff d < 0
                float2 d01[ILP], d23[ILP];
                uint32_t sgn = 0u;
#pragma unroll
                for (int k = 0; k < ILP; k++) {
                    d01[k] = __ffma2_rn(mx2[k], X01, __ffma2_rn(my2[k], Y01, __fadd2_rn(B01, nu2[k])));
                    d23[k] = __ffma2_rn(mx2[k], X23, __ffma2_rn(my2[k], Y23, __fadd2_rn(B23, nu2[k])));
                    sgn |= __float_as_uint(d01[k].x) | __float_as_uint(d01[k].y) | __float_as_uint(d23[k].x) |
                           __float_as_uint(d23[k].y);
                }
                if (__any_sync(0xffffffffu, (int)sgn < 0)) {
                    // slots where every lane passed all 4 j: evaluate the chunk
                    // now, all lanes on the same j (no hit bits, no per-lane
                    // j lookup); the other slots record this lane's hits, the
                    // sign bits of the 4 j
                    uint32_t full = 0u;
#pragma unroll
                    for (int k = 0; k < ILP; k++) {
                        const uint32_t all4 = __float_as_uint(d01[k].x) & __float_as_uint(d01[k].y) &
                                              __float_as_uint(d23[k].x) & __float_as_uint(d23[k].y);
                        full |= (__all_sync(0xffffffffu, (int)all4 < 0) ? 1u : 0u) << k;
                    }
                    if (full) direct_chunk(c, full);
#pragma unroll
                    for (int k = 0; k < ILP; k++) {
                        const uint32_t bits = (__float_as_uint(d01[k].x) >> 31) |
                                              ((__float_as_uint(d01[k].y) >> 30) & 2u) |
                                              ((__float_as_uint(d23[k].x) >> 29) & 4u) |
                                              ((__float_as_uint(d23[k].y) >> 28) & 8u);
                        hits[k] |= ((full >> k) & 1u) ? 0u : bits << (4 * nb);
                    }
                    any_hit = true;
                }
                nb++;
            }
            if (!live || nb == 8) {  // bits full, or the tile is done: its j are overwritten next
                if (any_hit) flush_hits(cbase);
                any_hit = false;
                nb = 0;
                cbase = c + NW;
                if (!live) break;
            }
        }
        }
    }
    };

    __syncthreads();  // s_cold complete
    if constexpr (!CULL) {
        // chunks dealt round-robin: chunk c belongs to rank c % S, so every
        // rank (and every warp) samples the whole cloud evenly
        const int nch_all = (n + 3) >> 2;
        const int my_nch = (nch_all - rank + S - 1) / S;  // chunks of this rank
        sweep(my_nch, [&](int q) { return q * S + rank; }, std::false_type{});
    } else {
        // 32-particle groups dealt round-robin to ranks; a group whose box is
        // beyond the cutoff from the tile's box is skipped whole (it holds no
        // pair the reference counts).  The survivors keep their order.
        const float4 *__restrict__ gb = P.c.gbox[b];
        const int ngroups = (n + 31) >> 5;
        float4 tb = gb[tile * ILP];
#pragma unroll
        for (int k = 1; k < ILP; k++) {
            if (tile * ILP + k < ngroups) {  // a cloud's last tile may hold fewer groups
                const float4 v = gb[tile * ILP + k];
                tb = make_float4(fminf(tb.x, v.x), fminf(tb.y, v.y), fmaxf(tb.z, v.z), fmaxf(tb.w, v.w));
            }
        }
        const int my_ng = (ngroups - rank + S - 1) / S;
        unsigned long long swept = 0ull;
        int *s_glist2 = s_wcount + NW;  // [NT] groups entirely inside the cutoff
        int *s_wcount2 = s_glist2 + NT;  // [NW]
        for (int t0 = 0; t0 < my_ng; t0 += NT) {
            const int t = t0 + tid;
            const int g = t * S + rank;
            bool near = false, inside = false;
            if (t < my_ng) {
                const float4 gbox = gb[g];
                near = boxes_near(tb, gbox, P.rc2_hi);
                // the tile's own groups hold the pairs j == i: filtered path
                inside = near && g / ILP != tile && boxes_inside(tb, gbox, P.rc2_lo);
            }
            const uint32_t bal = __ballot_sync(0xffffffffu, near && !inside);
            const uint32_t bal2 = __ballot_sync(0xffffffffu, inside);
            if (lane == 0) {
                s_wcount[warp] = __popc(bal);
                s_wcount2[warp] = __popc(bal2);
            }
            __syncthreads();
            int off = 0, total = 0, off2 = 0, total2 = 0;
#pragma unroll
            for (int w = 0; w < NW; w++) {
                const int cw = s_wcount[w], cw2 = s_wcount2[w];
                off += (w < warp) ? cw : 0;
                off2 += (w < warp) ? cw2 : 0;
                total += cw;
                total2 += cw2;
            }
            const uint32_t below = (1u << lane) - 1u;
            if (near && !inside) s_glist[off + __popc(bal & below)] = g;
            if (inside) s_glist2[off2 + __popc(bal2 & below)] = g;
            sweep(8 * total, [&](int q) { return 8 * s_glist[q >> 3] + (q & 7); }, std::false_type{});
            sweep(8 * total2, [&](int q) { return 8 * s_glist2[q >> 3] + (q & 7); }, std::true_type{});
            swept += (unsigned long long)(total + total2);
            __syncthreads();  // the lists and counts are reused by the next batch
        }
        if (tid == 0 && swept) atomicAdd(P.c.eval_pairs, swept * 32ull * (unsigned long long)TILE);
    }

    // combine the NW warps in fixed order with a compensated FP32 sum (each
    // warp's Kahan pair (s, c) stands for s - c); FP64 comes later, once per
    // particle (FP64 runs at 1/64 of the FP32 rate here)
    __syncthreads();
    for (int e = tid; e < TILE; e += NT) {
        float sx = 0.0f, cx = 0.0f, sy = 0.0f, cy = 0.0f;
#pragma unroll
        for (int w = 0; w < NW; w++) {
            const float4 v = s_acc[w * ILP * 32 + e];
            kahan_add(sx, cx, v.x);
            kahan_add(sx, cx, -v.z);
            kahan_add(sy, cy, v.y);
            kahan_add(sy, cy, -v.w);
        }
        s_red[e] = make_float4(sx, sy, cx, cy);
    }
    __syncthreads();
}

// CL = true: the S ranks of a tile form a thread-block cluster, combine
// through distributed shared memory and run the stage epilogue in the same
// launch.  CL = false: plain blocks; each writes its partial sums to global
// memory and stage_finish (below) completes the stage.
// Occupancy: with two i slots per lane the kernel fits 64 registers without
// spills, so 32 warps per SM are resident (more latency hidden in the sparse
// phases, where a block is short and bound by dependent loads and barriers);
// four slots need more registers and stay at 24 warps.
template <int NW, int ILP>
constexpr int fp32c_min_blocks() {
    return (ILP <= 2 ? 32 : 24) / NW > 0 ? (ILP <= 2 ? 32 : 24) / NW : 1;
}

template <int NW, int ILP, int TC, bool CL, bool CULL = false>
__global__ void __launch_bounds__(NW * 32, fp32c_min_blocks<NW, ILP>())
    pair_stage_fp32c(const StageParams P, const ExpConsts E) {
    pdl_wait();
    constexpr int TILE = 32 * ILP;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int S = CL ? (int)cg::this_cluster().num_blocks() : P.split;
    const int rank = CL ? (int)cg::this_cluster().block_rank() : (int)(blockIdx.x % P.split);
    const int tile = blockIdx.x / S;
    const int tid = threadIdx.x;
    const int n = P.c.n, n_pad = P.c.n_pad;
    fp32c_sweep<NW, ILP, TC, CULL>(P, E, tile, rank, S, smem_raw);
    float4 *s_red = reinterpret_cast<float4 *>(smem_raw) + Fp32cSmem<NW, ILP, TC>::red_offset;
    if constexpr (!CL) {
        for (int e = tid; e < TILE; e += NW * 32)
            if (tile * TILE + e < n) P.partial[(size_t)rank * n_pad + tile * TILE + e] = s_red[e];
    } else {
        // finalise particles [rank*fchunk, (rank+1)*fchunk) of the tile in
        // whole warps: an FP64 warp instruction costs the same with 1 or 32
        // active lanes, so the FP64 epilogue runs on as few warps as possible
        cg::cluster_group cl = cg::this_cluster();
        const int fchunk = max(32, (TILE + S - 1) / S);
        cl.sync();
        if (tid < fchunk) {
            const int e = rank * fchunk + tid;
            if (e < TILE && tile * TILE + e < n) {
                const int i = tile * TILE + e;
                double fx = 0.0, fy = 0.0;
                for (int r = 0; r < S; r++) {
                    const float4 v = *cl.map_shared_rank(s_red + e, r);
                    fx += (double)v.x - (double)v.z;
                    fy += (double)v.y - (double)v.w;
                }
                stage_epilogue(P, i, fx, fy, stage_thermal(P, i));
            }
        }
        stage_step_advance(P);
        cl.sync();
    }
}

// Completes a stage after a non-cluster pair launch: per particle, the
// split partial sums in rank order (FP64), then the stage epilogue.  One
// particle per thread: the FP64 work runs in full warps on every SM.
static __global__ void __launch_bounds__(64) stage_finish(const StageParams P) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P.c.n) {
        // One warp per 32 particles is little parallelism for the chain of
        // dependent loads below (the split partials, then the epilogue's
        // state): the epilogue's operands are prefetched into L1 first, so
        // their round trip overlaps the partials'.
        {
            const CloudDev &c = P.c;
            const int b = (P.mode == kModeForceOnly) ? P.fo_buf : (P.stage - 1) & 1;
            const bool first = P.mode == kModeForceOnly || P.stage == 1;
            prefetch_l1(c.px[b] + i);
            prefetch_l1(c.py[b] + i);
            prefetch_l1((first ? c.vx : c.vxc) + i);
            prefetch_l1((first ? c.vy : c.vyc) + i);
            prefetch_l1(c.q + i);
            prefetch_l1(c.m + i);
            prefetch_l1(c.orig + i);
            if (P.mode != kModeForceOnly) {
                prefetch_l1(c.x + i);
                prefetch_l1(c.y + i);
                if (!first) {
                    prefetch_l1(c.vx + i);
                    prefetch_l1(c.vy + i);
                }
                if (P.stage >= 3)
                    for (int k = 0; k < 4; k++) prefetch_l1(c.a23[k] + i);
                if (P.stage == 4)
                    for (int k = 0; k < 4; k++) prefetch_l1(c.a1[k] + i);
            }
        }
        // each partial (s, c) stands for s - c; the s are summed exactly as
        // an unevaluated float pair (TwoSum), the small c plainly, in rank
        // order, and FP64 is used once: FP64 runs at ~1/64 of the FP32 rate
        // here and an FP64 sum over the ranks dominated this kernel
        TwoFloatSum sx, sy;
        float cx = 0.0f, cy = 0.0f;
        const float4 *p = P.partial + i;
        const size_t stride = (size_t)P.c.n_pad;
        int r = 0;
        for (; r + 16 <= P.split; r += 16) {  // 16 loads in flight, summed in rank order
            float4 v[16];
#pragma unroll
            for (int u = 0; u < 16; u++) v[u] = p[(size_t)(r + u) * stride];
#pragma unroll
            for (int u = 0; u < 16; u++) {
                sx.add(v[u].x);
                sy.add(v[u].y);
                cx += v[u].z;
                cy += v[u].w;
            }
        }
        for (; r + 8 <= P.split; r += 8) {  // 8 loads in flight, summed in rank order
            float4 v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) v[u] = p[(size_t)(r + u) * stride];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                sx.add(v[u].x);
                sy.add(v[u].y);
                cx += v[u].z;
                cy += v[u].w;
            }
        }
        for (; r < P.split; r++) {
            const float4 v = p[(size_t)r * stride];
            sx.add(v.x);
            sy.add(v.y);
            cx += v.z;
            cy += v.w;
        }
        const double fx = (double)sx.hi + ((double)sx.lo - (double)cx);
        const double fy = (double)sy.hi + ((double)sy.lo - (double)cy);
        stage_epilogue(P, i, fx, fy, stage_thermal(P, i));
    }
    if (P.box_out) {  // a warp is one 32-particle group: its box in the buffer just written
        const int bw = P.stage & 1;
        float x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
        if (i < P.c.n) {
            const float4 A = P.c.pa[bw][i];
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
        if ((threadIdx.x & 31) == 0 && i < P.c.n_pad) P.c.gbox[bw][i >> 5] = make_float4(x0, y0, x1, y1);
    }
    stage_step_advance(P);
}

// ---------------------------------------------------------------------------
// Plain FP64 kernel: same decomposition (G j-groups x NI i-lanes, cluster
// j split, one uniform branch per j), every operation in FP64.
// ---------------------------------------------------------------------------
struct alignas(32) JD {
    double x, y, b, q;
};

template <int NI, int G, int ILP>
struct Fp64Smem {
    static constexpr size_t part = (size_t)G * ILP * NI * sizeof(double2);
    static constexpr size_t red = (size_t)ILP * NI * sizeof(double2);
    static size_t bytes(int jt) { return (size_t)jt * sizeof(JD) + part + red; }
};

template <int NI, int G, int ILP, int JT>
__global__ void __launch_bounds__(NI * G, 2) pair_stage_fp64(const StageParams P) {
    pdl_wait();
    constexpr int NT = NI * G;
    static_assert(NI % 32 == 0 && JT % G == 0, "shape");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    JD *s_j = reinterpret_cast<JD *>(smem_raw);
    double2 *s_part = reinterpret_cast<double2 *>(s_j + JT);  // [G][ILP][NI]
    double2 *s_red = s_part + G * ILP * NI;                     // [ILP*NI]

    cg::cluster_group cl = cg::this_cluster();
    const int S = (int)cl.num_blocks();
    const int rank = (int)cl.block_rank();
    const int tile = blockIdx.x / S;
    const int tid = threadIdx.x;
    const int t = tid % NI, g = tid / NI;
    const int n = P.c.n, n_pad = P.c.n_pad;
    const int b = (P.mode == kModeForceOnly) ? P.fo_buf : (P.stage - 1) & 1;
    const double *__restrict__ px = P.c.px[b];
    const double *__restrict__ py = P.c.py[b];
    const double *__restrict__ qa = P.c.q;
    const double kappa = P.f.shielding;
    const double C = P.coulomb;
    const double rc = sqrt(P.rc2);

    double xi[ILP], yi[ILP], qi[ILP], U[ILP], fx[ILP], fy[ILP];
    int ii[ILP];
#pragma unroll
    for (int k = 0; k < ILP; k++) {
        const int i = tile * NI * ILP + k * NI + t;
        ii[k] = i;
        fx[k] = fy[k] = 0.0;
        if (i < n) {
            xi[k] = px[i];
            yi[k] = py[i];
            qi[k] = qa[i];
            const double a2 = __dadd_rn(__dmul_rn(xi[k], xi[k]), __dmul_rn(yi[k], yi[k]));
            const double pr = sqrt(a2) + rc;
            U[k] = (P.rc2 - a2) + 5.684341886080802e-14 * pr * pr;
        } else {
            xi[k] = yi[k] = qi[k] = 0.0;
            U[k] = -INFINITY;
        }
    }

    const int per = ((n_pad + S - 1) / S + 63) & ~63;
    const int j0 = rank * per;
    const int j1 = min(n_pad, j0 + per);
    constexpr int SUB = JT / G;

    for (int jt = j0; jt < j1; jt += JT) {
        const int cnt = min(JT, j1 - jt);
        __syncthreads();
        for (int e = tid; e < cnt; e += NT) {
            const double xj = px[jt + e], yj = py[jt + e];
            JD d;
            d.x = xj;
            d.y = yj;
            d.b = __dadd_rn(__dmul_rn(xj, xj), __dmul_rn(yj, yj));
            d.q = qa[jt + e];
            s_j[e] = d;
        }
        __syncthreads();
        const int lo = g * SUB;
        const int hi = min(cnt, lo + SUB);
#pragma unroll 2
        for (int jj = lo; jj < hi; jj++) {
            const JD d = s_j[jj];
            double r2e[ILP];
            bool hit = false;
#pragma unroll
            for (int k = 0; k < ILP; k++) {
                r2e[k] = fma(-2.0 * xi[k], d.x, fma(-2.0 * yi[k], d.y, d.b));
                hit |= r2e[k] < U[k];
            }
            if (__any_sync(0xffffffffu, hit)) {
                const int jg = jt + jj;
#pragma unroll
                for (int k = 0; k < ILP; k++) {
                    if (r2e[k] < U[k] && jg != ii[k]) {
                        const double dx = __dsub_rn(xi[k], d.x);
                        const double dy = __dsub_rn(yi[k], d.y);
                        double r, a;
                        if (ref_in_cutoff(dx, dy, kappa, r, a)) {
                            // C*qq*(1+a)*exp(-a)/((r*r)*r) in the reference's
                            // block order (ShieldedCoulombForce.cpp:183-184)
                            const double f = __ddiv_rn(
                                __dmul_rn(__dmul_rn(__dmul_rn(C, __dmul_rn(qi[k], d.q)),
                                                    __dadd_rn(1.0, a)),
                                          exp(-a)),
                                __dmul_rn(__dmul_rn(r, r), r));
                            fx[k] = __dadd_rn(fx[k], __dmul_rn(f, dx));
                            fy[k] = __dadd_rn(fy[k], __dmul_rn(f, dy));
                        }
                    }
                }
            }
        }
    }

#pragma unroll
    for (int k = 0; k < ILP; k++) s_part[(g * ILP + k) * NI + t] = make_double2(fx[k], fy[k]);
    __syncthreads();
    for (int e = tid; e < ILP * NI; e += NT) {
        double sx = 0.0, sy = 0.0;
#pragma unroll
        for (int gg = 0; gg < G; gg++) {
            const double2 v = s_part[gg * ILP * NI + e];
            sx = __dadd_rn(sx, v.x);
            sy = __dadd_rn(sy, v.y);
        }
        s_red[e] = make_double2(sx, sy);
    }
    cl.sync();
    for (int e = rank * NT + tid; e < NI * ILP; e += NT * S) {
        const int i = tile * NI * ILP + e;
        if (i < n) {
            double sxx = 0.0, syy = 0.0;
            for (int r = 0; r < S; r++) {
                const double2 v = *cl.map_shared_rank(s_red + e, r);
                sxx = __dadd_rn(sxx, v.x);
                syy = __dadd_rn(syy, v.y);
            }
            stage_epilogue(P, i, sxx, syy, stage_thermal(P, i));
        }
    }
    stage_step_advance(P);
    cl.sync();
}

}  // namespace dm
