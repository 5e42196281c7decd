// dm_pair.cuh -- tiled all-pairs shielded-Coulomb (Yukawa) kernels with the
// RK4 stage epilogue fused in, for sm_103a.
//
// Replaces ShieldedCoulombForce::force1..4 (ShieldedCoulombForce.cpp:37-237)
// plus, in the epilogue, the per-particle forces, CacheOperator and the RK4
// stage/combine loops (see dm_device.cuh).
//
// Work decomposition (owner computes, no atomics on forces):
//   * an i-tile of 32*ILP particles belongs to S CTAs (a thread-block
//     cluster, or S plain blocks whose partial sums stage_finish adds); lane
//     l of every warp of those CTAs owns particles i = tile*32*ILP + k*32 + l,
//     k < ILP (the lane's i "slots"), kept in registers;
//   * rank r of the S sweeps every S-th chunk of 4 j (or, culling, every
//     S-th 32-particle j group within reach of the tile), staging them in
//     shared memory; the CTA's warps deal the staged chunks round-robin;
//   * pairs of groups that may hold a pair within the cutoff are first
//     filtered with the expanded distance |p_j|^2 - 2 p_i.p_j against a per-i
//     bound (two j per packed FMA) -- the GPU form of the reference's early
//     exit for kappa*r >= 10 (ShieldedCoulombForce.cpp:178-180); groups
//     entirely within the cutoff skip the filter;
//   * the pair terms are evaluated two j at a time in packed f32x2
//     arithmetic (pair2_terms); the per-particle sums are compensated and the
//     stage epilogue runs once per particle in FP64.
#pragma once

#include <cooperative_groups.h>

#include <type_traits>

#include "dm_device.cuh"

namespace dm {
namespace cg = cooperative_groups;

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

// ---------------------------------------------------------------------------
// Packed f32x2 arithmetic: one instruction evaluates the same operation for
// two j against one i (sm_100+ FADD2/FMUL2/FFMA2), halving the issue slots
// of the pair arithmetic.  Both halves round exactly like the scalar
// operations.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// One i particle, each value duplicated into both halves of a pair: hi and
// lo parts of the two-float position (x = xh + xl).
struct PairI {
    float2 xh, yh, xl, yl;
};

// The geometry of i with two j, the j values negated (nxh = -xh_j, ...):
//   dx = x_i - x_j as (xh_i - xh_j) + (xl_i - xl_j) (the hi difference is
//        exact for nearby particles, so dx keeps ~2^-24 of its own size),
//   r2 = dx^2 + dy^2, y = 1/r, ex = e^{-kappa r}.
// 1/r: hardware rsqrt plus one Newton step, which also gives r = r2 y
// refined; e^{-kappa r} = 2^{-(kappa log2 e) r} on the SFU.
__device__ __forceinline__ void pair2_core(const PairI &I, float2 nxh, float2 nyh, float2 nxl, float2 nyl,
                                           float2 nkl2e, float2 &dx, float2 &dy, float2 &r2, float2 &y,
                                           float2 &ex) {
    dx = add2(add2(I.xh, nxh), add2(I.xl, nxl));
    dy = add2(add2(I.yh, nyh), add2(I.yl, nyl));
    r2 = fma2(dx, dx, mul2(dy, dy));
    const float2 y0 = make_float2(rsqrt_approx(r2.x), rsqrt_approx(r2.y));
    const float2 u = mul2(r2, y0);                                  // r, unrefined
    const float2 h = mul2(fma2(u, y0, dup2(-1.0f)), dup2(-0.5f));  // (1 - r2 y0^2) / 2
    y = fma2(h, y0, y0);                                            // 1/r after one Newton step
    const float2 r = fma2(h, u, u);                                 // r = r2 y, from the same step
    const float2 nt = mul2(r, nkl2e);                               // -(kappa log2 e) r
    ex = make_float2(ex2_approx(nt.x), ex2_approx(nt.y));
}

// Pair terms of i with two j (pair2_core), w = q_j e^{-kappa r} y^2 (y +
// kappa), so that the force on i from j is C q_i w (dx, dy) = C q_i q_j (1 +
// kappa r) e^{-kappa r} / r^3 (dx, dy), the reference's pair force
// (ShieldedCoulombForce.cpp:144-157), C q_i applied once per particle.  A
// pair at r2 = 0 gives non-finite w: callers exclude j == i by a select.
__device__ __forceinline__ void pair2_terms(const PairI &I, float2 nxh, float2 nyh, float2 nxl, float2 nyl,
                                            float2 q, float2 kap, float2 nkl2e, float2 &dx, float2 &dy,
                                            float2 &r2, float2 &w) {
    float2 y, ex;
    pair2_core(I, nxh, nyh, nxl, nyl, nkl2e, dx, dy, r2, y, ex);
    w = mul2(mul2(q, ex), mul2(mul2(y, y), add2(y, kap)));
}

// The scalar form of one pair for the slow path (pairs within 4e-6 of the
// cutoff in r^2, decided exactly as the reference decides): w as in
// pair2_terms, 0 for a pair outside the cutoff.  j values negated.
__device__ __forceinline__ float border_pair(const StageParams &P, int b, const PairI &I, int ii, float nxh,
                                             float nyh, float nxl, float nyl, float q, int jg, float &dx,
                                             float &dy) {
    dx = (I.xh.x + nxh) + (I.xl.x + nxl);
    dy = (I.yh.x + nyh) + (I.yl.x + nyl);
    double r, a;
    if (jg == ii || jg < 0 ||
        !ref_in_cutoff(P.c.px[b][ii] - P.c.px[b][jg], P.c.py[b][ii] - P.c.py[b][jg], P.f.shielding, r, a))
        return 0.0f;
    const float r2 = fmaf(dx, dx, dy * dy);
    float y = rsqrt_approx(r2);
    const float u = r2 * y;
    const float h = -0.5f * fmaf(u, y, -1.0f);
    y = fmaf(h, y, y);
    const float rr = fmaf(h, u, u);
    const float ex = ex2_approx(rr * P.nkl2e);
    return (q * ex) * ((y * y) * (y + P.kappa_f));
}

struct PairTuning {
    int nt, ilp, jt, s;
};

// ---------------------------------------------------------------------------
// FP32-compensated kernel.
//
// A CTA of NW warps shares one i tile of 32*ILP particles (lane l, slot k ->
// i = tile*32*ILP + k*32 + l).  Each staged j chunk (4 j) goes to one warp;
// its pairs are classified:
//   * groups entirely within the cutoff of the tile (box test): evaluated
//     directly, every lane on the same j from shared-memory broadcasts, two
//     j per packed instruction, no filter and no cutoff test;
//   * other groups within reach: the packed filter on all 4 j and every
//     slot, one warp vote per chunk; where it fired, per slot, the number
//     of (lane, j) pairs that passed decides (a warp reduction): at least
//     P.direct_min of the 128 -> the chunk is evaluated directly for that
//     slot with the cutoff taken by a select; fewer -> each lane records its
//     own passing j as hit bits (4 per chunk, 8 chunks per 32-bit word) and
//     later evaluates them two at a time.
// Each lane accumulates only into its own sums (plain f32x2 sums over a few
// chunks, then Kahan), so the result is deterministic and needs no atomics.
// The sums leave out C q_i (applied in FP64 once per particle).
// ---------------------------------------------------------------------------
template <int NW, int ILP, int TC>
struct Fp32cSmem {
    // j tile: TC 4-j chunks, each field of the 4 j in one 16-byte word
    // (-xh, -yh, |p|^2, -xl, -yl, q, j): two consecutive j of a field load
    // straight into the register pair a packed instruction takes
    static constexpr size_t tile = (size_t)TC * 7 * sizeof(float4);
    static constexpr size_t cold = (size_t)ILP * 32 * sizeof(float4);
    static constexpr size_t acc = (size_t)NW * ILP * 32 * sizeof(float4);
    static constexpr size_t red = (size_t)ILP * 32 * sizeof(float4);
    // culling: near, inside and mostly-inside group lists (NT each) and
    // their per-warp counts
    static constexpr size_t glist = 3 * ((size_t)NW * 32 * sizeof(int) + NW * sizeof(int));
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

// The FP32C sweep of one i tile against rank `rank` of S of the j chunks:
// i-side setup, the classified j loop, and the combine of the NW warps'
// Kahan sums into s_red[TILE] = (sx, sy, cx, cy) (force / (C q_i) = s - c).
// Ends with the block synchronised.  `P` may live in shared memory (batched
// kernel).  Particles are those of P.c (n = P.c.n); j at or beyond n read as
// padding, so a cloud needs no padding of its own.
template <int NW, int ILP, int TC, bool CULL = false>
__device__ __forceinline__ void fp32c_sweep(const StageParams &P, int tile, int rank, int S,
                                            unsigned char *smem_raw) {
    constexpr int NT = NW * 32;
    constexpr int TILE = 32 * ILP;  // particles per i tile
    static_assert(ILP <= 4, "the i slots of a lane are selected with unrolled compares");
    float4 *s_x4 = reinterpret_cast<float4 *>(smem_raw);  // [TC] -xh of 4 j
    float4 *s_y4 = s_x4 + TC;                              // [TC] -yh
    float4 *s_b4 = s_y4 + TC;                              // [TC] xh^2 + yh^2
    float4 *s_xl4 = s_b4 + TC;                             // [TC] -xl
    float4 *s_yl4 = s_xl4 + TC;                            // [TC] -yl
    float4 *s_q4 = s_yl4 + TC;                             // [TC] q
    int4 *s_j4 = reinterpret_cast<int4 *>(s_q4 + TC);      // [TC] j (-1: padding)
    float4 *s_cold = reinterpret_cast<float4 *>(s_j4 + TC);  // [ILP][32] (xl, yl, -, i)
    float4 *s_acc = s_cold + ILP * 32;                     // [NW][ILP][32]
    float4 *s_red = s_acc + NW * ILP * 32;                 // [TILE]
    int *s_glist = reinterpret_cast<int *>(s_red + TILE);  // [NT] surviving groups
    int *s_wcount = s_glist + NT;                          // [NW]

    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int n = P.c.n;
    const int b = (P.mode == kModeForceOnly) ? P.fo_buf : (P.stage - 1) & 1;
    const float4 *__restrict__ pa = P.c.pa[b];
    const float4 *__restrict__ pb = P.c.pb[b];
    float4 *my_acc = s_acc + warp * ILP * 32;
    const float2 kap = dup2(P.kappa_f), nkl2e = dup2(P.nkl2e);
    const float rc2_lo = P.rc2_lo, rc2_hi = P.rc2_hi;

    // every warp owns the same TILE particles: lane l, slot k -> i = tile*TILE + k*32 + l.
    // i side duplicated into both halves of a packed pair: the packed FMAs
    // evaluate two consecutive j against one i
    float2 px2[ILP], py2[ILP], nu2[ILP];  // 2 xh_i, 2 yh_i, -(filter bound)
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
            cold = make_float4(B.x, B.y, 0.0f, __int_as_float(i));
        }
        px2[k] = dup2(2.0f * ax);
        py2[k] = dup2(2.0f * ay);
        nu2[k] = dup2(nu);
        if (warp == 0) s_cold[k * 32 + lane] = cold;
        my_acc[k * 32 + lane] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    // i side of slot k (runtime k: the slow paths exist once in the code)
    auto slot_i = [&](int k, int &ii) {
        float xh = 0.5f * px2[0].x, yh = 0.5f * py2[0].x;
#pragma unroll
        for (int t = 1; t < ILP; t++) {
            xh = (k == t) ? 0.5f * px2[t].x : xh;
            yh = (k == t) ? 0.5f * py2[t].x : yh;
        }
        const float4 c4 = s_cold[k * 32 + lane];
        ii = __float_as_int(c4.w);
        return PairI{dup2(xh), dup2(yh), dup2(c4.x), dup2(c4.y)};
    };

    // Filter hits are recorded per lane: bit 4*g + u of hits[k] is the pair
    // (slot k's i, j = 4*(cbase + g*NW) + u of the staged tile), for the
    // last (up to 8) chunks this warp swept.  The flush evaluates every
    // lane's own hits two at a time, slot by slot.
    uint32_t hits[ILP];
#pragma unroll
    for (int k = 0; k < ILP; k++) hits[k] = 0u;
    const float *s_xf = reinterpret_cast<const float *>(s_x4);
    const float *s_yf = reinterpret_cast<const float *>(s_y4);
    const float *s_xlf = reinterpret_cast<const float *>(s_xl4);
    const float *s_ylf = reinterpret_cast<const float *>(s_yl4);
    const float *s_qf = reinterpret_cast<const float *>(s_q4);
    const int *s_jf = reinterpret_cast<const int *>(s_j4);
    auto flush_hits = [&](int cbase) {
#pragma unroll 1
        for (int k = 0; k < ILP; k++) {
            uint32_t m = hits[0];
#pragma unroll
            for (int t = 1; t < ILP; t++) m = (k == t) ? hits[t] : m;
            if (!__any_sync(0xffffffffu, m != 0u)) continue;
            int ii;
            const PairI I = slot_i(k, ii);
            float4 acc = my_acc[k * 32 + lane];
            const int jbase = 4 * cbase;  // j of bit 0
            while (m) {
                // two hits per packed evaluation; a missing second one
                // repeats the first with q = 0 (a finite, zero term)
                const int e0 = __ffs(m) - 1;
                m &= m - 1u;
                const int e1 = m ? __ffs(m) - 1 : e0;
                const float q1 = m ? 1.0f : 0.0f;
                m &= m - 1u;
                const int j0 = jbase + (e0 >> 2) * (4 * NW) + (e0 & 3);  // index into the tile's j
                const int j1 = jbase + (e1 >> 2) * (4 * NW) + (e1 & 3);
                float2 dx, dy, r2, w;
                pair2_terms(I, make_float2(s_xf[j0], s_xf[j1]), make_float2(s_yf[j0], s_yf[j1]),
                            make_float2(s_xlf[j0], s_xlf[j1]), make_float2(s_ylf[j0], s_ylf[j1]),
                            make_float2(s_qf[j0], s_qf[j1] * q1), kap, nkl2e, dx, dy, r2, w);
                const int g0 = s_jf[j0], g1 = s_jf[j1];
                // certainly inside: r2 < rc2_lo; borderline pairs decided exactly
                w.x = (r2.x < rc2_lo && g0 != ii) ? w.x : 0.0f;
                w.y = (r2.y < rc2_lo && g1 != ii && q1 != 0.0f) ? w.y : 0.0f;
                if (!(r2.x < rc2_lo) && r2.x < rc2_hi) {
                    float bx, by;
                    w.x = border_pair(P, b, I, ii, s_xf[j0], s_yf[j0], s_xlf[j0], s_ylf[j0], s_qf[j0], g0, bx, by);
                }
                if (q1 != 0.0f && !(r2.y < rc2_lo) && r2.y < rc2_hi) {
                    float bx, by;
                    w.y = border_pair(P, b, I, ii, s_xf[j1], s_yf[j1], s_xlf[j1], s_ylf[j1], s_qf[j1], g1, bx, by);
                }
                const float2 fx = mul2(w, dx), fy = mul2(w, dy);
                kahan_add(acc.x, acc.z, fx.x + fx.y);
                kahan_add(acc.y, acc.w, fy.x + fy.y);
            }
            my_acc[k * 32 + lane] = acc;
        }
#pragma unroll
        for (int k = 0; k < ILP; k++) hits[k] = 0u;
    };

    // Chunk c of the staged tile against slot k (runtime k), every lane on
    // the same 4 j, the cutoff taken by a select (pairs within 4e-6 of it in
    // r^2 decided exactly, j == i excluded); the chunk's terms summed plainly
    // and added to the slot's compensated sums.
    const int tile_j0 = tile * TILE;  // the tile's own particles: the only chunks that can hold j == i
    auto direct_chunk = [&](int c, int k) {
        int ii;
        const PairI I = slot_i(k, ii);
        const float4 X = s_x4[c], Y = s_y4[c], XL = s_xl4[c], YL = s_yl4[c], Q = s_q4[c];
        float2 dx, dy, r2, w, dx2, dy2, r22, w2;
        pair2_terms(I, make_float2(X.x, X.y), make_float2(Y.x, Y.y), make_float2(XL.x, XL.y),
                    make_float2(YL.x, YL.y), make_float2(Q.x, Q.y), kap, nkl2e, dx, dy, r2, w);
        pair2_terms(I, make_float2(X.z, X.w), make_float2(Y.z, Y.w), make_float2(XL.z, XL.w),
                    make_float2(YL.z, YL.w), make_float2(Q.z, Q.w), kap, nkl2e, dx2, dy2, r22, w2);
        if ((unsigned)(s_jf[4 * c] - tile_j0) < (unsigned)TILE) {  // warp-uniform: this tile's own chunk
            const int4 J = s_j4[c];
            w.x = (r2.x < rc2_lo && J.x != ii) ? w.x : 0.0f;
            w.y = (r2.y < rc2_lo && J.y != ii) ? w.y : 0.0f;
            w2.x = (r22.x < rc2_lo && J.z != ii) ? w2.x : 0.0f;
            w2.y = (r22.y < rc2_lo && J.w != ii) ? w2.y : 0.0f;
        } else {
            w.x = (r2.x < rc2_lo) ? w.x : 0.0f;
            w.y = (r2.y < rc2_lo) ? w.y : 0.0f;
            w2.x = (r22.x < rc2_lo) ? w2.x : 0.0f;
            w2.y = (r22.y < rc2_lo) ? w2.y : 0.0f;
        }
        const bool bd = (!(r2.x < rc2_lo) && r2.x < rc2_hi) || (!(r2.y < rc2_lo) && r2.y < rc2_hi) ||
                        (!(r22.x < rc2_lo) && r22.x < rc2_hi) || (!(r22.y < rc2_lo) && r22.y < rc2_hi);
        float2 fx = fma2(w2, dx2, mul2(w, dx));
        float2 fy = fma2(w2, dy2, mul2(w, dy));
        if (bd) {  // rare: pairs within 4e-6 of the cutoff in r^2
#pragma unroll 1
            for (int u = 0; u < 4; u++) {
                const float rr = (u == 0) ? r2.x : (u == 1) ? r2.y : (u == 2) ? r22.x : r22.y;
                if (rr < rc2_lo || !(rr < rc2_hi)) continue;
                const int jj = 4 * c + u;
                float bx, by;
                const float wb = border_pair(P, b, I, ii, s_xf[jj], s_yf[jj], s_xlf[jj], s_ylf[jj], s_qf[jj],
                                             s_jf[jj], bx, by);
                fx.x = fmaf(wb, bx, fx.x);
                fy.x = fmaf(wb, by, fy.x);
            }
        }
        float4 acc = my_acc[k * 32 + lane];
        kahan_add(acc.x, acc.z, fx.x + fx.y);
        kahan_add(acc.y, acc.w, fy.x + fy.y);
        my_acc[k * 32 + lane] = acc;
    };

    // Sweeps the `count` chunks (4 consecutive j) of this CTA's list through
    // shared-memory tiles; chunk_of(q) is the cloud chunk index of entry q.
    // Within a tile, chunk c goes to warp c % NW.
    // MODE 0: the packed filter, then direct chunks or hit bits; 1: groups
    // entirely inside the cutoff; 2: groups mostly inside it, every chunk
    // evaluated directly with the cutoff taken by a select (no filter)
    auto sweep = [&](int count, auto chunk_of, auto mode_tag) {
    constexpr int MODE = decltype(mode_tag)::value;
    constexpr bool DENSE = MODE == 1;
    for (int q0 = 0; q0 < count; q0 += TC) {
        const int tcn = min(TC, count - q0);
        __syncthreads();
        for (int e = tid; e < tcn; e += NT) {
            const int jb = 4 * chunk_of(q0 + e);  // first j of the chunk
            float xs[4], ys[4], bs[4];
            float *xl = reinterpret_cast<float *>(s_xl4 + e), *yl = reinterpret_cast<float *>(s_yl4 + e);
            float *qs = reinterpret_cast<float *>(s_q4 + e);
            int *js = reinterpret_cast<int *>(s_j4 + e);
#pragma unroll
            for (int u = 0; u < 4; u++) {
                if (jb + u < n) {
                    const float4 A = pa[jb + u];
                    const float4 B = pb[jb + u];
                    xs[u] = -A.x;
                    ys[u] = -A.y;
                    bs[u] = A.z;
                    xl[u] = -B.x;
                    yl[u] = -B.y;
                    qs[u] = A.w;
                    js[u] = jb + u;
                } else {  // padding: never passes the filter; a finite, zero term
                    xs[u] = -kPadPosition;
                    ys[u] = -kPadPosition;
                    bs[u] = INFINITY;
                    xl[u] = yl[u] = qs[u] = 0.0f;
                    js[u] = -1;
                }
            }
            s_x4[e] = make_float4(xs[0], xs[1], xs[2], xs[3]);
            s_y4[e] = make_float4(ys[0], ys[1], ys[2], ys[3]);
            s_b4[e] = make_float4(bs[0], bs[1], bs[2], bs[3]);
        }
        __syncthreads();
        if constexpr (DENSE) {
            // every pair of these groups is inside the cutoff (and j != i):
            // no filter, no select; each lane evaluates its own i against the
            // chunk's 4 j, two per packed instruction, its i data and sums in
            // registers for the whole tile; plain sums over two chunks, then Kahan
            PairI I[ILP];
            float4 acc[ILP];
            float2 fx[ILP], fy[ILP];
#pragma unroll
            for (int k = 0; k < ILP; k++) {
                int ii;
                I[k] = slot_i(k, ii);
                acc[k] = my_acc[k * 32 + lane];
                fx[k] = fy[k] = dup2(0.0f);
            }
            int ng = 0;
            for (int c = warp; c < tcn; c += NW) {
                const float4 X = s_x4[c], Y = s_y4[c], XL = s_xl4[c], YL = s_yl4[c], Q = s_q4[c];
#pragma unroll
                for (int k = 0; k < ILP; k++) {
                    float2 dx, dy, r2, w;
                    pair2_terms(I[k], make_float2(X.x, X.y), make_float2(Y.x, Y.y), make_float2(XL.x, XL.y),
                                make_float2(YL.x, YL.y), make_float2(Q.x, Q.y), kap, nkl2e, dx, dy, r2, w);
                    fx[k] = fma2(w, dx, fx[k]);
                    fy[k] = fma2(w, dy, fy[k]);
                    pair2_terms(I[k], make_float2(X.z, X.w), make_float2(Y.z, Y.w), make_float2(XL.z, XL.w),
                                make_float2(YL.z, YL.w), make_float2(Q.z, Q.w), kap, nkl2e, dx, dy, r2, w);
                    fx[k] = fma2(w, dx, fx[k]);
                    fy[k] = fma2(w, dy, fy[k]);
                }
                if (++ng == 2) {
                    ng = 0;
#pragma unroll
                    for (int k = 0; k < ILP; k++) {
                        kahan_add(acc[k].x, acc[k].z, fx[k].x + fx[k].y);
                        kahan_add(acc[k].y, acc[k].w, fy[k].x + fy[k].y);
                        fx[k] = fy[k] = dup2(0.0f);
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < ILP; k++) {
                kahan_add(acc[k].x, acc[k].z, fx[k].x + fx[k].y);
                kahan_add(acc[k].y, acc[k].w, fy[k].x + fy[k].y);
                my_acc[k * 32 + lane] = acc[k];
            }
        } else if constexpr (MODE == 2) {
            for (int c = warp; c < tcn; c += NW) {
#pragma unroll 1
                for (int k = 0; k < ILP; k++) direct_chunk(c, k);
            }
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
                // d = |p_j|^2 - 2 p_i.p_j - bound_i: pair (i, j) passes iff d < 0
                float2 d01[ILP], d23[ILP];
                uint32_t sgn = 0u;
#pragma unroll
                for (int k = 0; k < ILP; k++) {
                    d01[k] = fma2(px2[k], X01, fma2(py2[k], Y01, add2(B01, nu2[k])));
                    d23[k] = fma2(px2[k], X23, fma2(py2[k], Y23, add2(B23, nu2[k])));
                    sgn |= __float_as_uint(d01[k].x) | __float_as_uint(d01[k].y) | __float_as_uint(d23[k].x) |
                           __float_as_uint(d23[k].y);
                }
                if (__any_sync(0xffffffffu, (int)sgn < 0)) {
                    // per slot: enough passing (lane, j) pairs -> the whole
                    // chunk directly; else this lane's hits as bits
                    uint32_t direct = 0u;
#pragma unroll
                    for (int k = 0; k < ILP; k++) {
                        const uint32_t bits = (__float_as_uint(d01[k].x) >> 31) |
                                              ((__float_as_uint(d01[k].y) >> 30) & 2u) |
                                              ((__float_as_uint(d23[k].x) >> 29) & 4u) |
                                              ((__float_as_uint(d23[k].y) >> 28) & 8u);
                        const bool dir = (int)__reduce_add_sync(0xffffffffu, __popc(bits)) >= P.direct_min;
                        direct |= (dir ? 1u : 0u) << k;
                        hits[k] |= dir ? 0u : bits << (4 * nb);
                    }
#pragma unroll 1
                    for (int k = 0; k < ILP; k++)
                        if ((direct >> k) & 1u) direct_chunk(c, k);
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
        sweep(my_nch, [&](int q) { return q * S + rank; }, std::integral_constant<int, 0>{});
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
        int *s_glist2 = s_wcount + NW;   // [NT] groups entirely inside the cutoff
        int *s_wcount2 = s_glist2 + NT;  // [NW]
        int *s_glist3 = s_wcount2 + NW;  // [NT] groups mostly inside it
        int *s_wcount3 = s_glist3 + NT;  // [NW]
        const float rc2_mostly = P.rc2_lo * P.near_direct_f2;  // 0: no such class
        for (int t0 = 0; t0 < my_ng; t0 += NT) {
            const int t = t0 + tid;
            const int g = t * S + rank;
            bool near = false, inside = false, mostly = false;
            if (t < my_ng) {
                const float4 gbox = gb[g];
                near = boxes_near(tb, gbox, P.rc2_hi);
                // the tile's own groups hold the pairs j == i: not "inside"
                inside = near && g / ILP != tile && boxes_inside(tb, gbox, P.rc2_lo);
                // farthest separation within sqrt(near_direct_f2) r_c: most
                // pairs pass the filter, so it is skipped
                mostly = near && !inside && rc2_mostly > 0.0f && boxes_inside(tb, gbox, rc2_mostly);
            }
            const uint32_t bal = __ballot_sync(0xffffffffu, near && !inside && !mostly);
            const uint32_t bal2 = __ballot_sync(0xffffffffu, inside);
            const uint32_t bal3 = __ballot_sync(0xffffffffu, mostly);
            if (lane == 0) {
                s_wcount[warp] = __popc(bal);
                s_wcount2[warp] = __popc(bal2);
                s_wcount3[warp] = __popc(bal3);
            }
            __syncthreads();
            int off = 0, total = 0, off2 = 0, total2 = 0, off3 = 0, total3 = 0;
#pragma unroll
            for (int w = 0; w < NW; w++) {
                const int cw = s_wcount[w], cw2 = s_wcount2[w], cw3 = s_wcount3[w];
                off += (w < warp) ? cw : 0;
                off2 += (w < warp) ? cw2 : 0;
                off3 += (w < warp) ? cw3 : 0;
                total += cw;
                total2 += cw2;
                total3 += cw3;
            }
            const uint32_t below = (1u << lane) - 1u;
            if (near && !inside && !mostly) s_glist[off + __popc(bal & below)] = g;
            if (inside) s_glist2[off2 + __popc(bal2 & below)] = g;
            if (mostly) s_glist3[off3 + __popc(bal3 & below)] = g;
            sweep(8 * total, [&](int q) { return 8 * s_glist[q >> 3] + (q & 7); }, std::integral_constant<int, 0>{});
            sweep(8 * total2, [&](int q) { return 8 * s_glist2[q >> 3] + (q & 7); },
                  std::integral_constant<int, 1>{});
            sweep(8 * total3, [&](int q) { return 8 * s_glist3[q >> 3] + (q & 7); },
                  std::integral_constant<int, 2>{});
            swept += (unsigned long long)(total + total2 + total3);
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

// C q_i in FP64: the factor the FP32C sweeps leave out of their sums.
__device__ __forceinline__ double pair_scale(const StageParams &P, int i) {
    return __dmul_rn(P.coulomb, P.c.q[i]);
}

// CL = true: the S ranks of a tile form a thread-block cluster, combine
// through distributed shared memory and run the stage epilogue in the same
// launch.  CL = false: plain blocks; each writes its partial sums to global
// memory and stage_finish (below) completes the stage.
// Occupancy: with two i slots per lane the kernel is bounded to 64
// registers, so 32 warps per SM are resident (more latency hidden in the
// sparse phases, where a block is short and bound by dependent loads and
// barriers); four slots need more registers and stay at 24 warps.
template <int NW, int ILP>
constexpr int fp32c_min_blocks() {
    return (ILP <= 2 ? 32 : 24) / NW > 0 ? (ILP <= 2 ? 32 : 24) / NW : 1;
}

template <int NW, int ILP, int TC, bool CL, bool CULL = false>
__global__ void __launch_bounds__(NW * 32, fp32c_min_blocks<NW, ILP>())
    pair_stage_fp32c(const StageParams P) {
    pdl_wait();
    constexpr int TILE = 32 * ILP;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int S = CL ? (int)cg::this_cluster().num_blocks() : P.split;
    const int rank = CL ? (int)cg::this_cluster().block_rank() : (int)(blockIdx.x % P.split);
    const int tile = blockIdx.x / S;
    const int tid = threadIdx.x;
    const int n = P.c.n, n_pad = P.c.n_pad;
    fp32c_sweep<NW, ILP, TC, CULL>(P, tile, rank, S, smem_raw);
    float4 *s_red = reinterpret_cast<float4 *>(smem_raw) + Fp32cSmem<NW, ILP, TC>::red_offset;
    if constexpr (!CL) {
        for (int e = tid; e < TILE; e += NW * 32)
            if (tile * TILE + e < n) {
                const float4 v = s_red[e];
                P.partial[(size_t)(2 * rank) * n_pad + tile * TILE + e] = make_float2(v.x, v.z);
                P.partial[(size_t)(2 * rank + 1) * n_pad + tile * TILE + e] = make_float2(v.y, v.w);
            }
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
                const double cq = pair_scale(P, i);
                stage_epilogue(P, i, __dmul_rn(cq, fx), __dmul_rn(cq, fy), stage_thermal(P, i));
            }
        }
        stage_step_advance(P);
        cl.sync();
    }
}

// Sum over the j split's ranks, in rank order, of one axis's partials
// (s, c) of particle i (each stands for s - c): the s exactly as an
// unevaluated float pair (TwoSum), the small c plainly, FP64 once -- FP64
// runs at ~1/64 of the FP32 rate here and an FP64 sum over the ranks
// dominated the finish.  Times C q_i (left out of the sweeps), in FP64.
__device__ __forceinline__ double finish_rank_sum(const StageParams &P, int i, int axis) {
    TwoFloatSum sa;
    float ca = 0.0f;
    const float2 *p = P.partial + (size_t)axis * P.c.n_pad + i;
    const size_t stride = 2 * (size_t)P.c.n_pad;
    int r = 0;
    for (; r + 16 <= P.split; r += 16) {  // 16 loads in flight, summed in rank order
        float2 v[16];
#pragma unroll
        for (int u = 0; u < 16; u++) v[u] = p[(size_t)(r + u) * stride];
#pragma unroll
        for (int u = 0; u < 16; u++) {
            sa.add(v[u].x);
            ca += v[u].y;
        }
    }
    for (; r + 8 <= P.split; r += 8) {  // 8 loads in flight, summed in rank order
        float2 v[8];
#pragma unroll
        for (int u = 0; u < 8; u++) v[u] = p[(size_t)(r + u) * stride];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            sa.add(v[u].x);
            ca += v[u].y;
        }
    }
    for (; r < P.split; r++) {
        const float2 v = p[(size_t)r * stride];
        sa.add(v.x);
        ca += v.y;
    }
    // the two small corrections combined in FP32 (their rounding is ~2^-24
    // of ~2^-24 of the sum): two FP64 operations fewer per particle and axis
    return __dmul_rn(pair_scale(P, i), (double)sa.hi + (double)(sa.lo - ca));
}

// Completes a stage after a non-cluster pair launch when forces outside
// kBasicForces are on (they couple the axes): one particle per thread, the
// rank sums of both axes, then the stage epilogue.
static __global__ void __launch_bounds__(64) stage_finish(const StageParams P) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P.c.n) {
        const double fx = finish_rank_sum(P, i, 0);
        const double fy = finish_rank_sum(P, i, 1);
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

// The same completion with one thread per particle and axis, for the
// forces in kBasicForces: block = one 32-particle group, warp 0 the x and
// warp 1 the y components.  Each axis runs exactly the operations
// stage_epilogue runs for it, in the same order, so the results are the
// same bits; the finish is a latency-bound chain (rank partials, FP64 at
// GB300's FP64 rate) and this gives it twice the warps.  The two warps
// meet once, in shared memory, for what needs both axes: the next stage's
// packed positions, filter bound and group box.
static __global__ void __launch_bounds__(64) stage_finish_axes(const StageParams P) {
    pdl_wait();
    __shared__ float s_hi[2][32], s_lo[2][32];
    const int lane = threadIdx.x & 31, ax = threadIdx.x >> 5;
    const int i = blockIdx.x * 32 + lane;
    const CloudDev &c = P.c;
    const bool live = i < c.n;
    const bool fo = P.mode == kModeForceOnly;
    const int s = fo ? 1 : P.stage;
    const int b = fo ? P.fo_buf : (s - 1) & 1;
    double na = 0.0;  // this axis's coordinate at the next stage
    if (live) {
        const double *pos = ax ? c.py[b] : c.px[b];
        const double *vel = (s == 1) ? (ax ? c.vy : c.vx) : (ax ? c.vyc : c.vxc);
        double *X = ax ? c.y : c.x;
        double *V = ax ? c.vy : c.vx;
        // the operands' round trip overlaps the partials' (see stage_finish)
        prefetch_l1(pos + i);
        prefetch_l1(vel + i);
        prefetch_l1(c.q + i);
        prefetch_l1(c.m + i);
        prefetch_l1(c.orig + i);
        if (!fo) {
            prefetch_l1(X + i);
            prefetch_l1(V + i);
            if (s >= 3) {
                prefetch_l1(c.a23[2 * ax] + i);
                prefetch_l1(c.a23[2 * ax + 1] + i);
            }
            if (s == 4) {
                prefetch_l1(c.a1[2 * ax] + i);
                prefetch_l1(c.a1[2 * ax + 1] + i);
            }
        }
        const double fpa = finish_rank_sum(P, i, ax);
        const double xs = pos[i], vs = vel[i], q = c.q[i], m = c.m[i];
        const long long fl = P.f.flags;
        double F = 0.0;
        if (fl & kConfinement) F = __dadd_rn(F, __dmul_rn(__dmul_rn(q, P.f.confine), xs));
        if (fl & kDrag) F = __dadd_rn(F, __dmul_rn(__dmul_rn(m, -P.f.gamma), vs));
        if (fl & kRectConfinement)
            F = __dadd_rn(F, __dmul_rn(__dmul_rn(q, ax ? P.f.confine_y : P.f.confine_x), xs));
        if (fl & kShieldedCoulomb) F = __dadd_rn(F, fpa);
        if (fl & kThermal) {
            const double2 t = stage_thermal(P, i);
            F = __dadd_rn(F, ax ? t.y : t.x);
        }
        if (fo) {
            (ax ? P.fy_out : P.fx_out)[c.orig[i]] = F;
        } else {
            const double dt = stage_dt(P);
            const double k = __ddiv_rn(__dmul_rn(dt, F), m);
            const double l = __dmul_rn(dt, vs);
            const double x = X[i], v = V[i];
            const bool last = (s == P.order);
            double nv = 0.0;
            if (last && s == 2) {  // Runge_Kutta2: x += l2, V += k2
                na = __dadd_rn(x, l);
                V[i] = __dadd_rn(v, k);
                X[i] = na;
            } else if (s == 1 || s == 2) {
                double *const *acc = (s == 1) ? c.a1 : c.a23;
                acc[2 * ax][i] = k;
                acc[2 * ax + 1][i] = l;
                na = __dadd_rn(__dmul_rn(0.5, l), x);
                nv = __dadd_rn(__dmul_rn(0.5, k), v);
            } else if (s == 3) {
                c.a23[2 * ax][i] = __dadd_rn(c.a23[2 * ax][i], k);
                c.a23[2 * ax + 1][i] = __dadd_rn(c.a23[2 * ax + 1][i], l);
                na = __dadd_rn(x, l);
                nv = __dadd_rn(v, k);
            } else {
                const double dv =
                    __ddiv_rn(__dadd_rn(c.a1[2 * ax][i], __dadd_rn(__dmul_rn(c.a23[2 * ax][i], 2.0), k)), 6.0);
                const double d =
                    __ddiv_rn(__dadd_rn(c.a1[2 * ax + 1][i], __dadd_rn(__dmul_rn(c.a23[2 * ax + 1][i], 2.0), l)), 6.0);
                na = __dadd_rn(x, d);
                V[i] = __dadd_rn(v, dv);
                X[i] = na;
            }
            (ax ? c.py : c.px)[b ^ 1][i] = na;
            if (!last) (ax ? c.vyc : c.vxc)[i] = nv;
            if (!isfinite(na)) atomicOr(c.err, 1);
        }
    }
    if (fo) return;  // uniform over the launch
    float h = 0.0f, lo = 0.0f;
    if (live) split2(na, h, lo);
    s_hi[ax][lane] = h;
    s_lo[ax][lane] = lo;
    __syncthreads();
    const int bw = b ^ 1;
    const float xh = s_hi[0][lane], yh = s_hi[1][lane];
    if (live) {  // write_stage_position's packed words, one float4 per warp
        const double q = c.q[i];
        if (ax == 0)
            c.pa[bw][i] = make_float4(xh, yh, fmaf(yh, yh, xh * xh), __double2float_rn(q));
        else
            c.pb[bw][i] = make_float4(s_lo[0][lane], s_lo[1][lane], -filter_threshold(xh, yh, c.rc2), 0.0f);
    }
    if (P.box_out && ax == 0) {  // the group's box in the buffer just written
        float x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
        if (live) {
            x0 = x1 = xh;
            y0 = y1 = yh;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
            y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
            x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
            y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
        }
        if (lane == 0 && i < c.n_pad) c.gbox[bw][blockIdx.x] = make_float4(x0, y0, x1, y1);
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
