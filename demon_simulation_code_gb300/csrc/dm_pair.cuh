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
// ---------------------------------------------------------------------------
template <int NT, int ILP, int JT>
__global__ void __launch_bounds__(NT) pair_stage_fp32c(const StageParams P, const ExpConsts E) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float4 *s_pa = reinterpret_cast<float4 *>(smem_raw);
    float4 *s_pb = s_pa + JT;
    float4 *s_red = s_pb + JT;  // [ILP][NT] (sx, sy, cx, cy)

    cg::cluster_group cl = cg::this_cluster();
    const int S = (int)cl.num_blocks();
    const int rank = (int)cl.block_rank();
    const int tile = blockIdx.x / S;
    const int tid = threadIdx.x;
    const int n = P.c.n, n_pad = P.c.n_pad;
    const int st = (P.mode == kModeForceOnly) ? 1 : P.stage;
    const int b = (st - 1) & 1;
    const float4 *__restrict__ pa = P.c.pa[b];
    const float4 *__restrict__ pb = P.c.pb[b];
    const double rc = sqrt(P.rc2);

    float m2x[ILP], m2y[ILP], U[ILP], xl[ILP], yl[ILP], qc[ILP];
    float sx[ILP], sy[ILP], cx[ILP], cy[ILP];
    int ii[ILP];
#pragma unroll
    for (int k = 0; k < ILP; k++) {
        const int i = tile * NT * ILP + k * NT + tid;
        ii[k] = i;
        sx[k] = sy[k] = cx[k] = cy[k] = 0.0f;
        if (i < n) {
            const float4 A = pa[i];
            const float4 B = pb[i];
            m2x[k] = -2.0f * A.x;
            m2y[k] = -2.0f * A.y;
            xl[k] = B.x;
            yl[k] = B.y;
            qc[k] = __double2float_rn(P.coulomb * P.c.q[i]);
            // filter threshold: (rc^2 - |p_i|^2) + margin, margin covering the
            // FP32 rounding of the expanded form and of the hi/lo split
            const double ax = A.x, ay = A.y;
            const double a2 = ax * ax + ay * ay;
            const double pr = sqrt(a2) + rc;
            U[k] = __double2float_ru(P.rc2 - a2 + 3.814697265625e-6 * pr * pr);
        } else {
            m2x[k] = m2y[k] = xl[k] = yl[k] = qc[k] = 0.0f;
            U[k] = -INFINITY;
        }
    }

    const int per = ((n_pad + S - 1) / S + 63) & ~63;
    const int j0 = rank * per;
    const int j1 = min(n_pad, j0 + per);
    const float kap = P.kappa_f;
    const float rc2_lo = P.rc2_lo, rc2_hi = P.rc2_hi;

    for (int jt = j0; jt < j1; jt += JT) {
        const int cnt = min(JT, j1 - jt);
        __syncthreads();
        for (int e = tid; e < cnt; e += NT) {
            s_pa[e] = pa[jt + e];
            s_pb[e] = pb[jt + e];
        }
        __syncthreads();
#pragma unroll 2
        for (int jj = 0; jj < cnt; jj++) {
            const float4 A = s_pa[jj];
#pragma unroll
            for (int k = 0; k < ILP; k++) {
                const float r2e = fmaf(m2x[k], A.x, fmaf(m2y[k], A.y, A.z));
                if (r2e < U[k]) {
                    const int jg = jt + jj;
                    if (jg != ii[k]) {
                        const float4 Bj = s_pb[jj];
                        const float dx = (-0.5f * m2x[k] - A.x) + (xl[k] - Bj.x);
                        const float dy = (-0.5f * m2y[k] - A.y) + (yl[k] - Bj.y);
                        const float r2 = fmaf(dx, dx, dy * dy);
                        bool in = r2 < rc2_hi;
                        if (in && !(r2 < rc2_lo)) {
                            // borderline: decide exactly as the reference does
                            double r, a;
                            in = ref_in_cutoff(P.c.px[b][ii[k]] - P.c.px[b][jg],
                                               P.c.py[b][ii[k]] - P.c.py[b][jg],
                                               P.f.shielding, r, a);
                        }
                        if (in) {
                            // 1/r: hardware rsqrt + one Newton step
                            float y = rsqrtf(r2);
                            const float h = r2 * y;
                            const float ee = fmaf(-h, y, 1.0f);
                            y = fmaf(0.5f * ee, y, y);
                            const float r = r2 * y;
                            const float kr = kap * r;
                            const float ex = exp_neg(kr, E);
                            // C q_i q_j (1 + kr) e^{-kr} / r^3
                            const float s = ((qc[k] * A.w) * (1.0f + kr)) * ex * ((y * y) * y);
                            kahan_add(sx[k], cx[k], s * dx);
                            kahan_add(sy[k], cy[k], s * dy);
                        }
                    }
                }
            }
        }
    }

#pragma unroll
    for (int k = 0; k < ILP; k++) s_red[k * NT + tid] = make_float4(sx[k], sy[k], cx[k], cy[k]);
    cl.sync();
    // finalize 1/S of the tile's particles in this CTA: combine the S partial
    // sums (rank order, FP64) and run the stage epilogue
    for (int e = rank * NT + tid; e < NT * ILP; e += NT * S) {
        const int i = tile * NT * ILP + e;
        if (i < n) {
            double fx = 0.0, fy = 0.0;
            for (int r = 0; r < S; r++) {
                const float4 v = *cl.map_shared_rank(s_red + e, r);
                fx += (double)v.x - (double)v.z;
                fy += (double)v.y - (double)v.w;
            }
            stage_epilogue(P, i, fx, fy);
        }
    }
    stage_step_advance(P);
    cl.sync();
}

// ---------------------------------------------------------------------------
// Plain FP64 kernel (same decomposition, every operation in FP64).
// ---------------------------------------------------------------------------
struct alignas(32) JD {
    double x, y, b, q;
};

template <int NT, int ILP, int JT>
__global__ void __launch_bounds__(NT) pair_stage_fp64(const StageParams P) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    JD *s_j = reinterpret_cast<JD *>(smem_raw);
    double2 *s_red = reinterpret_cast<double2 *>(s_j + JT);  // [ILP][NT]

    cg::cluster_group cl = cg::this_cluster();
    const int S = (int)cl.num_blocks();
    const int rank = (int)cl.block_rank();
    const int tile = blockIdx.x / S;
    const int tid = threadIdx.x;
    const int n = P.c.n, n_pad = P.c.n_pad;
    const int st = (P.mode == kModeForceOnly) ? 1 : P.stage;
    const int b = (st - 1) & 1;
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
        const int i = tile * NT * ILP + k * NT + tid;
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
#pragma unroll 2
        for (int jj = 0; jj < cnt; jj++) {
            const JD d = s_j[jj];
#pragma unroll
            for (int k = 0; k < ILP; k++) {
                const double r2e = fma(-2.0 * xi[k], d.x, fma(-2.0 * yi[k], d.y, d.b));
                if (r2e < U[k]) {
                    const int jg = jt + jj;
                    if (jg != ii[k]) {
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
    for (int k = 0; k < ILP; k++) s_red[k * NT + tid] = make_double2(fx[k], fy[k]);
    cl.sync();
    for (int e = rank * NT + tid; e < NT * ILP; e += NT * S) {
        const int i = tile * NT * ILP + e;
        if (i < n) {
            double sxx = 0.0, syy = 0.0;
            for (int r = 0; r < S; r++) {
                const double2 v = *cl.map_shared_rank(s_red + e, r);
                sxx = __dadd_rn(sxx, v.x);
                syy = __dadd_rn(syy, v.y);
            }
            stage_epilogue(P, i, sxx, syy);
        }
    }
    stage_step_advance(P);
    cl.sync();
}

}  // namespace dm
