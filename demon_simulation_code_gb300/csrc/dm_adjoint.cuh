// dm_adjoint.cuh -- forces and their vector-Jacobian product for the
// differentiable rollout, in FP64 or FP32-compensated pair arithmetic.
//
// Clouds are concatenated; cloud c owns particles [off_c, off_c + n_c) and
// its own kappa, confinement and drag.  For particle k with force adjoint
// a_k = dL/dF_k (a 2-vector) the VJP kernel produces
//   g_pos[k] = sum_j [ g (a_k - a_j) + h d (d . (a_k - a_j)) ] + q_k k_c a_k
//              (+ rect confinement (q c_x a_x, q c_y a_y))
//   g_vel[k] = -gamma m_k a_k                                    (drag)
//   g_q[k]   = (1/q_k) sum_j F_kj . (a_k - a_j) + k_c p_k . a_k  (dL/dq_k)
//   g_kap[k] = a_k . sum_j (dg/dkappa) d                          (per particle)
//   g_kc[k]  = q_k p_k . a_k                                       (per particle)
// with d = p_k - p_j, F_kj = g(r) d the pair force and, for kappa*r < 10,
//   g(r) = C q_k q_j (1 + kappa r) e^{-kappa r} / r^3,
//   h(r) = g'(r)/r = -g(r) (kappa^2/(1 + kappa r) + 3/r^2) / 1,   [since
//          d ln g/dr = -kappa^2 r/(1 + kappa r) - 3/r]
//   dg/dkappa = -C q_k q_j kappa e^{-kappa r} / r.
// This uses that dF_i/dp_i = sum_j G_ij, dF_i/dp_j = -G_ij with the symmetric
// G_ij = g I + h d d^T, so sum_i (dF_i/dp_k)^T a_i = sum_j G_kj (a_k - a_j).
// The cutoff is the reference's (ShieldedCoulombForce.cpp:147); the force is
// discontinuous there and its jump is not differentiated (measure zero).
#pragma once

#include "dm_pair.cuh"

namespace dm {

struct AdjCloud {
    int off, n;
    long long flags;
    double kappa, confine, confine_x, confine_y, gamma;
    double rc2;
    float rc2_lo, rc2_hi;  // FP32 certain-in / certain-out bounds on r^2
    float kappa_f, kappa2_f;
    float kl2e_hi, kl2e_lo;  // kappa*log2(e) as a float pair (SFU exponential)
    float nkl2e;             // -kappa*log2(e): e^{-kappa r} = 2^{nkl2e r} (packed pair terms)
};

constexpr int kAdjThreads = 128;
constexpr int kAdjTile = 256;

struct alignas(16) AdjJ {
    double x, y, q, ax, ay;
};

// FP32 candidate test, conservative for the FP64 cutoff decision.  With
// xf = fl32(x) (|xf - x| <= 2^-24 |x|) and dxf = fl32(xf_i - xf_j), the error of
// dxf is at most 2^-24 (|x_i| + |x_j|) + 2^-24 |dxf| <= e = 2^-22 (A_i + A_t),
// where A_i = max(|x_i|, |y_i|) and A_t bounds |x_j|, |y_j| over the j tile; the
// error vector of (dxf, dyf) is shorter than 2e.  So every pair with true
// r < r_c has fl32(dxf^2 + dyf^2) < (r_c + 2e)^2 (1 + 2^-20) -- the last factor
// covers the three FP32 roundings of the square sum and of r_c itself.  The
// exact decision is then the reference's FP64 test (ref_in_cutoff).
__device__ __forceinline__ float adj_candidate_bound(double rc, float ai, float at) {
    const float e = 2.384185791015625e-7f * (ai + at);  // 2^-22
    const float r = __fadd_ru(__double2float_ru(rc), 2.0f * e);
    return __fmul_ru(__fmul_ru(r, r), 1.0000009536743164f);  // 1 + 2^-20
}

// Pair sums of one particle: MODE 0 (sx, sy) = sum_j F_kj; MODE 1 the four
// VJP sums (position x, position y, charge, kappa).
struct AdjSums {
    double v[4];
};

// FP64 pair loop over one shared-memory j tile.
template <int MODE>
__device__ __forceinline__ void adj_tile_fp64(const AdjCloud &d, const AdjJ *sj, const float2 *sf, int cnt,
                                              int jbase, int li, double xi, double yi, double qi, double axi,
                                              double ayi, float xfi, float yfi, float bound, double coulomb,
                                              AdjSums &S) {
    for (int e = 0; e < cnt; e++) {
        const float2 f = sf[e];
        const float dxf = xfi - f.x, dyf = yfi - f.y;
        if (!(fmaf(dxf, dxf, dyf * dyf) < bound)) continue;
        if (jbase + e == li) continue;
        const AdjJ v = sj[e];
        const double dx = __dsub_rn(xi, v.x), dy = __dsub_rn(yi, v.y);
        double r, a;
        if (!ref_in_cutoff(dx, dy, d.kappa, r, a)) continue;
        const double ex = exp(-a);
        const double g = coulomb * qi * v.q * (1.0 + a) * ex / (r * r * r);
        if (MODE == 0) {
            S.v[0] += g * dx;
            S.v[1] += g * dy;
        } else {
            const double h = -g * (d.kappa * d.kappa / (1.0 + a) + 3.0 / (r * r));
            const double bx = axi - v.ax, by = ayi - v.ay;
            const double dd = dx * bx + dy * by;
            S.v[0] += g * bx + h * dx * dd;                             // position adjoint
            S.v[1] += g * by + h * dy * dd;
            S.v[2] += g * dd;                                            // F_kj . (a_k - a_j)
            S.v[3] += (-coulomb * qi * v.q * d.kappa * ex / r) * (axi * dx + ayi * dy);  // dg/dkappa
        }
    }
}

// FP32-compensated pair loop over one shared-memory j tile: positions as
// float pairs (hi, lo) so the differences keep ~2^-24 relative accuracy,
// pair terms in FP32, summed plainly over groups of four j and each group
// added to Kahan sums; pairs within 4e-6 of the cutoff in r^2 are decided by
// the reference's FP64 test on the FP64 positions.  e^{-kappa r} on the SFU
// with the rounding residue of kappa r restored (exp_neg_kr), 1/(1 + kappa r)
// from the fast reciprocal: a few ulp per pair term, far below the rounding
// of the FP32 pair sums themselves.
template <int MODE>
__device__ __forceinline__ void adj_tile_fp32c(const AdjCloud &d, const float4 *sp,
                                               const float4 *sa, int cnt, int jbase, int li, float xh, float yh,
                                               float xl, float yl, float qci, float axi, float ayi,
                                               const double *__restrict__ x, const double *__restrict__ y,
                                               double xi, double yi, float (&s)[4], float (&c)[4]) {
    constexpr int NS = MODE == 0 ? 2 : 4;
    for (int e0 = 0; e0 < cnt; e0 += 4) {
        float t[NS];
#pragma unroll
        for (int k = 0; k < NS; k++) t[k] = 0.0f;
        const int e1 = min(cnt, e0 + 4);
        for (int e = e0; e < e1; e++) {
            const float4 P = sp[e];
            const float dx = (xh - P.x) + (xl - P.z);
            const float dy = (yh - P.y) + (yl - P.w);
            const float r2 = fmaf(dx, dx, dy * dy);
            if (!(r2 < d.rc2_hi)) continue;
            if (jbase + e == li) continue;
            if (!(r2 < d.rc2_lo)) {
                const int j = d.off + jbase + e;
                double r, a;
                if (!ref_in_cutoff(__dsub_rn(xi, x[j]), __dsub_rn(yi, y[j]), d.kappa, r, a)) continue;
            }
            float w = rsqrtf(r2);  // 1/r, one Newton step
            w = fmaf(0.5f * fmaf(-(r2 * w), w, 1.0f), w, w);
            const float r = r2 * w;
            const float kr = d.kappa_f * r;
            const float ex = exp_neg_kr(r, d.kl2e_hi, d.kl2e_lo);
            const float4 A = sa[e];  // (q_j, a_j.x, a_j.y, -)
            const float qq = qci * A.x;
            const float g = (qq * (1.0f + kr)) * ex * ((w * w) * w);
            if constexpr (MODE == 0) {
                t[0] = fmaf(g, dx, t[0]);
                t[1] = fmaf(g, dy, t[1]);
            } else {
                const float h = -g * fmaf(d.kappa2_f, __fdividef(1.0f, 1.0f + kr), 3.0f * (w * w));
                const float bx = axi - A.y, by = ayi - A.z;
                const float dd = fmaf(dx, bx, dy * by);
                const float hd = h * dd;
                t[0] += fmaf(hd, dx, g * bx);
                t[1] += fmaf(hd, dy, g * by);
                t[2] = fmaf(g, dd, t[2]);
                t[NS - 1] = fmaf(-(qq * d.kappa_f) * ex * w, fmaf(axi, dx, ayi * dy), t[NS - 1]);
            }
        }
#pragma unroll
        for (int k = 0; k < NS; k++) kahan_add(s[k], c[k], t[k]);
    }
}

// One thread per particle i, j of the same cloud staged through shared
// memory.  MODE 0: forces (total F and pair-only Fp).  MODE 1: VJP.
// F32C selects the FP32-compensated pair arithmetic.
template <int MODE, bool F32C>
__global__ void __launch_bounds__(kAdjThreads) adjoint_kernel(
    const AdjCloud *__restrict__ desc, const int *__restrict__ cloud_of_block, const int *__restrict__ tile_of_block,
    const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ vx,
    const double *__restrict__ vy, const double *__restrict__ q, const double *__restrict__ m,
    const double *__restrict__ ax, const double *__restrict__ ay,  // MODE 1: force adjoint
    double *__restrict__ o0, double *__restrict__ o1, double *__restrict__ o2, double *__restrict__ o3,
    double *__restrict__ o4, double *__restrict__ o5, double *__restrict__ o6, double coulomb) {
    // FP64: AdjJ[kAdjTile] + float2[kAdjTile]; FP32C: two float4[kAdjTile]
    constexpr int kSmem = F32C ? 2 * 16 * kAdjTile : (int)(sizeof(AdjJ) + 8) * kAdjTile;
    __shared__ __align__(16) unsigned char smem[kSmem];
    __shared__ unsigned int s_amax;
    const AdjCloud d = desc[cloud_of_block[blockIdx.x]];
    const int li = tile_of_block[blockIdx.x] * kAdjThreads + threadIdx.x;  // index within the cloud
    const bool valid = li < d.n;
    const int i = d.off + (valid ? li : 0);
    const double xi = x[i], yi = y[i], qi = q[i];
    const double axi = (MODE == 1 && valid) ? ax[i] : 0.0, ayi = (MODE == 1 && valid) ? ay[i] : 0.0;
    const bool coul = (d.flags & kShieldedCoulomb) != 0;
    AdjSums S{};
    // FP64 path state
    const float xfi = (float)xi, yfi = (float)yi;
    const float ai = fmaxf(fabsf(xfi), fabsf(yfi));
    const double rc = sqrt(d.rc2);
    // FP32C path state
    const float xh = (float)xi, yh = (float)yi;
    const float xl = (float)(xi - (double)xh), yl = (float)(yi - (double)yh);
    const float qci = (float)(coulomb * qi);
    const float axf = (float)axi, ayf = (float)ayi;
    float fs[4] = {0.0f, 0.0f, 0.0f, 0.0f}, fc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int j0 = 0; j0 < d.n && coul; j0 += kAdjTile) {
        const int cnt = min(kAdjTile, d.n - j0);
        __syncthreads();
        if (F32C) {
            float4 *sp = reinterpret_cast<float4 *>(smem);
            float4 *sa = sp + kAdjTile;
            for (int e = threadIdx.x; e < cnt; e += kAdjThreads) {
                const int j = d.off + j0 + e;
                const double xj = x[j], yj = y[j];
                const float hx = (float)xj, hy = (float)yj;
                sp[e] = make_float4(hx, hy, (float)(xj - (double)hx), (float)(yj - (double)hy));
                sa[e] = make_float4((float)q[j], MODE == 1 ? (float)ax[j] : 0.0f, MODE == 1 ? (float)ay[j] : 0.0f,
                                    0.0f);
            }
            __syncthreads();
            if (valid)
                adj_tile_fp32c<MODE>(d, sp, sa, cnt, j0, li, xh, yh, xl, yl, qci, axf, ayf, x, y, xi, yi, fs,
                                     fc);
        } else {
            AdjJ *sj = reinterpret_cast<AdjJ *>(smem);
            float2 *sf = reinterpret_cast<float2 *>(sj + kAdjTile);
            if (threadIdx.x == 0) s_amax = 0u;
            __syncthreads();
            float am = 0.0f;
            for (int e = threadIdx.x; e < cnt; e += kAdjThreads) {
                const int j = d.off + j0 + e;
                AdjJ v;
                v.x = x[j];
                v.y = y[j];
                v.q = q[j];
                v.ax = (MODE == 1) ? ax[j] : 0.0;
                v.ay = (MODE == 1) ? ay[j] : 0.0;
                sj[e] = v;
                const float2 f = make_float2((float)v.x, (float)v.y);
                sf[e] = f;
                am = fmaxf(am, fmaxf(fabsf(f.x), fabsf(f.y)));  // NaN is dropped: its pairs fail the test
            }
            for (int o = 16; o > 0; o >>= 1) am = fmaxf(am, __shfl_xor_sync(0xffffffffu, am, o));
            if ((threadIdx.x & 31) == 0) atomicMax(&s_amax, __float_as_uint(am));  // non-negative: int order
            __syncthreads();
            if (valid)
                adj_tile_fp64<MODE>(d, sj, sf, cnt, j0, li, xi, yi, qi, axi, ayi, xfi, yfi,
                                    adj_candidate_bound(rc, ai, __uint_as_float(s_amax)), coulomb, S);
        }
    }
    if (!valid) return;
    if (F32C) {
#pragma unroll
        for (int k = 0; k < 4; k++) S.v[k] = (double)fs[k] - (double)fc[k];
    }
    const double xv = vx[i], yv = vy[i], mi = m[i];
    if (MODE == 0) {
        double fx = 0.0, fy = 0.0;
        if (d.flags & kConfinement) { fx += qi * d.confine * xi; fy += qi * d.confine * yi; }
        if (d.flags & kDrag) { fx += -d.gamma * mi * xv; fy += -d.gamma * mi * yv; }
        if (d.flags & kRectConfinement) { fx += qi * d.confine_x * xi; fy += qi * d.confine_y * yi; }
        fx += S.v[0];
        fy += S.v[1];
        o0[i] = fx;   // total force
        o1[i] = fy;
        if (o2) o2[i] = S.v[0];  // pair force only
        if (o3) o3[i] = S.v[1];
    } else {
        double gx = S.v[0], gy = S.v[1], gq = (qi != 0.0) ? S.v[2] / qi : 0.0, gkc = 0.0;
        if (d.flags & kConfinement) {
            gx += qi * d.confine * axi;
            gy += qi * d.confine * ayi;
            gq += d.confine * (xi * axi + yi * ayi);
            gkc = qi * (xi * axi + yi * ayi);
        }
        if (d.flags & kRectConfinement) {
            gx += qi * d.confine_x * axi;
            gy += qi * d.confine_y * ayi;
            gq += d.confine_x * xi * axi + d.confine_y * yi * ayi;
        }
        const double gv = (d.flags & kDrag) ? -d.gamma * mi : 0.0;
        o0[i] = gx;          // dL/dp (through the forces)
        o1[i] = gy;
        o2[i] = gv * axi;    // dL/dv (through drag)
        o3[i] = gv * ayi;
        o4[i] = gq;          // dL/dq_i
        o5[i] = S.v[3];      // dL/dkappa contribution of particle i
        o6[i] = gkc;         // dL/dk_c contribution of particle i
    }
}


// ===========================================================================
// Fused RK4 step and its adjoint for the differentiable rollout.
//
// One launch per RK4 stage.  Forward (adj_step_forces): the pair force at
// the stage's input state, the per-particle forces, and the stage algebra
// of the rollout's RK4 step in FP64 (for s = (x, y, vx, vy) and f(s) =
// (vx, vy, Fx/m, Fy/m)):
//     k_s = dt f(s_s),  s_2 = S + k_1/2, s_3 = S + k_2/2, s_4 = S + k_3,
//     S' = S + (k_1 + ((k_2 + k_3) 2 + k_4)) / 6,
// with the operations in that order (each rounded, nothing contracted).
// Backward (adj_step_vjp, stages 4, 3, 2, 1): given lam = dL/dS', the stage
// weights dk_4 = lam/6, dk_3 = lam/3 + mu_4, dk_2 = lam/3 + mu_3/2,
// dk_1 = lam/6 + mu_2/2 with mu_s = J(s_s)^T (dt dk_s), and finally
// dL/dS = lam + mu_1 + mu_2 + mu_3 + mu_4; the parameter gradients
// (dt dk_s)^T df/dtheta are added into per-particle accumulators.  J^T w
// for f is (the force VJP of a = w_v / m) for positions, w_p - gamma w_v
// for velocities.
//
// FP32C pair terms: one i per thread, j staged in shared memory as negated
// two-float positions (plus charge and, backward, the j's force adjoint), two
// j per packed f32x2 evaluation (pair2_terms), the cutoff by a select (pairs
// within 4e-6 of it in r^2 decided by the reference's FP64 test on the FP64
// positions), plain sums over four j, then Kahan; C q_i applied in FP64 per
// particle.  FP64: adj_tile_fp64.
// ===========================================================================

constexpr int kAsJ = 256;  // j staged per tile (a multiple of 4)

struct AdjStepIO {
    const double *x, *y, *vx, *vy;  // the stage's input state s_s
    double *sx, *sy, *svx, *svy;    // the step's base state S (stage 4 writes S' over it)
    double *k1[4], *k23[4];         // k_1 and k_2 + k_3
    double *nx, *ny, *nvx, *nvy;    // the next stage's input (stages 1-3)
    const double *q, *m;
    double dt;
    int stage;
};

struct AdjVjpIO {
    const double *x, *y, *vx, *vy;  // the stage's input state s_s
    const double *dk[4];            // dk_s (stage 4: lam, divided by 6 here)
    double *dkn[4];                 // dk_{s-1} (stages 4-2)
    double *lam[4];                 // dL/dS' in, dL/dS out (stage 1)
    double *mu[3][4];               // mu_4, mu_3, mu_2
    double *gq, *gkappa, *gkc;      // per-particle parameter gradients (added to)
    const double *q, *m;
    double dt;
    int stage;
};

// dk_s of particle k, component c.
__device__ __forceinline__ double adj_dk(const AdjVjpIO &V, int c, int k) {
    return V.stage == 4 ? __ddiv_rn(V.lam[c][k], 6.0) : V.dk[c][k];
}

// One pair term in FP32 for the slow path (pairs within 4e-6 of the cutoff
// in r^2): 0 outside the cutoff (the reference's FP64 test decides).
__device__ __forceinline__ bool adj_border_in(const AdjCloud &d, const double *x, const double *y, int i, int j) {
    double r, a;
    return ref_in_cutoff(__dsub_rn(x[i], x[j]), __dsub_rn(y[i], y[j]), d.kappa, r, a);
}

// FP32C pair sums of particle li of cloud d over the cloud's j, staged kAsJ
// at a time as chunks of 4 j (one float4 per quantity, so a chunk is read
// with a few broadcast loads).  MODE 0: out[0..1] = sum_j w_ij (dx, dy)
// (times C q_i: the pair force).  MODE 1 (a_i, a_j the force adjoints):
// out[0..1] = sum w b + h d (d . b), out[2] = sum w (d . b), out[3] = sum q_j
// e y (a_i . d) (times C q_i: the position VJP, F_ij . (a_i - a_j) and, times
// -kappa, dg/dkappa), with b = a_i - a_j.  j == i is the pair with r^2 = 0
// exactly (dx = dy = 0), left out by the select.  Every thread of the block
// calls it.
template <int MODE>
__device__ __forceinline__ void adj_pair_sums_fp32c(const AdjCloud &d, int li, bool valid, const double *x,
                                                    const double *y, const double *q, const float *ajx,
                                                    const float *ajy, float aix, float aiy, float (&out)[4]) {
    constexpr int NQ = MODE == 0 ? 5 : 7;  // -xh, -yh, -xl, -yl, q (, a_x, a_y)
    constexpr int NC = kAsJ / 4;
    __shared__ float4 s_c[NQ][NC];
    constexpr int NS = MODE == 0 ? 2 : 4;
    float sum[NS], cmp[NS];
#pragma unroll
    for (int k = 0; k < NS; k++) sum[k] = cmp[k] = 0.0f;
    const int i = d.off + (valid ? li : 0);
    float xh = 0.0f, yh = 0.0f, xl = 0.0f, yl = 0.0f;
    if (valid) split2(x[i], xh, xl), split2(y[i], yh, yl);
    const PairI I{dup2(xh), dup2(yh), dup2(xl), dup2(yl)};
    const float2 kap = dup2(d.kappa_f), nkl2e = dup2(d.nkl2e);
    const float2 nk2 = dup2(-d.kappa2_f), m3 = dup2(-3.0f);
    const float2 ax2 = dup2(aix), ay2 = dup2(aiy);
    const float lo = d.rc2_lo, hi = d.rc2_hi;
    float *s_f = reinterpret_cast<float *>(s_c);
    for (int j0 = 0; j0 < d.n; j0 += kAsJ) {
        const int cnt = min(kAsJ, d.n - j0);
        const int nch = (cnt + 3) >> 2;
        __syncthreads();
        for (int e = threadIdx.x; e < 4 * nch; e += blockDim.x) {
            float v[NQ];
            if (e < cnt) {
                const int j = d.off + j0 + e;
                float h, l;
                split2(x[j], h, l);
                v[0] = -h;
                v[2] = -l;
                split2(y[j], h, l);
                v[1] = -h;
                v[3] = -l;
                v[4] = (float)q[j];
                if (MODE == 1) {
                    v[5] = ajx[j];
                    v[6] = ajy[j];
                }
            } else {  // padding: far away, no charge (a finite, zero term)
                v[0] = v[1] = -kPadPosition;
                v[2] = v[3] = v[4] = 0.0f;
                if (MODE == 1) v[5] = v[6] = 0.0f;
            }
#pragma unroll
            for (int k = 0; k < NQ; k++) s_f[k * kAsJ + e] = v[k];  // s_c[k][e/4].{x,y,z,w}[e%4]
        }
        __syncthreads();
        if (!valid) continue;
        for (int c = 0; c < nch; c++) {
            float4 Q[NQ];
#pragma unroll
            for (int k = 0; k < NQ; k++) Q[k] = s_c[k][c];
            float2 part[NS];
#pragma unroll
            for (int k = 0; k < NS; k++) part[k] = dup2(0.0f);
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const float2 nxh = h ? make_float2(Q[0].z, Q[0].w) : make_float2(Q[0].x, Q[0].y);
                const float2 nyh = h ? make_float2(Q[1].z, Q[1].w) : make_float2(Q[1].x, Q[1].y);
                const float2 nxl = h ? make_float2(Q[2].z, Q[2].w) : make_float2(Q[2].x, Q[2].y);
                const float2 nyl = h ? make_float2(Q[3].z, Q[3].w) : make_float2(Q[3].x, Q[3].y);
                const float2 qj = h ? make_float2(Q[4].z, Q[4].w) : make_float2(Q[4].x, Q[4].y);
                float2 dx, dy, r2, yy, ex;
                pair2_core(I, nxh, nyh, nxl, nyl, nkl2e, dx, dy, r2, yy, ex);
                bool ina = r2.x < lo && r2.x > 0.0f, inb = r2.y < lo && r2.y > 0.0f;
                // pairs within 4e-6 of the cutoff in r^2: the reference's FP64 test
                if (__any_sync(0xffffffffu, (r2.x >= lo && r2.x < hi) || (r2.y >= lo && r2.y < hi))) {
                    const int ja = j0 + 4 * c + 2 * h;
                    if (r2.x >= lo && r2.x < hi && ja < d.n) ina = adj_border_in(d, x, y, i, d.off + ja);
                    if (r2.y >= lo && r2.y < hi && ja + 1 < d.n) inb = adj_border_in(d, x, y, i, d.off + ja + 1);
                }
                // q_j e^{-kappa r} and 1/r, both 0 outside the cutoff and for j == i
                // (where r = 0 made them non-finite), so every term below is 0 there
                float2 qe = mul2(qj, ex);
                qe.x = ina ? qe.x : 0.0f;
                qe.y = inb ? qe.y : 0.0f;
                yy.x = ina ? yy.x : 0.0f;
                yy.y = inb ? yy.y : 0.0f;
                const float2 y2 = mul2(yy, yy);
                const float2 t = add2(yy, kap);
                const float2 ww = mul2(qe, mul2(y2, t));  // g / (C q_i)
                if (MODE == 0) {
                    part[0] = fma2(ww, dx, part[0]);
                    part[1] = fma2(ww, dy, part[1]);
                } else {
                    const float2 ajx2 = h ? make_float2(Q[5].z, Q[5].w) : make_float2(Q[5].x, Q[5].y);
                    const float2 ajy2 = h ? make_float2(Q[6].z, Q[6].w) : make_float2(Q[6].x, Q[6].y);
                    // h / (C q_i) = -q_j e y^3 (kappa^2 + 3 y (y + kappa))
                    const float2 hv = mul2(mul2(qe, mul2(y2, yy)), fma2(mul2(yy, m3), t, nk2));
                    const float2 bx = add2(ax2, make_float2(-ajx2.x, -ajx2.y));
                    const float2 by = add2(ay2, make_float2(-ajy2.x, -ajy2.y));
                    const float2 dd = fma2(dx, bx, mul2(dy, by));
                    const float2 aid = fma2(ax2, dx, mul2(ay2, dy));
                    const float2 hdd = mul2(hv, dd);
                    part[0] = fma2(ww, bx, fma2(hdd, dx, part[0]));
                    part[1] = fma2(ww, by, fma2(hdd, dy, part[1]));
                    part[2] = fma2(ww, dd, part[2]);
                    part[3] = fma2(mul2(qe, yy), aid, part[3]);
                }
            }
#pragma unroll
            for (int k = 0; k < NS; k++) kahan_add(sum[k], cmp[k], part[k].x + part[k].y);
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) out[k] = (k < NS) ? sum[k] - cmp[k] : 0.0f;
}

// The pair sums of particle i in FP64 (adj_tile_fp64), the same outputs as
// adj_pair_sums_fp32c multiplied out (C q_i included).
template <int MODE>
__device__ __forceinline__ void adj_pair_sums_fp64(const AdjCloud &d, int li, bool valid, const double *x,
                                                   const double *y, const double *q, const double *ajx,
                                                   const double *ajy, double axi, double ayi, double coulomb,
                                                   double (&out)[4]) {
    __shared__ AdjJ sj[kAdjTile];
    __shared__ float2 sf[kAdjTile];
    __shared__ unsigned int s_amax;
    AdjSums S{};
    const int i = d.off + (valid ? li : 0);
    const double xi = x[i], yi = y[i], qi = q[i];
    const float xfi = (float)xi, yfi = (float)yi;
    const float ai = fmaxf(fabsf(xfi), fabsf(yfi));
    const double rc = sqrt(d.rc2);
    for (int j0 = 0; j0 < d.n; j0 += kAdjTile) {
        const int cnt = min(kAdjTile, d.n - j0);
        __syncthreads();
        if (threadIdx.x == 0) s_amax = 0u;
        __syncthreads();
        float am = 0.0f;
        for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
            const int j = d.off + j0 + e;
            AdjJ v;
            v.x = x[j];
            v.y = y[j];
            v.q = q[j];
            v.ax = (MODE == 1) ? ajx[j] : 0.0;
            v.ay = (MODE == 1) ? ajy[j] : 0.0;
            sj[e] = v;
            const float2 f = make_float2((float)v.x, (float)v.y);
            sf[e] = f;
            am = fmaxf(am, fmaxf(fabsf(f.x), fabsf(f.y)));
        }
        for (int o = 16; o > 0; o >>= 1) am = fmaxf(am, __shfl_xor_sync(0xffffffffu, am, o));
        if ((threadIdx.x & 31) == 0) atomicMax(&s_amax, __float_as_uint(am));  // non-negative: int order
        __syncthreads();
        if (valid)
            adj_tile_fp64<MODE>(d, sj, sf, cnt, j0, li, xi, yi, qi, axi, ayi, xfi, yfi,
                                adj_candidate_bound(rc, ai, __uint_as_float(s_amax)), coulomb, S);
    }
#pragma unroll
    for (int k = 0; k < 4; k++) out[k] = S.v[k];
}

// Forward stage of the fused RK4 step (one thread per particle).
template <bool F32C>
__global__ void __launch_bounds__(kAdjThreads) adj_step_forces(const AdjCloud *__restrict__ desc,
                                                               const int *__restrict__ cloud_of_block,
                                                               const int *__restrict__ tile_of_block,
                                                               const AdjStepIO io, double coulomb) {
    const AdjCloud d = desc[cloud_of_block[blockIdx.x]];
    const int li = tile_of_block[blockIdx.x] * kAdjThreads + threadIdx.x;
    const bool valid = li < d.n;
    const int i = d.off + (valid ? li : 0);
    double px = 0.0, py = 0.0;
    if (d.flags & kShieldedCoulomb) {
        if (F32C) {
            float o[4];
            adj_pair_sums_fp32c<0>(d, li, valid, io.x, io.y, io.q, nullptr, nullptr, 0.0f, 0.0f, o);
            const double cq = __dmul_rn(coulomb, io.q[i]);
            px = __dmul_rn(cq, (double)o[0]);
            py = __dmul_rn(cq, (double)o[1]);
        } else {
            double o[4];
            adj_pair_sums_fp64<0>(d, li, valid, io.x, io.y, io.q, nullptr, nullptr, 0.0, 0.0, coulomb, o);
            px = o[0];
            py = o[1];
        }
    }
    if (!valid) return;
    const double xi = io.x[i], yi = io.y[i], vxi = io.vx[i], vyi = io.vy[i], qi = io.q[i], mi = io.m[i];
    double fx = 0.0, fy = 0.0;
    if (d.flags & kConfinement) { fx += qi * d.confine * xi; fy += qi * d.confine * yi; }
    if (d.flags & kDrag) { fx += -d.gamma * mi * vxi; fy += -d.gamma * mi * vyi; }
    if (d.flags & kRectConfinement) { fx += qi * d.confine_x * xi; fy += qi * d.confine_y * yi; }
    fx += px;
    fy += py;
    const double dt = io.dt;
    const double k[4] = {__dmul_rn(dt, vxi), __dmul_rn(dt, vyi), __dmul_rn(dt, __ddiv_rn(fx, mi)),
                         __dmul_rn(dt, __ddiv_rn(fy, mi))};
    double *const S[4] = {io.sx, io.sy, io.svx, io.svy};
    double *const N[4] = {io.nx, io.ny, io.nvx, io.nvy};
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const double base = S[c][i];
        if (io.stage == 1) {
            io.k1[c][i] = k[c];
            N[c][i] = __dadd_rn(base, __dmul_rn(0.5, k[c]));
        } else if (io.stage == 2) {
            io.k23[c][i] = k[c];
            N[c][i] = __dadd_rn(base, __dmul_rn(0.5, k[c]));
        } else if (io.stage == 3) {
            io.k23[c][i] = __dadd_rn(io.k23[c][i], k[c]);
            N[c][i] = __dadd_rn(base, k[c]);
        } else {
            const double inc = __ddiv_rn(__dadd_rn(io.k1[c][i], __dadd_rn(__dmul_rn(io.k23[c][i], 2.0), k[c])), 6.0);
            S[c][i] = __dadd_rn(base, inc);
        }
    }
}

// The force adjoint a = dt dk_v / m of every particle for a VJP stage.
__global__ void adj_force_adjoint(const AdjVjpIO V, int n, float *axf, float *ayf, double *axd, double *ayd) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double ax = __ddiv_rn(__dmul_rn(V.dt, adj_dk(V, 2, k)), V.m[k]);
    const double ay = __ddiv_rn(__dmul_rn(V.dt, adj_dk(V, 3, k)), V.m[k]);
    axd[k] = ax;
    ayd[k] = ay;
    axf[k] = (float)ax;
    ayf[k] = (float)ay;
}

// Backward stage (one thread per particle); a = dt dk_v / m of every
// particle precomputed by adj_force_adjoint (axd/ayd, FP32 copies axf/ayf).
template <bool F32C>
__global__ void __launch_bounds__(kAdjThreads) adj_step_vjp(const AdjCloud *__restrict__ desc,
                                                            const int *__restrict__ cloud_of_block,
                                                            const int *__restrict__ tile_of_block, const AdjVjpIO V,
                                                            const float *__restrict__ axf, const float *__restrict__ ayf,
                                                            const double *__restrict__ axd,
                                                            const double *__restrict__ ayd, double coulomb) {
    const AdjCloud d = desc[cloud_of_block[blockIdx.x]];
    const int li = tile_of_block[blockIdx.x] * kAdjThreads + threadIdx.x;
    const bool valid = li < d.n;
    const int i = d.off + (valid ? li : 0);
    const double axi = axd[i], ayi = ayd[i];
    double S[4] = {0.0, 0.0, 0.0, 0.0};
    if (d.flags & kShieldedCoulomb) {
        if (F32C) {
            float o[4];
            adj_pair_sums_fp32c<1>(d, li, valid, V.x, V.y, V.q, axf, ayf, (float)axi, (float)ayi, o);
            const double cq = __dmul_rn(coulomb, V.q[i]);
            S[0] = __dmul_rn(cq, (double)o[0]);
            S[1] = __dmul_rn(cq, (double)o[1]);
            S[2] = __dmul_rn(cq, (double)o[2]);
            S[3] = __dmul_rn(__dmul_rn(-d.kappa, cq), (double)o[3]);
        } else {
            adj_pair_sums_fp64<1>(d, li, valid, V.x, V.y, V.q, axd, ayd, axi, ayi, coulomb, S);
        }
    }
    if (!valid) return;
    const double xi = V.x[i], yi = V.y[i], qi = V.q[i], mi = V.m[i];
    double gx = S[0], gy = S[1], gq = (qi != 0.0) ? S[2] / qi : 0.0, gkc = 0.0;
    if (d.flags & kConfinement) {
        gx += qi * d.confine * axi;
        gy += qi * d.confine * ayi;
        gq += d.confine * (xi * axi + yi * ayi);
        gkc = qi * (xi * axi + yi * ayi);
    }
    if (d.flags & kRectConfinement) {
        gx += qi * d.confine_x * axi;
        gy += qi * d.confine_y * ayi;
        gq += d.confine_x * xi * axi + d.confine_y * yi * ayi;
    }
    const double gv = (d.flags & kDrag) ? -d.gamma * mi : 0.0;
    const double dt = V.dt;
    // mu = J^T (dt dk): positions through the forces, velocities through
    // f_pos = v and the drag
    const double mu[4] = {gx, gy, __dadd_rn(__dmul_rn(dt, adj_dk(V, 0, i)), gv * axi),
                          __dadd_rn(__dmul_rn(dt, adj_dk(V, 1, i)), gv * ayi)};
    V.gq[i] += gq;
    V.gkappa[i] += S[3];
    V.gkc[i] += gkc;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const double l = V.lam[c][i];
        if (V.stage == 4) {
            V.mu[0][c][i] = mu[c];
            V.dkn[c][i] = __dadd_rn(__ddiv_rn(l, 3.0), mu[c]);
        } else if (V.stage == 3) {
            V.mu[1][c][i] = mu[c];
            V.dkn[c][i] = __dadd_rn(__ddiv_rn(l, 3.0), __dmul_rn(0.5, mu[c]));
        } else if (V.stage == 2) {
            V.mu[2][c][i] = mu[c];
            V.dkn[c][i] = __dadd_rn(__ddiv_rn(l, 6.0), __dmul_rn(0.5, mu[c]));
        } else {
            V.lam[c][i] = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(l, mu[c]), V.mu[2][c][i]), V.mu[1][c][i]),
                                    V.mu[0][c][i]);
        }
    }
}

}  // namespace dm
