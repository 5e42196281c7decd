// dm_adjoint.cuh -- forces and their vector-Jacobian product for the
// differentiable rollout (FP64).
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

#include "dm_device.cuh"

namespace dm {

struct AdjCloud {
    int off, n;
    long long flags;
    double kappa, confine, confine_x, confine_y, gamma;
    double rc2;
};

constexpr int kAdjThreads = 128;
constexpr int kAdjTile = 256;

struct alignas(16) AdjJ {
    double x, y, q, ax, ay, b;
};

// One thread per particle i, j of the same cloud staged through shared
// memory.  MODE 0: forces (total F and pair-only Fp).  MODE 1: VJP.
template <int MODE>
__global__ void __launch_bounds__(kAdjThreads) adjoint_kernel(
    const AdjCloud *__restrict__ desc, const int *__restrict__ cloud_of_block, const int *__restrict__ tile_of_block,
    const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ vx,
    const double *__restrict__ vy, const double *__restrict__ q, const double *__restrict__ m,
    const double *__restrict__ ax, const double *__restrict__ ay,  // MODE 1: force adjoint
    double *__restrict__ o0, double *__restrict__ o1, double *__restrict__ o2, double *__restrict__ o3,
    double *__restrict__ o4, double *__restrict__ o5, double *__restrict__ o6, double *__restrict__ o7,
    double coulomb) {
    __shared__ AdjJ sj[kAdjTile];
    const AdjCloud d = desc[cloud_of_block[blockIdx.x]];
    const int li = tile_of_block[blockIdx.x] * kAdjThreads + threadIdx.x;  // index within the cloud
    const bool valid = li < d.n;
    const int i = d.off + (valid ? li : 0);
    const double xi = x[i], yi = y[i], qi = q[i];
    const double axi = (MODE == 1 && valid) ? ax[i] : 0.0, ayi = (MODE == 1 && valid) ? ay[i] : 0.0;
    const double a2 = xi * xi + yi * yi;
    const double rc = sqrt(d.rc2);
    const double pr = sqrt(a2) + rc;
    const double U = (d.rc2 - a2) + 5.684341886080802e-14 * pr * pr;
    const bool coul = (d.flags & kShieldedCoulomb) != 0;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0, s4 = 0.0;
    for (int j0 = 0; j0 < d.n && coul; j0 += kAdjTile) {
        const int cnt = min(kAdjTile, d.n - j0);
        __syncthreads();
        for (int e = threadIdx.x; e < cnt; e += kAdjThreads) {
            const int j = d.off + j0 + e;
            AdjJ v;
            v.x = x[j];
            v.y = y[j];
            v.q = q[j];
            v.ax = (MODE == 1) ? ax[j] : 0.0;
            v.ay = (MODE == 1) ? ay[j] : 0.0;
            v.b = v.x * v.x + v.y * v.y;
            sj[e] = v;
        }
        __syncthreads();
        if (!valid) continue;
        for (int e = 0; e < cnt; e++) {
            const AdjJ v = sj[e];
            if (fma(-2.0 * xi, v.x, fma(-2.0 * yi, v.y, v.b)) >= U) continue;
            if (j0 + e == li) continue;
            const double dx = __dsub_rn(xi, v.x), dy = __dsub_rn(yi, v.y);
            double r, a;
            if (!ref_in_cutoff(dx, dy, d.kappa, r, a)) continue;
            const double ex = exp(-a);
            const double g = coulomb * qi * v.q * (1.0 + a) * ex / (r * r * r);
            if (MODE == 0) {
                s0 += g * dx;
                s1 += g * dy;
            } else {
                const double h = -g * (d.kappa * d.kappa / (1.0 + a) + 3.0 / (r * r));
                const double bx = axi - v.ax, by = ayi - v.ay;
                const double dd = dx * bx + dy * by;
                s0 += g * bx + h * dx * dd;         // position adjoint
                s1 += g * by + h * dy * dd;
                s2 += g * dd;                        // F_kj . (a_k - a_j)  (charge)
                const double gk = -coulomb * qi * v.q * d.kappa * ex / r;  // dg/dkappa
                s3 += gk * (axi * dx + ayi * dy);    // kappa
            }
        }
    }
    if (!valid) return;
    const double xv = vx[i], yv = vy[i], mi = m[i];
    if (MODE == 0) {
        double fx = 0.0, fy = 0.0;
        if (d.flags & kConfinement) { fx += qi * d.confine * xi; fy += qi * d.confine * yi; }
        if (d.flags & kDrag) { fx += -d.gamma * mi * xv; fy += -d.gamma * mi * yv; }
        if (d.flags & kRectConfinement) { fx += qi * d.confine_x * xi; fy += qi * d.confine_y * yi; }
        fx += s0;
        fy += s1;
        o0[i] = fx;   // total force
        o1[i] = fy;
        if (o2) o2[i] = s0;  // pair force only
        if (o3) o3[i] = s1;
    } else {
        double gx = s0, gy = s1, gq = (qi != 0.0) ? s2 / qi : 0.0, gkc = 0.0;
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
        o5[i] = s3;          // dL/dkappa contribution of particle i
        o6[i] = gkc;         // dL/dk_c contribution of particle i
        if (o7) o7[i] = 0.0;
    }
}

}  // namespace dm
