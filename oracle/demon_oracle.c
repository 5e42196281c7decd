/*
 * demon_oracle.c -- CPU oracle (test infrastructure only; see demon_oracle.h).
 *
 * Plain-C restatement of the reference's hot path.  Every function cites the
 * reference file:line it follows.  Build with -ffp-contract=off so no
 * multiply-add is fused: the reference is compiled for SSE4.2, which has no
 * FMA, and on aarch64 GCC would otherwise contract a*b+c.
 */
#include "demon_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Cloud::epsilon0 (Cloud.cpp:16) and ShieldedCoulombForce::coulomb
 * (ShieldedCoulombForce.cpp:21). */
static const double kEpsilon0 = 8.8541878E-12;

double or_coulomb(void) { return 1.0 / (4.0 * M_PI * kEpsilon0); }

/* ---------------------------------------------------------------------------
 * Shielded Coulomb (Yukawa) pair force.
 * ------------------------------------------------------------------------- */

/* Block form used for every pair outside the (i, i+1) 2-block
 * (ShieldedCoulombForce.cpp:172-198 and 211-237):
 *   r = sqrt(dx*dx + dy*dy); a = r*kappa; if a < 10:
 *   f = C*qq*(1+a)*exp(-a)/(r*r*r), F = f*(dx, dy).
 * Returns 1 and the force on the i side if the pair is inside the cutoff. */
static inline int pair_block(double dx, double dy, double qq, double kappa,
                             double coulomb, double *fxo, double *fyo) {
    const double r = sqrt(dx * dx + dy * dy);
    const double a = r * kappa;
    if (!(a < 10.0)) return 0;
    const double f = coulomb * qq * (1.0 + a) * exp(-a) / (r * r * r);
    *fxo = f * dx;
    *fyo = f * dy;
    return 1;
}

/* Intra-block form for the pair (i, i+1) (ShieldedCoulombForce.cpp:138-159):
 *   f = C*qq*(1+a)/(r*r*r*exp(a)). */
static inline int pair_intra(double dx, double dy, double qq, double kappa,
                             double coulomb, double *fxo, double *fyo) {
    const double r = sqrt(dx * dx + dy * dy);
    const double a = r * kappa;
    if (!(a < 10.0)) return 0;
    const double f = coulomb * qq * (1.0 + a) / (r * r * r * exp(a));
    *fxo = f * dx;
    *fyo = f * dy;
    return 1;
}

/* One call of the 2-lane block routines for i-block ib and j-block jb:
 * force(i, j) then forcer(i, j) (ShieldedCoulombForce.cpp:54-55), with each
 * element's += / -= in the reference's order. */
static inline void block_pair_serial(int ib, int jb, const double *x,
                                     const double *y, const double *q,
                                     double kappa, double C, double *fx,
                                     double *fy) {
    double ax, ay, bx, by;
    int ha, hb;
    /* force(i, j): lane0 = (ib, jb), lane1 = (ib+1, jb+1); F_i += ; F_j -= */
    ha = pair_block(x[ib] - x[jb], y[ib] - y[jb], q[ib] * q[jb], kappa, C, &ax, &ay);
    hb = pair_block(x[ib + 1] - x[jb + 1], y[ib + 1] - y[jb + 1], q[ib + 1] * q[jb + 1],
                    kappa, C, &bx, &by);
    if (ha || hb) {
        if (ha) { fx[ib] += ax; fy[ib] += ay; }
        if (hb) { fx[ib + 1] += bx; fy[ib + 1] += by; }
        if (ha) { fx[jb] -= ax; fy[jb] -= ay; }
        if (hb) { fx[jb + 1] -= bx; fy[jb + 1] -= by; }
    }
    /* forcer(i, j): lane0 = (ib, jb+1), lane1 = (ib+1, jb);
     * minusEqualr_pd subtracts lane0 from F_{j+1} and lane1 from F_j
     * (ShieldedCoulombForce.cpp:294-300). */
    ha = pair_block(x[ib] - x[jb + 1], y[ib] - y[jb + 1], q[ib] * q[jb + 1], kappa, C, &ax, &ay);
    hb = pair_block(x[ib + 1] - x[jb], y[ib + 1] - y[jb], q[ib + 1] * q[jb], kappa, C, &bx, &by);
    if (ha || hb) {
        if (ha) { fx[ib] += ax; fy[ib] += ay; }
        if (hb) { fx[ib + 1] += bx; fy[ib + 1] += by; }
        if (hb) { fx[jb] -= bx; fy[jb] -= by; }
        if (ha) { fx[jb + 1] -= ax; fy[jb + 1] -= ay; }
    }
}

void or_shielded_coulomb(int n, const double *x, const double *y,
                         const double *q, double kappa, double *fx,
                         double *fy) {
    const double C = or_coulomb();
    const int ne = n & ~1; /* the reference requires even n */
    /* ShieldedCoulombForce.cpp:43: for (i = 0; i < n-1; i += 2) */
    for (int ib = 0; ib + 1 < ne; ib += 2) {
        double ax, ay;
        /* force(i, q_i*q_{i+1}, hsub(x, y)) (ShieldedCoulombForce.cpp:51) */
        if (pair_intra(x[ib] - x[ib + 1], y[ib] - y[ib + 1], q[ib] * q[ib + 1], kappa,
                       C, &ax, &ay)) {
            fx[ib] += ax; fy[ib] += ay;
            fx[ib + 1] += -ax; fy[ib + 1] += -ay;
        }
        /* ShieldedCoulombForce.cpp:52-56 */
        for (int jb = ib + 2; jb < ne; jb += 2)
            block_pair_serial(ib, jb, x, y, q, kappa, C, fx, fy);
    }
    if (n & 1) {
        /* odd tail (outside the reference's domain): same block formula */
        const int k = n - 1;
        for (int i = 0; i < k; i++) {
            double ax, ay;
            if (pair_block(x[i] - x[k], y[i] - y[k], q[i] * q[k], kappa, C, &ax, &ay)) {
                fx[i] += ax; fy[i] += ay;
                fx[k] -= ax; fy[k] -= ay;
            }
        }
    }
}

void or_shielded_coulomb_omp(int n, const double *x, const double *y,
                             const double *q, double kappa, double *fx,
                             double *fy, int nthreads) {
#ifdef _OPENMP
    const double C = or_coulomb();
    const int ne = n & ~1;
    const int nblocks = ne / 2;
    omp_lock_t *locks = (omp_lock_t *)malloc(sizeof(omp_lock_t) * (size_t)(nblocks > 0 ? nblocks : 1));
    for (int b = 0; b < nblocks; b++) omp_init_lock(&locks[b]);
    if (nthreads <= 0) nthreads = omp_get_num_procs();
    /* ShieldedCoulombForce.cpp:43-57: OpenMP dynamic over i blocks, one lock
     * per 2-particle block taken around each += and -= (lines 154-157,
     * 188-197, 227-236). */
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
    for (int ib = 0; ib < ne - 1; ib += 2) {
        double ax, ay, bx, by;
        int ha, hb;
        if (pair_intra(x[ib] - x[ib + 1], y[ib] - y[ib + 1], q[ib] * q[ib + 1], kappa, C,
                       &ax, &ay)) {
            omp_set_lock(&locks[ib / 2]);
            fx[ib] += ax; fy[ib] += ay;
            fx[ib + 1] += -ax; fy[ib + 1] += -ay;
            omp_unset_lock(&locks[ib / 2]);
        }
        for (int jb = ib + 2; jb < ne; jb += 2) {
            ha = pair_block(x[ib] - x[jb], y[ib] - y[jb], q[ib] * q[jb], kappa, C, &ax, &ay);
            hb = pair_block(x[ib + 1] - x[jb + 1], y[ib + 1] - y[jb + 1],
                            q[ib + 1] * q[jb + 1], kappa, C, &bx, &by);
            if (ha || hb) {
                omp_set_lock(&locks[ib / 2]);
                if (ha) { fx[ib] += ax; fy[ib] += ay; }
                if (hb) { fx[ib + 1] += bx; fy[ib + 1] += by; }
                omp_unset_lock(&locks[ib / 2]);
                omp_set_lock(&locks[jb / 2]);
                if (ha) { fx[jb] -= ax; fy[jb] -= ay; }
                if (hb) { fx[jb + 1] -= bx; fy[jb + 1] -= by; }
                omp_unset_lock(&locks[jb / 2]);
            }
            ha = pair_block(x[ib] - x[jb + 1], y[ib] - y[jb + 1], q[ib] * q[jb + 1], kappa, C,
                            &ax, &ay);
            hb = pair_block(x[ib + 1] - x[jb], y[ib + 1] - y[jb], q[ib + 1] * q[jb], kappa, C,
                            &bx, &by);
            if (ha || hb) {
                omp_set_lock(&locks[ib / 2]);
                if (ha) { fx[ib] += ax; fy[ib] += ay; }
                if (hb) { fx[ib + 1] += bx; fy[ib + 1] += by; }
                omp_unset_lock(&locks[ib / 2]);
                omp_set_lock(&locks[jb / 2]);
                if (hb) { fx[jb] -= bx; fy[jb] -= by; }
                if (ha) { fx[jb + 1] -= ax; fy[jb + 1] -= ay; }
                omp_unset_lock(&locks[jb / 2]);
            }
        }
    }
    for (int b = 0; b < nblocks; b++) omp_destroy_lock(&locks[b]);
    free(locks);
    if (n & 1) {
        const int k = n - 1;
        for (int i = 0; i < k; i++) {
            double ax, ay;
            if (pair_block(x[i] - x[k], y[i] - y[k], q[i] * q[k], kappa, C, &ax, &ay)) {
                fx[i] += ax; fy[i] += ay;
                fx[k] -= ax; fy[k] -= ay;
            }
        }
    }
#else
    (void)nthreads;
    or_shielded_coulomb(n, x, y, q, kappa, fx, fy);
#endif
}

/* ---------------------------------------------------------------------------
 * Counter-based thermal kick.
 * ------------------------------------------------------------------------- */

/* Philox4x32-10 (Salmon et al., "Parallel random numbers: as easy as 1, 2,
 * 3", SC'11): 10 rounds of two 32x32->64 multiplies with the published
 * multipliers and Weyl key increments. */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)M0 * c0;
        const uint64_t p1 = (uint64_t)M1 * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += W0;
        k1 += W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Thermal kick arithmetic: FP32 Box-Muller from correctly rounded IEEE
 * single operations in a fixed order (this file is built with
 * -ffp-contract=off, fmaf is the correctly rounded fused multiply-add), the
 * same sequence as the CUDA path, so both give identical bits. */
static inline float u24(uint32_t w) {
    return ((float)(w >> 8) + 0.5f) * 5.9604644775390625e-8f;
}

static float thermal_log(float u) {
    uint32_t bits;
    memcpy(&bits, &u, 4);
    int e = (int)(bits >> 23) - 127;
    const uint32_t mb = (bits & 0x007FFFFFu) | 0x3F800000u;
    float m;
    memcpy(&m, &mb, 4);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = fmaf(s2, 0.111111111f, 0.142857143f);
    p = fmaf(s2, p, 0.2f);
    p = fmaf(s2, p, 0.333333333f);
    p = fmaf(s2, p, 1.0f);
    const float lnm = (2.0f * s) * p;
    return fmaf((float)e, 0.693147181f, lnm);
}

static void thermal_sincos(float u, float *sn, float *cs) {
    const float r = u * 4.0f;
    const float qf = floorf(r);
    const int q = (int)qf;
    const float a = (r - qf) * 1.57079633f;
    const float a2 = a * a;
    float ps = fmaf(a2, 1.60590438e-10f, -2.50521084e-8f);
    ps = fmaf(a2, ps, 2.75573192e-6f);
    ps = fmaf(a2, ps, -1.98412698e-4f);
    ps = fmaf(a2, ps, 8.33333333e-3f);
    ps = fmaf(a2, ps, -1.66666667e-1f);
    ps = fmaf(a2, ps, 1.0f);
    const float sa = a * ps;
    float pc = fmaf(a2, -1.14707456e-11f, 2.08767570e-9f);
    pc = fmaf(a2, pc, -2.75573192e-7f);
    pc = fmaf(a2, pc, 2.48015873e-5f);
    pc = fmaf(a2, pc, -1.38888889e-3f);
    pc = fmaf(a2, pc, 4.16666667e-2f);
    pc = fmaf(a2, pc, -0.5f);
    const float ca = fmaf(a2, pc, 1.0f);
    switch (q & 3) {
        case 0: *sn = sa; *cs = ca; break;
        case 1: *sn = ca; *cs = -sa; break;
        case 2: *sn = -sa; *cs = -ca; break;
        default: *sn = -ca; *cs = sa; break;
    }
}

/* One counter-based kick of magnitude scale `heat`: counter (i, step lo,
 * step hi, stream).  Stream = stage for ThermalForce, stage + 16 for
 * ThermalForceLocalized, stage + 32 for TimeVaryingThermalForce, so forces
 * that are on together draw independent numbers. */
static void thermal_draw(const or_params *p, uint32_t i, uint64_t step, int stream, double heat,
                         double *tx, double *ty) {
    const uint32_t ctr[4] = {i, (uint32_t)step, (uint32_t)(step >> 32), (uint32_t)stream};
    const uint32_t key[2] = {(uint32_t)p->seed, (uint32_t)(p->seed >> 32)};
    uint32_t o[4];
    or_philox4x32_10(ctr, key, o);
    const float u1 = u24(o[0]);
    const float u2 = u24(o[1]);
    float sn, cs;
    thermal_sincos(u2, &sn, &cs);
    /* mode 0: ThermalForce::force (ThermalForce.cpp:118-140), heatVal*U*(cos, sin);
     * mode 1: Gaussian, sigma = heat per axis (Box-Muller) */
    const float amp = (p->thermal_mode == 0) ? u1 : sqrtf(-2.0f * thermal_log(u1));
    *tx = heat * (double)(amp * cs);
    *ty = heat * (double)(amp * sn);
}

void or_thermal_one(const or_params *p, uint32_t i, uint64_t step, int stage,
                    double *tx, double *ty) {
    thermal_draw(p, i, step, stage, p->heat, tx, ty);
}

/* ---------------------------------------------------------------------------
 * The per-particle forces, one particle at a time.
 *
 * Each force adds into (*fx, *fy) exactly as the reference's force() adds
 * into forceX/forceY with plusEqual_pd/minusEqual_pd; a particle's sum in
 * the reference is the same sequence of additions whether the loops run
 * force-major (the reference) or particle-major (here).
 * ------------------------------------------------------------------------- */

/* DrivingForce::waveNum, angFreq (DrivingForce.cpp:14-15). */
static const double kWaveNum = 2.0 * M_PI / 0.002;
static const double kAngFreq = 2.0 * M_PI * 10.0;

typedef struct pstate {
    uint32_t i;
    double x, y, vx, vy, q, m;
} pstate;

/* ConfinementForce::force (ConfinementForce.cpp:48-54) */
static inline void f_confinement(const or_params *p, const pstate *s, double *fx, double *fy) {
    const double c = s->q * p->confine;
    *fx += c * s->x;
    *fy += c * s->y;
}

/* ConfinementForceVoid::force (ConfinementForceVoid.cpp:48-55), after the
 * ConfinementForce term it inherits (ConfinementForceVoid.cpp:13-17):
 * F += (q*(-decay)) * (exp(r*(-decay)) / r) * (x, y). */
static inline void f_void(const or_params *p, const pstate *s, double *fx, double *fy) {
    f_confinement(p, s, fx, fy);
    const double decayV = s->q * -p->void_decay;
    const double r = sqrt(s->x * s->x + s->y * s->y);
    const double expR = exp(r * -p->void_decay) / r;
    *fx += (decayV * expR) * s->x;
    *fy += (decayV * expR) * s->y;
}

/* DragForce::force (DragForce.cpp:49-55) with dragConst */
static inline void f_drag(double dragConst, const pstate *s, double *fx, double *fy) {
    const double d = s->m * dragConst;
    *fx += d * s->vx;
    *fy += d * s->vy;
}

/* DrivingForce::force (DrivingForce.cpp:52-61): the stored driveConst is
 * -drive_const (DrivingForce.h:17-18), so the exponent is
 * (dist - dist) / drive_const: exp(+-0) = 1 for a finite position. */
static inline void f_driving(const or_params *p, const pstate *s, double t, double *fx) {
    const double driveConst = -p->drive_const;
    const double distV = s->x - p->drive_shift;
    const double sinArg = s->x * kWaveNum - t * kAngFreq;
    const double expArg = (distV - distV) / -driveConst;
    *fx += (sin(sinArg) * exp(expArg)) * p->drive_amplitude;
}

/* MagneticForce::force (MagneticForce.cpp:48-54): F = q*(v x B), B along z */
static inline void f_magnetic(const or_params *p, const pstate *s, double *fx, double *fy) {
    const double qB = s->q * p->magnetic;
    *fx += qB * s->vy;
    *fy -= qB * s->vx;
}

/* RectConfinementForce::force (RectConfinementForce.cpp:50-59) */
static inline void f_rect(const or_params *p, const pstate *s, double *fx, double *fy) {
    *fx += (s->q * p->confine_x) * s->x;
    *fy += (s->q * p->confine_y) * s->y;
}

/* RotationalForce::force (RotationalForce.cpp:50-66): inside rmin < r < rmax,
 * F -= c*y/r along x and F += c*x/r along y. */
static inline void f_rotational(const or_params *p, const pstate *s, double *fx, double *fy) {
    const double r = sqrt(s->x * s->x + s->y * s->y);
    if (!(r > p->rot_rmin && r < p->rot_rmax)) return;
    *fx -= (p->rot_const * s->y) / r;
    *fy += (p->rot_const * s->x) / r;
}

/* ThermalForceLocalized::force (ThermalForceLocalized.cpp:124-133): heatVal1
 * (heat_in) inside r < heatingRadius, heatVal2 (heat_out) outside. */
static inline void f_thermal_localized(const or_params *p, const pstate *s, uint64_t step, int stage,
                                       double *fx, double *fy) {
    const double r = sqrt(s->x * s->x + s->y * s->y);
    const double heat = (r < p->heat_radius) ? p->heat_in : p->heat_out;
    double tx, ty;
    thermal_draw(p, s->i, step, stage + 16, heat, &tx, &ty);
    *fx += tx;
    *fy += ty;
}

/* TimeVaryingThermalForce: heatVal = heatValScale*t + heatValOffset
 * (TimeVaryingThermalForce.cpp:14-44), then ThermalForce's kick. */
static inline void f_thermal_tv(const or_params *p, const pstate *s, double t, uint64_t step, int stage,
                                double *fx, double *fy) {
    const double heat = p->heat_scale * t + p->heat_offset;
    double tx, ty;
    thermal_draw(p, s->i, step, stage + 32, heat, &tx, &ty);
    *fx += tx;
    *fy += ty;
}

/* ElectricForce::force (ElectricForce.cpp:48-62): F = q*E*exp(r/(-R))*(x, y) */
static inline void f_electric(const or_params *p, const pstate *s, double *fx, double *fy) {
    const double cV = s->q * p->electric;
    const double R = sqrt(s->x * s->x + s->y * s->y);
    const double eV = cV * exp(R / (p->electric_radius * (-1)));
    *fx += eV * s->x;
    *fy += eV * s->y;
}

/* GravitationalForce::force (GravitationalForce.cpp:46-50): Fy += m*g */
static inline void f_gravity(const or_params *p, const pstate *s, double *fy) {
    *fy += s->m * p->gravity;
}

/* VertElectricForce::force (VertElectricForce.cpp:47-53): Fy += q*E*exp(y/d) */
static inline void f_vert_electric(const or_params *p, const pstate *s, double *fy) {
    const double cV = s->q * p->vert_electric;
    *fy += cV * exp(s->y / p->vert_decay);
}

/* The forces the driver pushes before ShieldedCoulomb (driver.cpp:373-386):
 * Confinement, ConfinementVoid, Drag, Driving, Magnetic, RectConfinement,
 * Rotational. */
static void forces_before_pairs(const or_params *p, const pstate *s, double t, double *fx, double *fy) {
    const long long fl = p->flags;
    if (fl & OR_CONFINEMENT_FORCE) f_confinement(p, s, fx, fy);
    if (fl & OR_CONFINEMENT_VOID_FORCE) f_void(p, s, fx, fy);
    if (fl & OR_DRAG_FORCE) f_drag(-p->gamma, s, fx, fy);  /* dragConst = -gamma (DragForce.h:16-17) */
    if (fl & OR_DRIVING_FORCE) f_driving(p, s, t, fx);
    if (fl & OR_MAGNETIC_FORCE) f_magnetic(p, s, fx, fy);
    if (fl & OR_RECT_CONFINEMENT_FORCE) f_rect(p, s, fx, fy);
    if (fl & OR_ROTATIONAL_FORCE) f_rotational(p, s, fx, fy);
}

/* The forces pushed after it (driver.cpp:389-402): Thermal,
 * ThermalLocalized, TimeVaryingDrag, TimeVaryingThermal, Electric,
 * Gravitational, VertElectric. */
static void forces_after_pairs(const or_params *p, const pstate *s, double t, uint64_t step, int stage,
                               double *fx, double *fy) {
    const long long fl = p->flags;
    if (fl & OR_THERMAL_FORCE) {
        double tx, ty;
        or_thermal_one(p, s->i, step, stage, &tx, &ty);
        *fx += tx;
        *fy += ty;
    }
    if (fl & OR_THERMAL_LOCALIZED_FORCE) f_thermal_localized(p, s, step, stage, fx, fy);
    /* TimeVaryingDragForce: dragConst = -(scaleConst*t + offsetConst)
     * (TimeVaryingDragForce.cpp:14-38), then DragForce's force */
    if (fl & OR_TIME_VARYING_DRAG_FORCE) f_drag(-(p->drag_scale * t + p->drag_offset), s, fx, fy);
    if (fl & OR_TIME_VARYING_THERMAL_FORCE) f_thermal_tv(p, s, t, step, stage, fx, fy);
    if (fl & OR_ELECTRIC_FORCE) f_electric(p, s, fx, fy);
    if (fl & OR_GRAVITATIONAL_FORCE) f_gravity(p, s, fy);
    if (fl & OR_VERT_ELECTRIC_FORCE) f_vert_electric(p, s, fy);
}

static inline pstate particle(int i, const double *xs, const double *ys, const double *vxs,
                              const double *vys, const double *q, const double *m) {
    pstate s = {(uint32_t)i, xs[i], ys[i], vxs[i], vys[i], q[i], m[i]};
    return s;
}

/* ---------------------------------------------------------------------------
 * All forces of one RK stage.
 * ------------------------------------------------------------------------- */

void or_forces_rows(int n, const double *xs, const double *ys,
                    const double *vxs, const double *vys, const double *q,
                    const double *m, const or_params *p, uint64_t step,
                    int stage, double t, int nrows, const int *rows, double *fx,
                    double *fy, int nthreads) {
    const double C = or_coulomb();
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads > 0 ? nthreads : 1)
    for (int k = 0; k < nrows; k++) {
        const int i = rows[k];
        const pstate s = particle(i, xs, ys, vxs, vys, q, m);
        double sx = 0.0, sy = 0.0;
        forces_before_pairs(p, &s, t, &sx, &sy);
        if (p->flags & OR_SHIELDED_COULOMB_FORCE) {
            double px = 0.0, py = 0.0;
            for (int j = 0; j < n; j++) {
                if (j == i) continue;
                double ax, ay;
                /* the (i, i+1) pair of an even-aligned 2-block takes the
                 * intra-block form, every other pair the block form; a pair's
                 * value is the same from either side (qq and r are symmetric) */
                const int hit = ((j ^ 1) == i && (i | 1) < n)
                    ? pair_intra(xs[i] - xs[j], ys[i] - ys[j], q[i] * q[j], p->shielding, C, &ax, &ay)
                    : pair_block(xs[i] - xs[j], ys[i] - ys[j], q[i] * q[j], p->shielding, C, &ax, &ay);
                if (hit) { px += ax; py += ay; }
            }
            sx += px;
            sy += py;
        }
        forces_after_pairs(p, &s, t, step, stage, &sx, &sy);
        fx[k] = sx;
        fy[k] = sy;
    }
}

void or_forces(int n, const double *xs, const double *ys, const double *vxs,
               const double *vys, const double *q, const double *m,
               const or_params *p, uint64_t step, int stage, double t, double *fx,
               double *fy, int nthreads) {
    /* driver.cpp:372-402 push order; the pair force adds pair by pair into
     * the running sums (ShieldedCoulombForce.cpp:154-159, 193-198) */
    for (int i = 0; i < n; i++) {
        const pstate s = particle(i, xs, ys, vxs, vys, q, m);
        fx[i] = 0.0;
        fy[i] = 0.0;
        forces_before_pairs(p, &s, t, &fx[i], &fy[i]);
    }
    if (p->flags & OR_SHIELDED_COULOMB_FORCE) {
        if (nthreads == 1)
            or_shielded_coulomb(n, xs, ys, q, p->shielding, fx, fy);
        else
            or_shielded_coulomb_omp(n, xs, ys, q, p->shielding, fx, fy, nthreads);
    }
    for (int i = 0; i < n; i++) {
        const pstate s = particle(i, xs, ys, vxs, vys, q, m);
        forces_after_pairs(p, &s, t, step, stage, &fx[i], &fy[i]);
    }
}

/* ---------------------------------------------------------------------------
 * RK4.
 * ------------------------------------------------------------------------- */

/* Runge_Kutta4::da (Runge_Kutta4.cpp:147-151): (a1 + (2*(a2+a3) + a4)) / 6 */
static inline double rk_da(double a1, double a2, double a3, double a4) {
    return (a1 + ((a2 + a3) * 2.0 + a4)) / 6.0;
}

typedef struct rk_work {
    double *k[4], *l[4], *mm[4], *nn[4];
    double *xc, *yc, *vxc, *vyc, *fx, *fy;
    double *block;
} rk_work;

static int rk_work_alloc(rk_work *w, int n) {
    const size_t sz = (size_t)(n > 0 ? n : 1);
    w->block = (double *)calloc(sz * 22, sizeof(double));
    if (!w->block) return -1;
    double *b = w->block;
    for (int s = 0; s < 4; s++) {
        w->k[s] = b; b += sz;
        w->l[s] = b; b += sz;
        w->mm[s] = b; b += sz;
        w->nn[s] = b; b += sz;
    }
    w->xc = b; b += sz;
    w->yc = b; b += sz;
    w->vxc = b; b += sz;
    w->vyc = b; b += sz;
    w->fx = b; b += sz;
    w->fy = b;
    return 0;
}

/* One RK4 step with a given dt (Runge_Kutta4.cpp:26-135 after line 25). */
static void rk4_one_step(int n, double *x, double *y, double *vx, double *vy,
                         const double *q, const double *m, const or_params *p,
                         double t, double dt, uint64_t step, int nthreads, rk_work *w) {
    for (int s = 0; s < 4; s++) {
        /* force times t, t + dt/2.0, t + dt/2.0, t + dt (Runge_Kutta4.cpp:30-88) */
        const double ts = (s == 0) ? t : (s == 3) ? t + dt : t + dt / 2.0;
        const double *xs, *ys, *vxs, *vys;
        if (s == 0) {
            /* operation1 is a no-op (CacheOperator.cpp:18-20): stage 1 reads x, Vx */
            xs = x; ys = y; vxs = vx; vys = vy;
        } else {
            /* operation2/3: cache = 0.5*tidbit + base (CacheOperator.cpp:28-56,
             * fmadd_pd is mul then add under SSE4.2, VectorCompatibility.h:99-105);
             * operation4: cache = base + tidbit (CacheOperator.cpp:64-73) */
            const double *kp = w->k[s - 1], *lp = w->l[s - 1];
            const double *mp = w->mm[s - 1], *np = w->nn[s - 1];
            for (int i = 0; i < n; i++) {
                if (s < 3) {
                    w->xc[i] = 0.5 * lp[i] + x[i];
                    w->yc[i] = 0.5 * np[i] + y[i];
                    w->vxc[i] = 0.5 * kp[i] + vx[i];
                    w->vyc[i] = 0.5 * mp[i] + vy[i];
                } else {
                    w->xc[i] = x[i] + lp[i];
                    w->yc[i] = y[i] + np[i];
                    w->vxc[i] = vx[i] + kp[i];
                    w->vyc[i] = vy[i] + mp[i];
                }
            }
            xs = w->xc; ys = w->yc; vxs = w->vxc; vys = w->vyc;
        }
        or_forces(n, xs, ys, vxs, vys, q, m, p, step, s + 1, ts, w->fx, w->fy, nthreads);
        /* stage kernels (Runge_Kutta4.cpp:32-47 etc.):
         * k = (dt*Fx)/m, l = dt*Vx_stage, m = (dt*Fy)/m, n = dt*Vy_stage */
        for (int i = 0; i < n; i++) {
            w->k[s][i] = (dt * w->fx[i]) / m[i];
            w->l[s][i] = dt * vxs[i];
            w->mm[s][i] = (dt * w->fy[i]) / m[i];
            w->nn[s][i] = dt * vys[i];
        }
    }
    /* Runge_Kutta4.cpp:107-133 */
    for (int i = 0; i < n; i++) {
        vx[i] += rk_da(w->k[0][i], w->k[1][i], w->k[2][i], w->k[3][i]);
        x[i] += rk_da(w->l[0][i], w->l[1][i], w->l[2][i], w->l[3][i]);
        vy[i] += rk_da(w->mm[0][i], w->mm[1][i], w->mm[2][i], w->mm[3][i]);
        y[i] += rk_da(w->nn[0][i], w->nn[1][i], w->nn[2][i], w->nn[3][i]);
    }
}

void or_rk4_fixed(int n, double *x, double *y, double *vx, double *vy,
                  const double *q, const double *m, const or_params *p,
                  double t0, double dt, int nsteps, uint64_t step0, int nthreads) {
    rk_work w;
    if (rk_work_alloc(&w, n)) return;
    double t = t0;
    for (int s = 0; s < nsteps; s++) {
        rk4_one_step(n, x, y, vx, vy, q, m, p, t, dt, step0 + (uint64_t)s, nthreads, &w);
        t += dt;  /* Runge_Kutta4.cpp:135 */
    }
    free(w.block);
}

/* ---------------------------------------------------------------------------
 * Adaptive time step.
 * ------------------------------------------------------------------------- */

static inline float sep_r2(float ax, float ay, float bx, float by) {
    const float sx = ax - bx, sy = ay - by;
    return sx * sx + sy * sy;
}

/* Integrator::modifyTimeStep (Integrator.cpp:90-131).  loadFloatVector
 * (Integrator.cpp:162-169) puts x[o+3-L] in lane L; the two hsub tests
 * (lines 96-104) cover all 6 pairs inside a 4-block; between 4-blocks the
 * shuffles (lines 112-129; _MM_SHUFFLE(3,2,1,0) is the identity) pair outer
 * element k with inner element (k - d) mod 4 for d = 0, 1, 2 only. */
float or_checked_min_dist(int n, const double *x, const double *y) {
    float best = INFINITY;
    for (int o = 0; o + 3 < n; o += 4) {
        float ox[4], oy[4];
        for (int k = 0; k < 4; k++) { ox[k] = (float)x[o + k]; oy[k] = (float)y[o + k]; }
        static const int intra[6][2] = {{0, 1}, {2, 3}, {0, 3}, {1, 2}, {1, 3}, {0, 2}};
        for (int t = 0; t < 6; t++) {
            const float r2 = sep_r2(ox[intra[t][0]], oy[intra[t][0]], ox[intra[t][1]], oy[intra[t][1]]);
            if (r2 < best) best = r2;
        }
        for (int in = o + 4; in + 3 < n; in += 4) {
            float ix[4], iy[4];
            for (int k = 0; k < 4; k++) { ix[k] = (float)x[in + k]; iy[k] = (float)y[in + k]; }
            for (int k = 0; k < 4; k++)
                for (int d = 0; d < 3; d++) {
                    const int mi = (k - d + 4) & 3;
                    const float r2 = sep_r2(ox[k], oy[k], ix[mi], iy[mi]);
                    if (r2 < best) best = r2;
                }
        }
    }
    return sqrtf(best);
}

double or_modify_timestep(int n, const double *x, const double *y, float dist,
                          double dt) {
    const float dmin = or_checked_min_dist(n, x, y);
    if (!(dmin > 0.0f)) return -1.0;
    /* tryToReduceTimeStep (Integrator.cpp:144-155): while within distance,
     * distance /= 10.0f, time /= 10.0f (a double divided by 10.0). */
    while (dmin <= dist) {
        dist /= 10.0f;
        dt /= 10.0f;
    }
    return dt;
}

int or_rk4_move_particles(int n, double *x, double *y, double *vx, double *vy,
                          const double *q, const double *m, const or_params *p,
                          double init_dt, double *t_inout, double end_time,
                          uint64_t step0, int nthreads) {
    rk_work w;
    if (rk_work_alloc(&w, n)) return -1;
    int steps = 0;
    double t = *t_inout;
    /* Runge_Kutta4::moveParticles (Runge_Kutta4.cpp:24-136) */
    while (t < end_time) {
        const double dt = or_modify_timestep(n, x, y, 1.0e-4f, init_dt);
        if (dt < 0.0) break;
        rk4_one_step(n, x, y, vx, vy, q, m, p, t, dt, step0 + (uint64_t)steps, nthreads, &w);
        t += dt;
        steps++;
    }
    *t_inout = t;
    free(w.block);
    return steps;
}

/* ---------------------------------------------------------------------------
 * RK2 (the midpoint method of Runge_Kutta2.cpp).
 * ------------------------------------------------------------------------- */

/* Runge_Kutta2::moveParticles one step (Runge_Kutta2.cpp:24-76): stage 1 at
 * (x, Vx, t), k1 = (dt*F)/m, l1 = dt*Vx; CacheOperator::operation2 cache =
 * 0.5*tidbit + base; stage 2 at the cache and t + dt/2.0; then
 * Vx += k2, x += l2, Vy += m2, y += n2. */
static void rk2_one_step(int n, double *x, double *y, double *vx, double *vy,
                         const double *q, const double *m, const or_params *p,
                         double t, double dt, uint64_t step, int nthreads, rk_work *w) {
    or_forces(n, x, y, vx, vy, q, m, p, step, 1, t, w->fx, w->fy, nthreads);
    for (int i = 0; i < n; i++) {
        w->k[0][i] = (dt * w->fx[i]) / m[i];
        w->l[0][i] = dt * vx[i];
        w->mm[0][i] = (dt * w->fy[i]) / m[i];
        w->nn[0][i] = dt * vy[i];
    }
    for (int i = 0; i < n; i++) {
        w->xc[i] = 0.5 * w->l[0][i] + x[i];
        w->yc[i] = 0.5 * w->nn[0][i] + y[i];
        w->vxc[i] = 0.5 * w->k[0][i] + vx[i];
        w->vyc[i] = 0.5 * w->mm[0][i] + vy[i];
    }
    or_forces(n, w->xc, w->yc, w->vxc, w->vyc, q, m, p, step, 2, t + dt / 2.0, w->fx, w->fy, nthreads);
    for (int i = 0; i < n; i++) {
        const double k2 = (dt * w->fx[i]) / m[i];
        const double l2 = dt * w->vxc[i];
        const double m2 = (dt * w->fy[i]) / m[i];
        const double n2 = dt * w->vyc[i];
        vx[i] += k2;
        x[i] += l2;
        vy[i] += m2;
        y[i] += n2;
    }
}

void or_rk2_fixed(int n, double *x, double *y, double *vx, double *vy,
                  const double *q, const double *m, const or_params *p,
                  double t0, double dt, int nsteps, uint64_t step0, int nthreads) {
    rk_work w;
    if (rk_work_alloc(&w, n)) return;
    double t = t0;
    for (int s = 0; s < nsteps; s++) {
        rk2_one_step(n, x, y, vx, vy, q, m, p, t, dt, step0 + (uint64_t)s, nthreads, &w);
        t += dt;  /* Runge_Kutta2.cpp:76 */
    }
    free(w.block);
}

int or_rk2_move_particles(int n, double *x, double *y, double *vx, double *vy,
                          const double *q, const double *m, const or_params *p,
                          double init_dt, double *t_inout, double end_time,
                          uint64_t step0, int nthreads) {
    rk_work w;
    if (rk_work_alloc(&w, n)) return -1;
    int steps = 0;
    double t = *t_inout;
    /* Runge_Kutta2::moveParticles (Runge_Kutta2.cpp:23-78) */
    while (t < end_time) {
        const double dt = or_modify_timestep(n, x, y, 1.0e-4f, init_dt);
        if (dt < 0.0) break;
        rk2_one_step(n, x, y, vx, vy, q, m, p, t, dt, step0 + (uint64_t)steps, nthreads, &w);
        t += dt;
        steps++;
    }
    *t_inout = t;
    free(w.block);
    return steps;
}

/* ---------------------------------------------------------------------------
 * Diagnostics (no reference counterpart; FP64 definitions of the energies
 * whose forces the reference integrates).
 * ------------------------------------------------------------------------- */

void or_diagnostics(int n, const double *x, const double *y, const double *vx,
                    const double *vy, const double *q, const double *m,
                    const or_params *p, double out[5]) {
    const double C = or_coulomb();
    double ke = 0.0, pe = 0.0, pc = 0.0, px = 0.0, py = 0.0;
    for (int i = 0; i < n; i++) {
        ke += 0.5 * m[i] * (vx[i] * vx[i] + vy[i] * vy[i]);
        px += m[i] * vx[i];
        py += m[i] * vy[i];
        /* F = q*k*x  =>  U = -q*k*x^2/2 */
        if (p->flags & OR_CONFINEMENT_FORCE)
            pc += -0.5 * q[i] * p->confine * (x[i] * x[i] + y[i] * y[i]);
        if (p->flags & OR_RECT_CONFINEMENT_FORCE)
            pc += -0.5 * q[i] * (p->confine_x * x[i] * x[i] + p->confine_y * y[i] * y[i]);
    }
    if (p->flags & OR_SHIELDED_COULOMB_FORCE) {
        for (int i = 0; i < n; i++)
            for (int j = i + 1; j < n; j++) {
                const double dx = x[i] - x[j], dy = y[i] - y[j];
                const double r = sqrt(dx * dx + dy * dy);
                const double a = r * p->shielding;
                if (a < 10.0) pe += C * q[i] * q[j] * exp(-a) / r;
            }
    }
    out[0] = ke; out[1] = pe; out[2] = pc; out[3] = px; out[4] = py;
}
