/*
 * ref_harness.cpp -- C ABI around the reference's OWN classes (test
 * infrastructure only).  Linked with the reference's unmodified library
 * sources by oracle/Makefile into oracle/_ref/libdemon_ref*.so; this file is
 * the only project code in those libraries.  Inputs are set directly into the
 * reference Cloud's arrays (the reference's initializeGrid/RandomNumbers are
 * time-seeded and are not used) and forces are zeroed first (Cloud.cpp:31
 * leaves forceX/forceY uninitialised).
 */
#include "Cloud.h"
#include "CacheOperator.h"
#include "ConfinementForce.h"
#include "ConfinementForceVoid.h"
#include "DragForce.h"
#include "DrivingForce.h"
#include "ElectricForce.h"
#include "GravitationalForce.h"
#include "MagneticForce.h"
#include "RectConfinementForce.h"
#include "RotationalForce.h"
#include "Runge_Kutta2.h"
#include "Runge_Kutta4.h"
#include "ShieldedCoulombForce.h"
#include "ThermalForce.h"
#include "ThermalForceLocalized.h"
#include "TimeVaryingDragForce.h"
#include "TimeVaryingThermalForce.h"
#include "VertElectricForce.h"

#include <cmath>
#include <cstring>
#include <vector>

/* Statics the reference defines in driver.cpp:122-127. */
double Cloud::interParticleSpacing = 0.003;
double Cloud::dustParticleMassDensity = 2200;
double Cloud::justX = 0;
double Cloud::justY = 0;
double Cloud::velX = 0.0;
double Cloud::velY = 0.0;

namespace {

struct Params {               /* same layout as or_params / dm_force_params */
    long long flags;
    double shielding, confine, confine_x, confine_y, gamma, heat;
    int thermal_mode, reserved;
    unsigned long long seed;
    double void_decay, drive_const, drive_amplitude, drive_shift, magnetic, rot_rmin, rot_rmax, rot_const;
    double heat_in, heat_out, heat_radius, drag_scale, drag_offset, heat_scale, heat_offset;
    double electric, electric_radius, gravity, vert_electric, vert_decay;
};

void load(Cloud &c, const double *x, const double *y, const double *vx,
          const double *vy, const double *q, const double *m) {
    const size_t n = (size_t)c.n;
    std::memcpy(c.x, x, n * sizeof(double));
    std::memcpy(c.y, y, n * sizeof(double));
    std::memcpy(c.Vx, vx, n * sizeof(double));
    std::memcpy(c.Vy, vy, n * sizeof(double));
    std::memcpy(c.charge, q, n * sizeof(double));
    std::memcpy(c.mass, m, n * sizeof(double));
    std::memset(c.forceX, 0, n * sizeof(double));
    std::memset(c.forceY, 0, n * sizeof(double));
}

/* Force construction in driver.cpp's order and with its constructor
 * arguments (driver.cpp:372-402).  The three thermal forces draw from the
 * Cloud's RandomNumbers, which is seeded from the clock
 * (RandomNumbers.cpp:19-21), so they are built only when asked for. */
void make_forces(Cloud *c, const Params *p, ForceArray &fa, bool thermal = false) {
    const long long f = p->flags;
    if (f & ConfinementForceFlag) fa.push_back(new ConfinementForce(c, p->confine));
    if (f & ConfinementForceVoidFlag) fa.push_back(new ConfinementForceVoid(c, p->confine, p->void_decay));
    if (f & DragForceFlag) fa.push_back(new DragForce(c, p->gamma));
    if (f & DrivingForceFlag)
        fa.push_back(new DrivingForce(c, p->drive_const, p->drive_amplitude, p->drive_shift));
    if (f & MagneticForceFlag) fa.push_back(new MagneticForce(c, p->magnetic));
    if (f & RectConfinementForceFlag)
        fa.push_back(new RectConfinementForce(c, p->confine_x, p->confine_y));
    if (f & RotationalForceFlag) fa.push_back(new RotationalForce(c, p->rot_rmin, p->rot_rmax, p->rot_const));
    if (f & ShieldedCoulombForceFlag) fa.push_back(new ShieldedCoulombForce(c, p->shielding));
    if (thermal && (f & ThermalForceFlag)) fa.push_back(new ThermalForce(c, p->heat));
    if (thermal && (f & ThermalForceLocalizedFlag))
        fa.push_back(new ThermalForceLocalized(c, p->heat_in, p->heat_out, p->heat_radius));
    if (f & TimeVaryingDragForceFlag) fa.push_back(new TimeVaryingDragForce(c, p->drag_scale, p->drag_offset));
    if (thermal && (f & TimeVaryingThermalForceFlag))
        fa.push_back(new TimeVaryingThermalForce(c, p->heat_scale, p->heat_offset));
    if (f & ElectricForceFlag) fa.push_back(new ElectricForce(c, p->electric, p->electric_radius));
    if (f & GravitationalForceFlag) fa.push_back(new GravitationalForce(c, p->gravity));
    if (f & VertElectricForceFlag) fa.push_back(new VertElectricForce(c, p->vert_electric, p->vert_decay));
}

void free_forces(ForceArray &fa) {
    for (Force *f : fa) delete f;
    fa.clear();
}

}  // namespace

extern "C" {

/* ShieldedCoulombForce::force1 alone; fx, fy receive the force. */
int ref_shielded_coulomb(int n, const double *x, const double *y, const double *q,
                         double kappa, double *fx, double *fy) {
    if (n < 2 || (n & 1)) return -1;
    Cloud c(n);
    std::vector<double> zeros((size_t)n, 0.0);
    load(c, x, y, zeros.data(), zeros.data(), q, zeros.data());
    ShieldedCoulombForce F(&c, kappa);
    F.force1(0.0);
    std::memcpy(fx, c.forceX, (size_t)n * sizeof(double));
    std::memcpy(fy, c.forceY, (size_t)n * sizeof(double));
    return 0;
}

/* Every flagged force's force1(t) in driver order, summed as the reference
 * sums them into forceX/forceY; thermal != 0 includes the thermal forces. */
int ref_forces_at(int n, const double *x, const double *y, const double *vx,
                  const double *vy, const double *q, const double *m,
                  const void *params, double t, int thermal, double *fx, double *fy) {
    if (n < 2 || (n & 1)) return -1;
    const Params *p = (const Params *)params;
    Cloud c(n);
    load(c, x, y, vx, vy, q, m);
    ForceArray fa;
    make_forces(&c, p, fa, thermal != 0);
    for (Force *f : fa) f->force1(t);
    std::memcpy(fx, c.forceX, (size_t)n * sizeof(double));
    std::memcpy(fy, c.forceY, (size_t)n * sizeof(double));
    free_forces(fa);
    return 0;
}

/* The reference's own Runge_Kutta4::moveParticles(endTime), adaptive dt
 * included (Runge_Kutta4.cpp:23-137).  Returns the number of steps taken
 * and the final time. */
int ref_rk4_move_particles(int n, double *x, double *y, double *vx, double *vy,
                           const double *q, const double *m, const void *params,
                           double dt, double t0, double end_time, double *t_out) {
    if (n < 4 || (n & 3)) return -1;
    const Params *p = (const Params *)params;
    Cloud c(n);
    load(c, x, y, vx, vy, q, m);
    ForceArray fa;
    make_forces(&c, p, fa);
    int steps = 0;
    {
        Runge_Kutta4 I(&c, fa, dt, t0);
        /* step-by-step so the step count is observable; each call advances
         * while currentTime < target, i.e. exactly one step */
        while (I.currentTime < end_time) {
            I.moveParticles(std::nextafter(I.currentTime, HUGE_VAL));
            steps++;
        }
        if (t_out) *t_out = I.currentTime;
    }
    const size_t bytes = (size_t)n * sizeof(double);
    std::memcpy(x, c.x, bytes);
    std::memcpy(y, c.y, bytes);
    std::memcpy(vx, c.Vx, bytes);
    std::memcpy(vy, c.Vy, bytes);
    free_forces(fa);
    return steps;
}

/* The reference's own Runge_Kutta2::moveParticles(endTime), adaptive dt
 * included (Runge_Kutta2.cpp:23-78), one step per call as above. */
int ref_rk2_move_particles(int n, double *x, double *y, double *vx, double *vy,
                           const double *q, const double *m, const void *params,
                           double dt, double t0, double end_time, double *t_out) {
    if (n < 4 || (n & 3)) return -1;
    const Params *p = (const Params *)params;
    Cloud c(n);
    load(c, x, y, vx, vy, q, m);
    ForceArray fa;
    make_forces(&c, p, fa);
    int steps = 0;
    {
        Runge_Kutta2 I(&c, fa, dt, t0);
        while (I.currentTime < end_time) {
            I.moveParticles(std::nextafter(I.currentTime, HUGE_VAL));
            steps++;
        }
        if (t_out) *t_out = I.currentTime;
    }
    const size_t bytes = (size_t)n * sizeof(double);
    std::memcpy(x, c.x, bytes);
    std::memcpy(y, c.y, bytes);
    std::memcpy(vx, c.Vx, bytes);
    std::memcpy(vy, c.Vy, bytes);
    free_forces(fa);
    return steps;
}

/* Fixed-dt RK4 for an explicit step count from time t0: the reference's
 * CacheOperator and Force objects drive every stage at the reference's stage
 * times; only the stage bookkeeping of Runge_Kutta4.cpp:26-135 (without line
 * 25's modifyTimeStep) is restated. */
int ref_rk4_fixed(int n, double *x, double *y, double *vx, double *vy,
                  const double *q, const double *m, const void *params,
                  double t0, double dt, int nsteps) {
    if (n < 2 || (n & 1)) return -1;
    const Params *p = (const Params *)params;
    Cloud c(n);
    load(c, x, y, vx, vy, q, m);
    ForceArray fa;
    make_forces(&c, p, fa);
    CacheOperator op(&c);
    double *K[4] = {c.k1, c.k2, c.k3, c.k4}, *L[4] = {c.l1, c.l2, c.l3, c.l4};
    double *M[4] = {c.m1, c.m2, c.m3, c.m4}, *NN[4] = {c.n1, c.n2, c.n3, c.n4};
    double t = t0;
    for (int s = 0; s < nsteps; s++) {
        for (int st = 0; st < 4; st++) {
            switch (st) {  // Runge_Kutta4.cpp:30-31, 49-50, 68-69, 87-88
                case 0: op.operation1(t); for (Force *f : fa) f->force1(t); break;
                case 1: op.operation2(t + dt / 2.0); for (Force *f : fa) f->force2(t + dt / 2.0); break;
                case 2: op.operation3(t + dt / 2.0); for (Force *f : fa) f->force3(t + dt / 2.0); break;
                default: op.operation4(t + dt); for (Force *f : fa) f->force4(t + dt); break;
            }
            for (cloud_index i = 0; i < (cloud_index)n; i += DOUBLE_STRIDE) {
                const doubleV vm = load_pd(c.mass + i);
                const doubleV vdt = set1_pd(dt);
                doubleV vxs, vys;
                switch (st) {
                    case 0: vxs = c.getVx1_pd(i); vys = c.getVy1_pd(i); break;
                    case 1: vxs = c.getVx2_pd(i); vys = c.getVy2_pd(i); break;
                    case 2: vxs = c.getVx3_pd(i); vys = c.getVy3_pd(i); break;
                    default: vxs = c.getVx4_pd(i); vys = c.getVy4_pd(i); break;
                }
                store_pd(K[st] + i, div_pd(mul_pd(vdt, load_pd(c.forceX + i)), vm));
                store_pd(L[st] + i, mul_pd(vdt, vxs));
                store_pd(M[st] + i, div_pd(mul_pd(vdt, load_pd(c.forceY + i)), vm));
                store_pd(NN[st] + i, mul_pd(vdt, vys));
                store_pd(c.forceX + i, set0_pd());
                store_pd(c.forceY + i, set0_pd());
            }
        }
        for (cloud_index i = 0; i < (cloud_index)n; i++) {
            c.Vx[i] += (c.k1[i] + ((c.k2[i] + c.k3[i]) * 2.0 + c.k4[i])) / 6.0;
            c.x[i] += (c.l1[i] + ((c.l2[i] + c.l3[i]) * 2.0 + c.l4[i])) / 6.0;
            c.Vy[i] += (c.m1[i] + ((c.m2[i] + c.m3[i]) * 2.0 + c.m4[i])) / 6.0;
            c.y[i] += (c.n1[i] + ((c.n2[i] + c.n3[i]) * 2.0 + c.n4[i])) / 6.0;
        }
        t += dt;  // Runge_Kutta4.cpp:135
    }
    const size_t bytes = (size_t)n * sizeof(double);
    std::memcpy(x, c.x, bytes);
    std::memcpy(y, c.y, bytes);
    std::memcpy(vx, c.Vx, bytes);
    std::memcpy(vy, c.Vy, bytes);
    free_forces(fa);
    return nsteps;
}

}  // extern "C"
