/*
 * demon_oracle.h -- CPU oracle for the DEMON RK4 / shielded-Coulomb hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (AU-PSL/demon_simulation_code), used by tests/, by the smoke check
 * and by bench.py's CPU-baseline leg as the checker.  The product library
 * (demon_simulation_code_gb300, libdemon_gb300.so) never links or calls it.
 *
 * Parity of this restatement is pinned against the reference itself: the
 * reference's own sources are compiled (oracle/Makefile -> oracle/_ref) and
 * tests/golden/make_golden.py records their outputs as fixtures; the
 * restatement must reproduce them (bit-exact for the single-threaded pair
 * order, 1e-14 relative for trajectories).
 *
 * All functions are FP64 and take structure-of-arrays double buffers, like
 * the reference's Cloud (Cloud.h:21-29).
 */
#ifndef DEMON_ORACLE_H
#define DEMON_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Force flag bits: same values as the reference's ForceFlag (Force.h:75-91). */
#define OR_CONFINEMENT_FORCE       1LL
#define OR_DRAG_FORCE              2LL
#define OR_SHIELDED_COULOMB_FORCE  4LL
#define OR_GRAVITATIONAL_FORCE     8LL
#define OR_THERMAL_FORCE           16LL
#define OR_THERMAL_LOCALIZED_FORCE 32LL
#define OR_DRIVING_FORCE           64LL
#define OR_ROTATIONAL_FORCE        128LL
#define OR_TIME_VARYING_DRAG_FORCE 256LL
#define OR_TIME_VARYING_THERMAL_FORCE 512LL
#define OR_MAGNETIC_FORCE          1024LL
#define OR_CONFINEMENT_VOID_FORCE  2048LL
#define OR_ELECTRIC_FORCE          4096LL
#define OR_RECT_CONFINEMENT_FORCE  8192LL
#define OR_VERT_ELECTRIC_FORCE     16384LL

/* Parameters of the forces.  Field layout is identical to dm_force_params
 * in include/demon_gb300.h, which documents each field. */
typedef struct or_params {
    long long flags;        /* ForceFlag bitmask */
    double shielding;       /* ShieldedCoulombForce::shielding, kappa [1/m] */
    double confine;         /* ConfinementForce::confine [V/m^2] */
    double confine_x;       /* RectConfinementForce::confineX [V/m^2] */
    double confine_y;       /* RectConfinementForce::confineY [V/m^2] */
    double gamma;           /* DragForce gamma [1/s]; dragConst = -gamma */
    double heat;            /* ThermalForce heatVal [N] (mode 0) or sigma [N] (mode 1) */
    int thermal_mode;       /* 0: heat*U(0,1)*(cos,sin)(U(0,2pi)); 1: N(0,heat^2) per axis */
    int reserved;
    uint64_t seed;          /* counter-based RNG key */
    /* the reference's other per-particle forces (see dm_force_params) */
    double void_decay, drive_const, drive_amplitude, drive_shift, magnetic, rot_rmin, rot_rmax, rot_const;
    double heat_in, heat_out, heat_radius, drag_scale, drag_offset, heat_scale, heat_offset;
    double electric, electric_radius, gravity, vert_electric, vert_decay;
} or_params;

/* Coulomb constant 1/(4 pi eps0) with eps0 = 8.8541878e-12
 * (ShieldedCoulombForce.cpp:21, Cloud.cpp:15-16). */
double or_coulomb(void);

/* ShieldedCoulombForce::force1 (ShieldedCoulombForce.cpp:37-237), serial, in
 * the reference's own visiting and accumulation order: ADDS into fx, fy.
 * Even n follows the reference bit for bit; odd n (which the reference does
 * not accept) adds the last particle with the same pair formula. */
void or_shielded_coulomb(int n, const double *x, const double *y,
                         const double *q, double kappa,
                         double *fx, double *fy);

/* The same algorithm parallelised the way the reference is (OpenMP dynamic
 * over 2-particle i blocks, one lock per 2-particle block, Parallel.h:14-46,
 * ShieldedCoulombForce.cpp:24-29,154-197).  Summation order depends on thread
 * timing, exactly as in the reference.  Used for CPU-baseline timing. */
void or_shielded_coulomb_omp(int n, const double *x, const double *y,
                             const double *q, double kappa,
                             double *fx, double *fy, int nthreads);

/* Counter-based thermal kick for particle i at (step, stage): writes the
 * force (not +=).  Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) keyed by
 * seed, counter (i, step lo, step hi, stage); two 24-bit uniforms and FP32
 * Box-Muller arithmetic shared bit for bit with the CUDA path; mode 0 is
 * the reference's form (ThermalForce.cpp:118-140), mode 1 Box-Muller. */
void or_thermal_one(const or_params *p, uint32_t i, uint64_t step, int stage,
                    double *tx, double *ty);

/* Philox4x32-10 block (exposed for known-answer tests). */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Sum of all enabled forces at the given stage positions/velocities and
 * force time t, in the reference driver's force order (driver.cpp:372-402):
 * Confinement, ConfinementVoid, Drag, Driving, Magnetic, RectConfinement,
 * Rotational, ShieldedCoulomb, Thermal, ThermalLocalized, TimeVaryingDrag,
 * TimeVaryingThermal, Electric, Gravitational, VertElectric.  fx, fy are
 * overwritten (the reference zeroes forces after each stage,
 * Runge_Kutta4.cpp:45-46).  The three thermal forces draw counter-based
 * kicks (or_thermal_one) on streams stage, stage + 16 and stage + 32. */
void or_forces(int n, const double *xs, const double *ys,
               const double *vxs, const double *vys,
               const double *q, const double *m, const or_params *p,
               uint64_t step, int stage, double t, double *fx, double *fy, int nthreads);

/* The same total force for selected particles only (fx[k], fy[k] for
 * particle rows[k]), each row's pair sum in index order j = 0..n-1 with the
 * reference's pair formulas (ShieldedCoulombForce.cpp:138-159 for the
 * particle's 2-block partner, :172-237 otherwise).  Pair values are those of
 * or_forces; only the summation order differs.  For spot checks at sizes
 * where the full O(N^2) pass is too slow on the CPU. */
void or_forces_rows(int n, const double *xs, const double *ys,
                    const double *vxs, const double *vys, const double *q,
                    const double *m, const or_params *p, uint64_t step,
                    int stage, double t, int nrows, const int *rows, double *fx,
                    double *fy, int nthreads);

/* Runge_Kutta4::moveParticles (Runge_Kutta4.cpp:23-137) with CacheOperator
 * (CacheOperator.cpp:18-73) and a FIXED dt (line 25's modifyTimeStep left out),
 * for an explicit step count from time t0 (stage force times t, t + dt/2,
 * t + dt/2, t + dt; t += dt per step).  x, y, vx, vy are updated in place.
 * step0 is the RNG step index of the first step. */
void or_rk4_fixed(int n, double *x, double *y, double *vx, double *vy,
                  const double *q, const double *m, const or_params *p,
                  double t0, double dt, int nsteps, uint64_t step0, int nthreads);

/* Integrator::modifyTimeStep (Integrator.cpp:68-134): the FP32 distance test
 * over exactly the pairs the reference checks, returning the reduced dt.
 * n must be a multiple of 4.  Returns a negative value if a checked pair has
 * zero separation (the reference loops forever there). */
double or_modify_timestep(int n, const double *x, const double *y,
                          float dist, double dt);

/* Minimum FP32 separation over the pairs modifyTimeStep checks. */
float or_checked_min_dist(int n, const double *x, const double *y);

/* Runge_Kutta4::moveParticles(endTime) including the adaptive dt, from
 * *t_inout until *t_inout >= end_time.  Returns the number of steps taken. */
int or_rk4_move_particles(int n, double *x, double *y, double *vx, double *vy,
                          const double *q, const double *m, const or_params *p,
                          double init_dt, double *t_inout, double end_time,
                          uint64_t step0, int nthreads);

/* Runge_Kutta2::moveParticles (Runge_Kutta2.cpp:23-78), the midpoint
 * method over the same forces and CacheOperator::operation2: fixed dt for an
 * explicit step count from t0 (force times t, t + dt/2), and the adaptive
 * form from *t_inout until end_time (returns the steps taken). */
void or_rk2_fixed(int n, double *x, double *y, double *vx, double *vy,
                  const double *q, const double *m, const or_params *p,
                  double t0, double dt, int nsteps, uint64_t step0, int nthreads);
int or_rk2_move_particles(int n, double *x, double *y, double *vx, double *vy,
                          const double *q, const double *m, const or_params *p,
                          double init_dt, double *t_inout, double end_time,
                          uint64_t step0, int nthreads);

/* FP64 diagnostics: out[0]=kinetic, out[1]=Yukawa potential (pairs with
 * kappa*r < 10), out[2]=confinement potential, out[3]=px, out[4]=py. */
void or_diagnostics(int n, const double *x, const double *y,
                    const double *vx, const double *vy,
                    const double *q, const double *m, const or_params *p,
                    double out[5]);

#ifdef __cplusplus
}
#endif
#endif /* DEMON_ORACLE_H */
