/*
 * demon_gb300.h -- C ABI of the GB300 (sm_103a) implementation of DEMON's
 * RK4 / shielded-Coulomb hot path.
 *
 * The reference (AU-PSL/demon_simulation_code) has no C ABI: its hot path is
 * a set of C++ virtual classes.  Each entry point below replaces one piece of
 * that class API; the comment on each names the reference interface it
 * stands in for (file:line).  The C++ classes in
 * demon_simulation_code_gb300/host/ re-expose the reference's class names
 * on top of these calls.
 *
 * Conventions
 *  - Every call returns an int status: 0 (DM_OK) on success, a DM_ERR_* code
 *    otherwise; dm_last_error() returns the message.  No call exits the
 *    process or throws across the ABI (the reference exit(1)s on FITS errors,
 *    driver.cpp:202-213).
 *  - Plain pointers and sizes only.  "host" arrays are ordinary CPU memory
 *    (pinned memory makes copies faster but is not required); "device"
 *    arrays are CUDA device pointers on the context's device.
 *  - One context drives one GPU through one CUDA stream.  Calls on one
 *    context are not thread-safe; use one context per host thread.
 *  - All particle arrays are FP64 structure-of-arrays, like the reference's
 *    Cloud (Cloud.h:21-29).  Units: m, m/s, C, kg, N, s.
 */
#ifndef DEMON_GB300_H
#define DEMON_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DM_ABI_VERSION 1

typedef enum dm_status {
    DM_OK = 0,
    DM_ERR_ARG = 1,         /* invalid argument (null pointer, bad size, bad enum) */
    DM_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    DM_ERR_NOMEM = 3,       /* device or host allocation failed */
    DM_ERR_STATE = 4,       /* object in the wrong state for this call */
    DM_ERR_NUMERIC = 5,     /* non-finite result detected on the device */
    DM_ERR_UNSUPPORTED = 6  /* feature not available on this device/build */
} dm_status;

/* Pair-force arithmetic.  The RK4 state update is FP64 in both modes. */
typedef enum dm_precision {
    DM_FP64 = 0,   /* all pair arithmetic in FP64 */
    DM_FP32C = 1   /* FP32 pair arithmetic, two-float position differences,
                      Kahan-compensated per-particle sums, FP64 cutoff
                      decision for borderline pairs */
} dm_precision;

/* Force flag bits: identical values to the reference's ForceFlag enum
 * (Force.h:75-91). */
#define DM_CONFINEMENT_FORCE       1LL
#define DM_DRAG_FORCE              2LL
#define DM_SHIELDED_COULOMB_FORCE  4LL
#define DM_GRAVITATIONAL_FORCE     8LL
#define DM_THERMAL_FORCE           16LL
#define DM_THERMAL_LOCALIZED_FORCE 32LL
#define DM_DRIVING_FORCE           64LL
#define DM_ROTATIONAL_FORCE        128LL
#define DM_TIME_VARYING_DRAG_FORCE 256LL
#define DM_TIME_VARYING_THERMAL_FORCE 512LL
#define DM_MAGNETIC_FORCE          1024LL
#define DM_CONFINEMENT_VOID_FORCE  2048LL
#define DM_ELECTRIC_FORCE          4096LL
#define DM_RECT_CONFINEMENT_FORCE  8192LL
#define DM_VERT_ELECTRIC_FORCE     16384LL

/* Parameters of the forces; one struct replaces the constructor
 * arguments of ConfinementForce (ConfinementForce.h:15-16),
 * RectConfinementForce (RectConfinementForce.h:18-19), DragForce
 * (DragForce.h:16-17), ShieldedCoulombForce (ShieldedCoulombForce.h:17) and
 * ThermalForce (ThermalForce.h:16). */
typedef struct dm_force_params {
    long long flags;        /* ForceFlag bitmask of enabled forces */
    double shielding;       /* kappa [1/m]; pairs count only while kappa*r < 10 */
    double confine;         /* ConfinementForce: F = q*confine*(x, y) */
    double confine_x;       /* RectConfinementForce: Fx = q*confine_x*x */
    double confine_y;       /*                       Fy = q*confine_y*y */
    double gamma;           /* DragForce: F = -gamma*m*v */
    double heat;            /* ThermalForce: heatVal [N] (mode 0) or sigma [N] (mode 1) */
    int thermal_mode;       /* 0: heat*U(0,1)*(cos t, sin t), t~U(0,2pi) (ThermalForce.cpp:118-122)
                               1: Gaussian N(0, heat^2) per axis */
    int reserved;           /* must be 0 */
    uint64_t seed;          /* thermal RNG key (Philox4x32-10, counter = particle, step, stage) */
    /* the reference's other per-particle forces (driver.cpp:372-402), each
     * evaluated at the substep's positions, velocities and force time */
    double void_decay;      /* ConfinementForceVoid(C, confine, voidDecay): the confinement force
                               plus F += q*(-decay)*exp(-decay*r)/r*(x, y)
                               (ConfinementForceVoid.cpp:48-55) */
    double drive_const;     /* DrivingForce(C, driveConst, amplitude, shift): */
    double drive_amplitude; /*   F_x += amplitude*sin(x*2pi/2mm - t*2pi*10Hz)*exp(0/driveConst) */
    double drive_shift;     /*   (DrivingForce.cpp:52-61) */
    double magnetic;        /* MagneticForce(C, B): F += q*B*(vy, -vx) (MagneticForce.cpp:48-54) */
    double rot_rmin;        /* RotationalForce(C, rmin, rmax, c): for rmin < r < rmax */
    double rot_rmax;        /*   F += c*(-y, x)/r (RotationalForce.cpp:50-66) */
    double rot_const;
    double heat_in;         /* ThermalForceLocalized(C, heatIn, heatOut, radius): a thermal kick */
    double heat_out;        /*   of scale heatIn for r < radius, heatOut beyond */
    double heat_radius;     /*   (ThermalForceLocalized.cpp:124-133) */
    double drag_scale;      /* TimeVaryingDragForce(C, scale, offset): DragForce with */
    double drag_offset;     /*   dragConst = -(scale*t + offset) (TimeVaryingDragForce.cpp:11-40) */
    double heat_scale;      /* TimeVaryingThermalForce(C, scale, offset): ThermalForce with */
    double heat_offset;     /*   heat = scale*t + offset (TimeVaryingThermalForce.cpp:14-42) */
    double electric;        /* ElectricForce(C, E, R): F += q*E*exp(r/(-R))*(x, y) */
    double electric_radius; /*   (ElectricForce.cpp:48-62) */
    double gravity;         /* GravitationalForce(C, g): F_y += m*g (GravitationalForce.cpp:46-50) */
    double vert_electric;   /* VertElectricForce(C, E, d): F_y += q*E*exp(y/d) */
    double vert_decay;      /*   (VertElectricForce.cpp:47-53) */
} dm_force_params;

typedef struct dm_ctx dm_ctx;
typedef struct dm_cloud dm_cloud;
typedef struct dm_batch dm_batch;

/* ---- context ---------------------------------------------------------- */

/* ABI version of the loaded library (DM_ABI_VERSION). */
int dm_version(void);

/* Creates a context on CUDA device `device` with its own stream.
 * No reference counterpart (the reference is host-only). */
int dm_ctx_create(int device, dm_ctx **out);
int dm_ctx_destroy(dm_ctx *ctx);

/* Use an existing cudaStream_t (passed as void*) for all later work; NULL
 * means the CUDA default (legacy) stream, as in the CUDA runtime. */
int dm_ctx_set_stream(dm_ctx *ctx, void *cuda_stream);
/* Back to the context's own stream. */
int dm_ctx_reset_stream(dm_ctx *ctx);

/* Blocks until all work queued on the context's stream has finished and
 * reports any asynchronous error (including device-side numeric flags). */
int dm_ctx_synchronize(dm_ctx *ctx);

/* Copies the last error message of `ctx` (or of the last failed
 * dm_ctx_create if ctx is NULL) into buf. */
int dm_last_error(const dm_ctx *ctx, char *buf, size_t len);

/* Kernel-duration accounting: when enabled, every pair-force kernel launch
 * is bracketed by CUDA events on the context's stream (CUDA graphs are not
 * used while enabled).  dm_ctx_profile_read synchronizes and returns the
 * summed duration [ms], the launch count and the ordered pairs those
 * launches covered, then resets the counters. */
int dm_ctx_profile_enable(dm_ctx *ctx, int enable);
/* Kernels this library has launched on the context so far (graph replays
 * count every kernel node). */
int dm_ctx_launch_count(dm_ctx *ctx, long long *count);
int dm_ctx_profile_read(dm_ctx *ctx, double *total_ms, long long *launches, double *pairs);

/* Autotuning of the pair kernels (default on).  On a cloud's first step (or
 * dm_cloud_autotune) every compiled kernel variant of the precision is timed
 * on that cloud over a set of j splits (force-only launches, no state
 * change) and the fastest is kept; results are cached per (n, precision) in
 * the context.  Off: a fixed default variant with a cost-model split.  No
 * reference counterpart. */
int dm_ctx_set_autotune(dm_ctx *ctx, int enable);

/* Measures this GPU's FP32 FMA (kind 0) or FP64 FMA (kind 1) throughput
 * [TFLOP/s] with a dependent-chain-free FMA loop; used as the roofline peak. */
int dm_probe_peak(dm_ctx *ctx, int kind, double *tflops);

/* ---- one cloud -------------------------------------------------------- */

/* Creates a device-resident cloud of n particles from host arrays (copied).
 * Replaces `new Cloud(n)` + filling its arrays (Cloud.cpp:23-37); the
 * device owns its buffers for the life of the cloud.  n >= 1 (the reference
 * requires even n, ShieldedCoulombForce.cpp:15-19; this library does not). */
int dm_cloud_create(dm_ctx *ctx, int n, const double *x, const double *y,
                    const double *vx, const double *vy, const double *q,
                    const double *m, dm_cloud **out);
int dm_cloud_destroy(dm_cloud *cloud);
int dm_cloud_size(const dm_cloud *cloud, int *n);

/* Host -> device state (positions, velocities); charges/masses unchanged.
 * Replaces writing Cloud::x/y/Vx/Vy directly (Cloud.h:22).  Page-locked
 * buffers (any for which cudaPointerGetAttributes gives a device address)
 * are read by one device copy kernel; other memory is copied by DMA.  The
 * same holds for dm_cloud_download's outputs. */
int dm_cloud_upload(dm_cloud *cloud, const double *x, const double *y,
                    const double *vx, const double *vy);

/* Device -> host state.  The reference's driver reads Cloud::x.. before
 * Cloud::writeTimeStep (driver.cpp:448-449, Cloud.cpp:258-271).  One stream
 * synchronisation: the device error flags come back with the state.  Host
 * buffers in page-locked memory (cudaMallocHost) are copied by DMA. */
int dm_cloud_download(dm_cloud *cloud, double *x, double *y, double *vx,
                      double *vy);

/* Replaces per-particle charges and masses (Cloud::charge, Cloud::mass). */
int dm_cloud_set_charge_mass(dm_cloud *cloud, const double *q, const double *m);

/* Selects the forces and their parameters.  Replaces constructing the
 * ForceArray (driver.cpp:372-402, Force.h:71): every ForceFlag of the
 * reference is available and they are summed in the driver's order;
 * bits outside the fifteen flags give DM_ERR_UNSUPPORTED. */
int dm_cloud_set_forces(dm_cloud *cloud, const dm_force_params *params);

/* One force evaluation of every enabled force at the current state, i.e.
 * the sum of Force::force1 over the ForceArray (Runge_Kutta2.cpp:90-93,
 * Force.h:28-49) written to host fx, fy (not accumulated).  ThermalForce's
 * kicks are those of substep 1 of the step counter's step. */
int dm_cloud_eval_forces(dm_cloud *cloud, int precision, double *fx, double *fy);
/* The same at the current state taken as the inputs of RK substep `stage`
 * (1..4): the thermal kicks are substep `stage`'s.  Stands in for
 * Force::force1..4 (Force.h:28-49) when the caller supplies the substep
 * positions and velocities (dm_cloud_upload). */
int dm_cloud_eval_forces_stage(dm_cloud *cloud, int precision, int stage,
                               double *fx, double *fy);

/* Same, writing to device arrays of n doubles. */
int dm_cloud_eval_forces_device(dm_cloud *cloud, int precision, double *d_fx,
                                double *d_fy);

/* Advances nsteps RK4 steps of fixed dt: Runge_Kutta4::moveParticles
 * (Runge_Kutta4.cpp:23-137) with CacheOperator (CacheOperator.cpp:18-73)
 * for an explicit step count, without the adaptive dt of line 25.
 * With t_inout, the force time is set to *t_inout first and *t_inout is
 * advanced by dt per step with the reference's accumulation (currentTime
 * += dt); with NULL the steps continue from the cloud's force time
 * (dm_cloud_set_time). */
int dm_cloud_step(dm_cloud *cloud, int nsteps, double dt, int precision,
                  double *t_inout);

/* Runge_Kutta4::moveParticles(endTime) (Runge_Kutta4.cpp:23-137): steps
 * while *t_inout < end_time.  adaptive = 0 uses dt throughout; adaptive = 1
 * reproduces Integrator::modifyTimeStep (Integrator.cpp:68-134), reducing
 * dt by 10x per 10x reduction of the 1e-4 m test distance.  Returns the
 * steps taken in *steps (may be NULL). */
int dm_cloud_move_particles(dm_cloud *cloud, double end_time, double dt,
                            int precision, int adaptive, double *t_inout,
                            int *steps);

/* The adaptive-dt test alone: the minimum FP32 separation over the pairs
 * Integrator::modifyTimeStep checks (Integrator.cpp:90-131) and the dt it
 * would return for init_dt.  Requires n % 4 == 0. */
int dm_cloud_modify_timestep(dm_cloud *cloud, double init_dt, float *min_dist,
                             double *dt_out);

/* FP64 diagnostics at the current state: out[0] kinetic energy, out[1]
 * Yukawa potential energy (pairs with kappa*r < 10), out[2] confinement
 * potential energy, out[3..4] momentum.  No reference counterpart. */
int dm_cloud_diagnostics(dm_cloud *cloud, double out[5]);

/* Runs (or reuses) the autotuner for `precision` and reports the chosen
 * kernel variant name and j split. */
int dm_cloud_autotune(dm_cloud *cloud, int precision, char *variant, size_t len, int *split);

/* Names of the compiled pair-kernel variants, ';'-separated. */
int dm_kernel_variants(char *buf, size_t len);

/* Pins the cloud to one kernel variant (by name) and j split (0 = cost
 * model) instead of the autotuner's choice, for its precision. */
int dm_cloud_set_kernel(dm_cloud *cloud, const char *variant, int split);

/* The device keeps the cloud in Morton (space-filling-curve) order so each
 * warp's particles are spatially compact and the pair kernels' cutoff test
 * wakes the precise arithmetic for few j; the order is internal (every
 * array crossing this ABI is in the caller's order).  The cloud is re-sorted
 * every `steps` RK4 steps (0 = only after an upload; otherwise a power of
 * two <= 16).  Default: every step (clouds of up to 16384 particles are
 * sorted by one thread-block cluster in one launch).  No reference
 * counterpart. */
int dm_cloud_set_reorder_interval(dm_cloud *cloud, int steps);

/* Ordered pairs the culling kernel variants actually swept so far (32-
 * particle j groups within reach of an i tile's box, times the tile), the
 * rest having been skipped by the box test; 0 while no culling variant has
 * run.  Work counter for reports: the pair-interaction metric counts all
 * N(N-1) ordered pairs per force evaluation either way.  No reference
 * counterpart (the reference tests every pair). */
int dm_cloud_evaluated_pairs(dm_cloud *cloud, unsigned long long *pairs);
/* RNG step counter used by the thermal forces (advanced by one per RK4 step). */
int dm_cloud_set_step_counter(dm_cloud *cloud, uint64_t step);
int dm_cloud_get_step_counter(dm_cloud *cloud, uint64_t *step);
/* Integrator of dm_cloud_step and dm_cloud_move_particles: 4 =
 * Runge_Kutta4 (the default), 2 = Runge_Kutta2, the midpoint method
 * (Runge_Kutta2.cpp:23-78, the reference driver's -I): stage 1 at (x, v, t),
 * CacheOperator::operation2, stage 2 at the midpoint and t + dt/2, then
 * v += k2, x += l2.  Same forces, thermal counters and adaptive dt. */
int dm_cloud_set_integrator(dm_cloud *cloud, int order);

/* Force time, the reference's Integrator::currentTime (Integrator.h): RK4
 * step k's stages see t, t + dt/2, t + dt/2, t + dt (Runge_Kutta4.cpp:30-88)
 * and each step advances it by dt (Runge_Kutta4.cpp:135).  Only the
 * time-dependent forces (DrivingForce, TimeVaryingDragForce,
 * TimeVaryingThermalForce) read it; force-only evaluations
 * (dm_cloud_eval_forces*) see the current time.  0 at creation;
 * dm_cloud_move_particles sets it from *t_inout.  Set is stream-ordered. */
int dm_cloud_set_time(dm_cloud *cloud, double t);
int dm_cloud_get_time(dm_cloud *cloud, double *t);

/* ---- many clouds in one launch --------------------------------------- */

/* A batch of independent clouds of uneven size, each with its own force
 * parameters (params[c]).  Arrays are concatenated in cloud order (cloud 0's
 * n[0] particles, then cloud 1's, ...).  Each RK4 stage of the whole batch is
 * one persistent FP32C launch handing out (cloud, i-tile) work items, largest
 * clouds first; kernel variants are autotuned at creation.  The reference
 * runs one cloud per process; this has no reference counterpart beyond
 * dm_cloud_* applied to each cloud. */
int dm_batch_create(dm_ctx *ctx, int nclouds, const int *n, const double *x,
                    const double *y, const double *vx, const double *vy,
                    const double *q, const double *m,
                    const dm_force_params *params, dm_batch **out);
int dm_batch_destroy(dm_batch *batch);
/* nsteps fixed-dt RK4 steps of every cloud (precision must be DM_FP32C). */
int dm_batch_step(dm_batch *batch, int nsteps, double dt, int precision);
/* All forces of every cloud at the current state (caller order). */
int dm_batch_eval_forces(dm_batch *batch, int precision, double *fx, double *fy);
int dm_batch_download(dm_batch *batch, double *x, double *y, double *vx, double *vy);
/* Names of the compiled batch kernel variants, ';'-separated, and pinning
 * one (instead of the autotuner's choice). */
int dm_batch_variants(char *buf, size_t len);
int dm_batch_set_kernel(dm_batch *batch, const char *variant);
/* Ordered pairs the batch's culling kernel variants swept so far (see
 * dm_cloud_evaluated_pairs). */
int dm_batch_evaluated_pairs(dm_batch *batch, unsigned long long *pairs);
/* The autotuned kernel variant, work-item count and persistent grid size. */
int dm_batch_info(dm_batch *batch, char *variant, size_t len, int *nitems, int *grid);
int dm_batch_set_step_counter(dm_batch *batch, uint64_t step);
/* Integrator of dm_batch_step (see dm_cloud_set_integrator). */
int dm_batch_set_integrator(dm_batch *batch, int order);
/* Force time shared by every cloud of the batch (see dm_cloud_set_time). */
int dm_batch_set_time(dm_batch *batch, double t);
int dm_batch_get_time(dm_batch *batch, double *t);

/* ---- differentiable rollout ------------------------------------------ */

/* FP64 forces and their vector-Jacobian product for concatenated clouds on
 * caller-owned DEVICE arrays (the rollout itself is driven from the host,
 * e.g. by torch.autograd).  No reference counterpart: the reference has no
 * derivatives.  Only Confinement, RectConfinement, Drag and ShieldedCoulomb
 * are differentiated; the cutoff jump at kappa*r = 10 is not. */
typedef struct dm_adjoint dm_adjoint;
int dm_adjoint_create(dm_ctx *ctx, int nclouds, const int *n,
                      const dm_force_params *params, dm_adjoint **out);
int dm_adjoint_destroy(dm_adjoint *adj);
/* New per-cloud parameters (kappa, confinement, drag) for later calls. */
int dm_adjoint_set_params(dm_adjoint *adj, const dm_force_params *params);
/* Total force (fx, fy) and, if fpx/fpy are non-NULL, the pair force alone.
 * precision: DM_FP64, or DM_FP32C (FP32 pair terms, Kahan sums, FP64 per
 * particle; ~1e-6 relative).  All pointers are device arrays of the
 * concatenated clouds. */
int dm_adjoint_forces(dm_adjoint *adj, int precision, const double *x,
                      const double *y, const double *vx, const double *vy,
                      const double *q, const double *m, double *fx, double *fy,
                      double *fpx, double *fpy);
/* Given a = dL/dF per particle, writes dL/dp (gx, gy), dL/dv (gvx, gvy),
 * dL/dq_i (gq) and per-particle contributions to dL/dkappa and dL/dk_c of
 * the particle's cloud (gkappa, gkc; sum them over the cloud). */
int dm_adjoint_vjp(dm_adjoint *adj, int precision, const double *x,
                   const double *y, const double *vx, const double *vy,
                   const double *q, const double *m, const double *ax,
                   const double *ay, double *gx, double *gy, double *gvx,
                   double *gvy, double *gq, double *gkappa, double *gkc);

/* One RK4 step of the rollout, fused: four launches, each the pair force at
 * the stage's input state plus the per-particle forces and the stage
 * algebra k_s = dt f(s_s), s_2 = S + k_1/2, s_3 = S + k_2/2, s_4 = S + k_3,
 * S' = S + (k_1 + ((k_2 + k_3) 2 + k_4)) / 6 with f(s) = (vx, vy, F/m) --
 * the reference's Runge_Kutta4::moveParticles written for the state s
 * (Runge_Kutta4.cpp:23-137).  x, y, vx, vy (device arrays of the
 * concatenated clouds) are advanced in place.  stages: NULL, or a device
 * array of 16 * total doubles that receives the four stage inputs (stage s
 * at offset 4 (s-1) total: x, y, vx, vy), for dm_adjoint_rk4_step_vjp. */
int dm_adjoint_rk4_step(dm_adjoint *adj, int precision, double dt, double *x,
                        double *y, double *vx, double *vy, const double *q,
                        const double *m, double *stages);
/* The adjoint of one such step from its stage inputs: (lx, ly, lvx, lvy) =
 * dL/d(output state) on entry, dL/d(input state) on return; the step's
 * contributions to dL/dq_i, and per particle to dL/dkappa and dL/dk_c of its
 * cloud, are ADDED to gq, gkappa, gkc.  Four launches (stages 4..1), each
 * the force VJP at the stage's input and the per-particle adjoint
 * recurrences of RK4.  No reference counterpart. */
int dm_adjoint_rk4_step_vjp(dm_adjoint *adj, int precision, double dt,
                            const double *stages, const double *q, const double *m,
                            double *lx, double *ly, double *lvx, double *lvy,
                            double *gq, double *gkappa, double *gkc);

/* ---- allocation-free diagnostics ------------------------------------- */

/* No counterpart in the reference.  dm_cloud_diagnostics' computation for
 * callers that can't allocate device memory: a host application that owns
 * every device byte through its own pool or budget, or code that must not
 * trigger cudaMalloc's implicit device-wide synchronisation while its other
 * streams run.  The caller passes its own device arrays (n FP64 values each),
 * the force parameters (host struct) and a device output of 5 doubles
 * (same meaning as dm_cloud_diagnostics' out); the work is queued on
 * `stream` (a cudaStream_t, NULL = the legacy default stream) and the call
 * returns without waiting.  It needs no dm_ctx or dm_cloud and calls no
 * allocating CUDA or library routine: its partial sums live in a fixed
 * file-scope device array of 4096 x 5 doubles (160 KiB, held by every GPU
 * that loads this library until the process exits).
 *  - n must be in [1, 524288]; larger n returns DM_ERR_ARG without launching.
 *  - params are checked as dm_cloud_set_forces checks them.
 *  - Every call looks up that array's device address on the current device
 *    (so the address stays right after a cudaDeviceReset); the first call on
 *    a device may load this library's module there, so make that first call
 *    before any stream capture.
 *  - All calls share the array: calls that overlap on the GPU race on it and
 *    must be serialised by the caller (e.g. one stream).
 * Errors are reported by the status code only (dm_last_error is not set). */
int dm_diagnostics_noalloc(int n, const double *d_x, const double *d_y,
                           const double *d_vx, const double *d_vy,
                           const double *d_q, const double *d_m,
                           const dm_force_params *params, double *d_out,
                           void *stream);

#ifdef __cplusplus
}
#endif
#endif /* DEMON_GB300_H */
