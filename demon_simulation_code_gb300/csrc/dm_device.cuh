// dm_device.cuh -- device-side data layout and per-particle arithmetic of the
// DEMON hot path on sm_103a.
//
// Layout in HBM (one cloud, n particles padded to n_pad, a multiple of 64):
//   base state       x, y, vx, vy, q, m                      FP64 [n_pad]
//   stage velocity   vxc, vyc  (CacheOperator's VxCache/VyCache) FP64 [n_pad]
//   RK4 increments   a1[4] = k1, l1, m1, n1                 FP64 [n_pad]
//                    a23[4] = k2+k3, l2+l3, m2+m3, n2+n3     FP64 [n_pad]
//   stage positions  two buffers b = 0, 1; stage s reads b = (s-1)&1 and its
//                    epilogue writes the next stage's positions into b^1:
//                      px[b], py[b]  FP64 (CacheOperator's xCache/yCache)
//                      pa[b] = (xh, yh, xh^2+yh^2, (float)q)  float4
//                      pb[b] = (xl, yl, -threshold, 0)        float4
//                    (threshold = the FP32 pair filter's bound, see
//                    filter_threshold; computed once per particle here
//                    instead of in every CTA that reads the particle)
//                    with x = xh + xl exactly to 48 bits (two-float form).
//   padding          particles n..n_pad-1 sit at 1e18 m with q = 0, so the
//                    cutoff test never selects them.
#pragma once

#include <cfloat>
#include <cstdint>
#include <cuda_runtime.h>

namespace dm {

// ForceFlag bits (Force.h:75-91)
constexpr long long kConfinement = 1;
constexpr long long kDrag = 2;
constexpr long long kShieldedCoulomb = 4;
constexpr long long kGravitational = 8;
constexpr long long kThermal = 16;
constexpr long long kThermalLocalized = 32;
constexpr long long kDriving = 64;
constexpr long long kRotational = 128;
constexpr long long kTimeVaryingDrag = 256;
constexpr long long kTimeVaryingThermal = 512;
constexpr long long kMagnetic = 1024;
constexpr long long kConfinementVoid = 2048;
constexpr long long kElectric = 4096;
constexpr long long kRectConfinement = 8192;
constexpr long long kVertElectric = 16384;
constexpr long long kAllForces = 32767;
// forces that read the force time
constexpr long long kTimeForces = kDriving | kTimeVaryingDrag | kTimeVaryingThermal;
// Forces whose x and y components are independent (the fast epilogue path)
constexpr long long kBasicForces = kConfinement | kDrag | kRectConfinement | kShieldedCoulomb | kThermal;

constexpr float kPadPosition = 1.0e18f;

struct ForceParams {  // same layout as dm_force_params
    long long flags;
    double shielding, confine, confine_x, confine_y, gamma, heat;
    int thermal_mode, reserved;
    unsigned long long seed;
    double void_decay, drive_const, drive_amplitude, drive_shift, magnetic, rot_rmin, rot_rmax, rot_const;
    double heat_in, heat_out, heat_radius, drag_scale, drag_offset, heat_scale, heat_offset;
    double electric, electric_radius, gravity, vert_electric, vert_decay;
};

struct CloudDev {
    int n, n_pad;
    double *x, *y, *vx, *vy, *q, *m;
    double *vxc, *vyc;
    double *a1[4];
    double *a23[4];
    double *px[2], *py[2];
    float4 *pa[2], *pb[2];
    float4 *gbox[2];               // [n_pad/32] FP32 box (x0, y0, x1, y1) of each 32-particle group
    unsigned long long *eval_pairs;  // ordered pairs the culling kernels swept (cumulative)
    unsigned long long *step_ctr;  // [2], see stage_step_index()
    double *time;                  // [2] force time slots, see stage_time()
    int *err;                      // device error flags
    double rc2;                    // (10/kappa)^2 of the current force parameters
    double coulomb;                // 1/(4 pi eps0)
    int *orig;                     // caller's index of internal slot s (Morton order)
};

// Host-side check of a force parameter set, shared by every entry point that
// takes one: DM_OK (0), or a status with *why set to a static message.
// Flags must be among the fifteen ForceFlag bits (status 6, unsupported);
// with ShieldedCoulomb on, kappa must be positive and finite (the cutoff is
// kappa*r < 10) and thermal_mode must be 0 or 1 (status 1, bad argument).
inline int check_force_params(const ForceParams &p, const char **why) {
    if (p.flags & ~kAllForces) {
        *why = "unknown force flags";
        return 6;
    }
    if ((p.flags & kShieldedCoulomb) && !(p.shielding > 0.0 && p.shielding <= DBL_MAX)) {
        *why = "shielding must be positive and finite";
        return 1;
    }
    if (p.thermal_mode != 0 && p.thermal_mode != 1) {
        *why = "thermal_mode must be 0 or 1";
        return 1;
    }
    return 0;
}

enum StageMode : int { kModeStep = 0, kModeForceOnly = 1 };

// Everything a stage kernel needs, passed by value.
struct StageParams {
    CloudDev c;
    ForceParams f;
    int stage;            // 1..order
    int order;            // 4: Runge_Kutta4; 2: Runge_Kutta2 (the midpoint method)
    int mode;             // StageMode
    int therm_stage;      // substep index of the thermal kicks (force-only: any of 1..4)
    int fo_buf;           // force-only launches: stage position buffer to read (0 = the state)
    double dt;            // fixed dt (used when dt_dev == nullptr)
    const double *dt_dev; // adaptive dt computed on the device
    double coulomb;       // 1/(4 pi eps0)
    double *fx_out, *fy_out;  // kModeForceOnly outputs
    // pair-kernel constants
    double rc2;           // (10/kappa)^2
    float rc2_lo, rc2_hi; // FP32 certain-in / certain-out bounds on r^2
    float kappa_f;
    float nkl2e;          // -kappa*log2(e): e^{-kappa r} = 2^{nkl2e r}
    // FP32C sweep: a filtered chunk whose 4 j pass the filter for at least
    // this many of the 128 (lane, j) pairs of a slot is evaluated directly
    // (all lanes, cutoff by a select) instead of through per-lane hit bits
    int direct_min;
    // culling: a near group whose farthest separation from the tile is
    // within sqrt(near_direct_f2) r_c skips the filter (every chunk
    // evaluated directly); 0: no such class
    float near_direct_f2;
    // j split without clusters: rank r of tile t is block t*split + r and
    // writes its partial sums (s, c) of particle i to the float2 planes
    // partial[(2r + axis)*n_pad + i]; stage_finish sums them
    int split;
    float2 *partial;
    int box_out;  // stage_finish: also write the group boxes of the buffer the epilogue writes
};

// ---------------------------------------------------------------------------
// Counter-based RNG: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t hi0 = __umulhi(M0, c[0]), lo0 = M0 * c[0];
        const uint32_t hi1 = __umulhi(M1, c[2]), lo1 = M1 * c[2];
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += W0; k1 += W1;
    }
}

// Thermal kick arithmetic: FP32 Box-Muller built only from correctly rounded
// IEEE single operations (add, mul, fma, div, sqrt) in a fixed order, so the
// CPU oracle reproduces it bit for bit (oracle/demon_oracle.c).  The kick is
// noise of relative size ~1e-5 of the forces it is added to; FP32 (rather
// than FP64, which runs at 1/64 of the FP32 rate on this GPU) loses nothing.
//
// u in (0, 1): 24 random bits, (k + 0.5) * 2^-24.
__device__ __forceinline__ float u24(uint32_t w) {
    return __fmul_rn(__fadd_rn((float)(w >> 8), 0.5f), 5.9604644775390625e-8f);
}

// ln(u), u in (0, 1]: u = 2^e m with m in [sqrt(1/2), sqrt(2)),
// ln m = 2 atanh(s), s = (m-1)/(m+1), atanh by its odd series to s^9
// (|s| < 0.1716: truncation < 2e-9).
__device__ __forceinline__ float thermal_log(float u) {
    const uint32_t bits = __float_as_uint(u);
    int e = (int)(bits >> 23) - 127;
    float m = __uint_as_float((bits & 0x007FFFFFu) | 0x3F800000u);
    if (m > 1.41421356f) {
        m = __fmul_rn(m, 0.5f);
        e += 1;
    }
    const float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
    const float s2 = __fmul_rn(s, s);
    float p = __fmaf_rn(s2, 0.111111111f, 0.142857143f);
    p = __fmaf_rn(s2, p, 0.2f);
    p = __fmaf_rn(s2, p, 0.333333333f);
    p = __fmaf_rn(s2, p, 1.0f);
    const float lnm = __fmul_rn(__fmul_rn(2.0f, s), p);
    return __fmaf_rn((float)e, 0.693147181f, lnm);
}

// sin and cos of 2 pi u, u in [0, 1): quadrant q = floor(4u), a = (4u - q) pi/2
// in [0, pi/2), Taylor polynomials to a^13 (sin) and a^14 (cos), truncation
// < 7e-10, then the exact quadrant rotation.
__device__ __forceinline__ void thermal_sincos(float u, float &sn, float &cs) {
    const float r = __fmul_rn(u, 4.0f);
    const float qf = floorf(r);
    const int q = (int)qf;
    const float a = __fmul_rn(__fsub_rn(r, qf), 1.57079633f);
    const float a2 = __fmul_rn(a, a);
    float ps = __fmaf_rn(a2, 1.60590438e-10f, -2.50521084e-8f);
    ps = __fmaf_rn(a2, ps, 2.75573192e-6f);
    ps = __fmaf_rn(a2, ps, -1.98412698e-4f);
    ps = __fmaf_rn(a2, ps, 8.33333333e-3f);
    ps = __fmaf_rn(a2, ps, -1.66666667e-1f);
    ps = __fmaf_rn(a2, ps, 1.0f);
    const float sa = __fmul_rn(a, ps);
    float pc = __fmaf_rn(a2, -1.14707456e-11f, 2.08767570e-9f);
    pc = __fmaf_rn(a2, pc, -2.75573192e-7f);
    pc = __fmaf_rn(a2, pc, 2.48015873e-5f);
    pc = __fmaf_rn(a2, pc, -1.38888889e-3f);
    pc = __fmaf_rn(a2, pc, 4.16666667e-2f);
    pc = __fmaf_rn(a2, pc, -0.5f);
    const float ca = __fmaf_rn(a2, pc, 1.0f);
    switch (q & 3) {
        case 0: sn = sa; cs = ca; break;
        case 1: sn = ca; cs = -sa; break;
        case 2: sn = -sa; cs = -ca; break;
        default: sn = -ca; cs = sa; break;
    }
}

// Counter-based kick of scale `heat` for particle i: counter (i, step lo,
// step hi, stream).  Mode 0 is the reference's form heatVal*U*(cos t, sin t),
// t ~ U(0, 2pi) (ThermalForce.cpp:118-140) with counter-based uniforms; mode
// 1 is a Gaussian of standard deviation `heat` per axis (Box-Muller).
// Streams: stage for ThermalForce, stage + 16 for ThermalForceLocalized,
// stage + 32 for TimeVaryingThermalForce.
__device__ __forceinline__ void thermal_draw(const ForceParams &f, uint32_t i,
                                             unsigned long long step, int stream, double heat,
                                             double &tx, double &ty) {
    uint32_t c[4] = {i, (uint32_t)step, (uint32_t)(step >> 32), (uint32_t)stream};
    philox4x32_10(c, (uint32_t)f.seed, (uint32_t)(f.seed >> 32));
    const float u1 = u24(c[0]);
    const float u2 = u24(c[1]);
    float sn, cs;
    thermal_sincos(u2, sn, cs);
    float amp;
    if (f.thermal_mode == 0) amp = u1;
    else amp = __fsqrt_rn(__fmul_rn(-2.0f, thermal_log(u1)));
    tx = __dmul_rn(heat, (double)__fmul_rn(amp, cs));
    ty = __dmul_rn(heat, (double)__fmul_rn(amp, sn));
}

__device__ __forceinline__ void thermal_kick(const ForceParams &f, uint32_t i,
                                             unsigned long long step, int stage,
                                             double &tx, double &ty) {
    thermal_draw(f, i, step, stage, f.heat, tx, ty);
}

// RNG step index of the running stage.  Stage 1 reads slot 0 and copies it
// to slot 1; stages 2-4 read slot 1; stage 4 advances slot 0.  Each slot is
// written only in a launch that never reads it, so no launch races itself.
__device__ __forceinline__ unsigned long long stage_step_index(const StageParams &P) {
    const int s = (P.mode == kModeForceOnly) ? 1 : P.stage;
    return (s == 1) ? P.c.step_ctr[0] : P.c.step_ctr[1];
}
// Force time of the running stage: t, t + dt/2.0, t + dt/2.0, t + dt for
// RK4 stages 1-4 (Runge_Kutta4.cpp:30-88), t, t + dt/2.0 for RK2 stages 1-2
// (Runge_Kutta2.cpp:28-50), t the time at the start of the step.  Same slot
// discipline as the step counter: stage 1 reads slot 0 and copies it to
// slot 1, later stages read slot 1, the last stage writes slot 0 = t + dt
// (currentTime += dt, Runge_Kutta4.cpp:135, Runge_Kutta2.cpp:76).
// Force-only launches use the time in slot 0.
__device__ __forceinline__ double stage_dt(const StageParams &P) {
    return P.dt_dev ? *P.dt_dev : P.dt;
}
__device__ __forceinline__ double stage_time(const StageParams &P) {
    if (P.mode == kModeForceOnly || P.stage == 1) return P.c.time[0];
    const double t = P.c.time[1], dt = stage_dt(P);
    return (P.stage == 4) ? __dadd_rn(t, dt) : __dadd_rn(t, __ddiv_rn(dt, 2.0));
}
__device__ __forceinline__ void stage_step_advance(const StageParams &P) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    if (P.mode == kModeForceOnly) return;
    if (P.stage == 1) {
        P.c.step_ctr[1] = P.c.step_ctr[0];
        P.c.time[1] = P.c.time[0];
    } else if (P.stage == P.order) {
        P.c.step_ctr[0] = P.c.step_ctr[1] + 1ull;
        P.c.time[0] = __dadd_rn(P.c.time[1], stage_dt(P));
    }
}

// Two-float split of a position: x = hi + lo.
__device__ __forceinline__ void split2(double x, float &hi, float &lo) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(__dsub_rn(x, (double)hi));
}

// Bound of the FP32 pair filter for particle i at hi position (xh, yh):
// the filter passes pair (i, j) iff |p_j|^2 - 2 p_i.p_j < rc^2 - |p_i|^2 +
// margin, evaluated in FP32 on the hi parts.  The margin 2^-17 (|p_i| + rc)^2
// is ~10x the worst FP32 rounding of that expanded form plus the hi/lo split
// error for any pair within rc of i, so no pair the reference keeps is
// filtered out.  Evaluated in FP32 with every operation rounded in the
// direction that keeps the result an upper bound of the exact value of
// rc^2 - |p_i|^2 + 2^-17 (|p_i| + rc)^2 (|p_i|^2 rounded down where it is
// subtracted, up where it feeds the margin), so the bound can only be
// looser, by a few FP32 ulps of |p_i|^2 -- ~1% of the margin.  GB300 runs
// FP64 at ~1/64 of the FP32 rate: one conversion is the only FP64 operation.
__device__ __forceinline__ float filter_threshold(float xh, float yh, double rc2) {
    const float rcf = __double2float_ru(rc2);                  // >= rc^2
    const float a2_dn = __fmaf_rd(xh, xh, __fmul_rd(yh, yh));  // <= |p_i|^2
    const float a2_up = __fmaf_ru(xh, xh, __fmul_ru(yh, yh));  // >= |p_i|^2
    const float pf = __fadd_ru(__fsqrt_ru(a2_up), __fsqrt_ru(rcf));  // >= |p_i| + rc
    const float margin = __fmul_ru(__fmul_ru(pf, pf), 7.62939453125e-6f);
    return __fadd_ru(__fsub_ru(rcf, a2_dn), margin);
}

// Programmatic dependent launch: a kernel launched with the programmatic-
// serialization attribute may be scheduled while its predecessor in the
// stream is still running.  pdl_wait() blocks until the predecessor grid has
// completed and its writes are visible, so every such kernel calls it before
// its first global memory access (a no-op for a kernel launched without the
// attribute).  No kernel here triggers its dependents early
// (griddepcontrol.launch_dependents after the wait): measured on the disk16k
// step sequence it made calm steps 25% slower (0.138 -> 0.172 ms), the next
// kernel's early blocks competing with the running grid's.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Starts bringing a global-memory line into L1 (no data returned, no fault on
// the address being read later by this thread).
__device__ __forceinline__ void prefetch_l1(const void *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

__device__ __forceinline__ void write_stage_position(const CloudDev &c, int b, int i,
                                                     double xs, double ys) {
    c.px[b][i] = xs;
    c.py[b][i] = ys;
    float xh, xl, yh, yl;
    split2(xs, xh, xl);
    split2(ys, yh, yl);
    const double q = c.q[i];
    c.pa[b][i] = make_float4(xh, yh, fmaf(yh, yh, xh * xh), __double2float_rn(q));
    c.pb[b][i] = make_float4(xl, yl, -filter_threshold(xh, yh, c.rc2), 0.0f);
}

// Reference cutoff decision for one pair, bit for bit:
// r = sqrt(dx*dx + dy*dy) (no fused multiply-add, SSE4.2 has none),
// kappa*r < 10 (ShieldedCoulombForce.cpp:144-147, 175-178).
__device__ __forceinline__ bool ref_in_cutoff(double dx, double dy, double kappa, double &r,
                                              double &a) {
    r = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    a = __dmul_rn(r, kappa);
    return a < 10.0;
}

// Thermal kick of particle i for the running stage (zero when the thermal
// force is off); computed ahead of the epilogue by the pair kernels.
__device__ __forceinline__ double2 stage_thermal(const StageParams &P, int i) {
    double tx = 0.0, ty = 0.0;
    if (P.f.flags & kThermal) {
        thermal_kick(P.f, (uint32_t)P.c.orig[i], stage_step_index(P), P.therm_stage, tx, ty);
    }
    return make_double2(tx, ty);
}

// DrivingForce::waveNum, angFreq (DrivingForce.cpp:14-15)
constexpr double kWaveNum = 2.0 * 3.14159265358979323846 / 0.002;
constexpr double kAngFreq = 2.0 * 3.14159265358979323846 * 10.0;

// One particle's per-particle forces, each added as the reference's force()
// adds into forceX/forceY (plusEqual_pd / minusEqual_pd); every FP64
// operation is an explicit round-to-nearest intrinsic so nothing is fused.
struct ParticleAt {
    double x, y, vx, vy, q, m;
};

// ConfinementForce::force (ConfinementForce.cpp:48-54)
__device__ __forceinline__ void add_confinement(const ForceParams &f, const ParticleAt &s, double &Fx,
                                                double &Fy) {
    const double cq = __dmul_rn(s.q, f.confine);
    Fx = __dadd_rn(Fx, __dmul_rn(cq, s.x));
    Fy = __dadd_rn(Fy, __dmul_rn(cq, s.y));
}

// DragForce::force (DragForce.cpp:49-55) with dragConst
__device__ __forceinline__ void add_drag(double dragConst, const ParticleAt &s, double &Fx, double &Fy) {
    const double d = __dmul_rn(s.m, dragConst);
    Fx = __dadd_rn(Fx, __dmul_rn(d, s.vx));
    Fy = __dadd_rn(Fy, __dmul_rn(d, s.vy));
}

// sqrt(x*x + y*y) without contraction (length_pd, VectorCompatibility.h:290-292)
__device__ __forceinline__ double radius_of(const ParticleAt &s) {
    return __dsqrt_rn(__dadd_rn(__dmul_rn(s.x, s.x), __dmul_rn(s.y, s.y)));
}

// The forces the reference driver pushes before ShieldedCoulomb other than
// Confinement and Drag (driver.cpp:375-386), in its order around them:
// ConfinementVoid (ConfinementForceVoid.cpp:13-17, 48-55) after Confinement,
// then Drag, Driving (DrivingForce.cpp:52-61), Magnetic
// (MagneticForce.cpp:48-54), RectConfinement (RectConfinementForce.cpp:50-59),
// Rotational (RotationalForce.cpp:50-66).
__device__ __forceinline__ void add_forces_before_pairs(const ForceParams &f, const ParticleAt &s,
                                                        double t, double &Fx, double &Fy) {
    const long long fl = f.flags;
    if (fl & kConfinement) add_confinement(f, s, Fx, Fy);
    if (fl & kConfinementVoid) {
        add_confinement(f, s, Fx, Fy);
        const double decayV = __dmul_rn(s.q, -f.void_decay);
        const double r = radius_of(s);
        const double expR = __ddiv_rn(exp(__dmul_rn(r, -f.void_decay)), r);
        Fx = __dadd_rn(Fx, __dmul_rn(__dmul_rn(decayV, expR), s.x));
        Fy = __dadd_rn(Fy, __dmul_rn(__dmul_rn(decayV, expR), s.y));
    }
    if (fl & kDrag) add_drag(-f.gamma, s, Fx, Fy);  // dragConst = -gamma (DragForce.h:16-17)
    if (fl & kDriving) {
        // the stored driveConst is -drive_const (DrivingForce.h:17-18)
        const double distV = __dsub_rn(s.x, f.drive_shift);
        const double sinArg = __dsub_rn(__dmul_rn(s.x, kWaveNum), __dmul_rn(t, kAngFreq));
        const double expArg = __ddiv_rn(__dsub_rn(distV, distV), f.drive_const);
        Fx = __dadd_rn(Fx, __dmul_rn(__dmul_rn(sin(sinArg), exp(expArg)), f.drive_amplitude));
    }
    if (fl & kMagnetic) {
        const double qB = __dmul_rn(s.q, f.magnetic);
        Fx = __dadd_rn(Fx, __dmul_rn(qB, s.vy));
        Fy = __dsub_rn(Fy, __dmul_rn(qB, s.vx));
    }
    if (fl & kRectConfinement) {
        Fx = __dadd_rn(Fx, __dmul_rn(__dmul_rn(s.q, f.confine_x), s.x));
        Fy = __dadd_rn(Fy, __dmul_rn(__dmul_rn(s.q, f.confine_y), s.y));
    }
    if (fl & kRotational) {
        const double r = radius_of(s);
        if (r > f.rot_rmin && r < f.rot_rmax) {
            Fx = __dsub_rn(Fx, __ddiv_rn(__dmul_rn(f.rot_const, s.y), r));
            Fy = __dadd_rn(Fy, __ddiv_rn(__dmul_rn(f.rot_const, s.x), r));
        }
    }
}

// The forces pushed after ShieldedCoulomb and Thermal (driver.cpp:391-402):
// ThermalLocalized (ThermalForceLocalized.cpp:124-133), TimeVaryingDrag
// (TimeVaryingDragForce.cpp:11-40), TimeVaryingThermal
// (TimeVaryingThermalForce.cpp:14-42), Electric (ElectricForce.cpp:48-62),
// Gravitational (GravitationalForce.cpp:46-50), VertElectric
// (VertElectricForce.cpp:47-53).
__device__ __forceinline__ void add_forces_after_pairs(const ForceParams &f, const ParticleAt &s,
                                                       double t, uint32_t id, unsigned long long step,
                                                       int stage, double &Fx, double &Fy) {
    const long long fl = f.flags;
    if (fl & kThermalLocalized) {
        const double heat = (radius_of(s) < f.heat_radius) ? f.heat_in : f.heat_out;
        double tx, ty;
        thermal_draw(f, id, step, stage + 16, heat, tx, ty);
        Fx = __dadd_rn(Fx, tx);
        Fy = __dadd_rn(Fy, ty);
    }
    if (fl & kTimeVaryingDrag) add_drag(-__dadd_rn(__dmul_rn(f.drag_scale, t), f.drag_offset), s, Fx, Fy);
    if (fl & kTimeVaryingThermal) {
        double tx, ty;
        thermal_draw(f, id, step, stage + 32, __dadd_rn(__dmul_rn(f.heat_scale, t), f.heat_offset), tx, ty);
        Fx = __dadd_rn(Fx, tx);
        Fy = __dadd_rn(Fy, ty);
    }
    if (fl & kElectric) {
        const double cV = __dmul_rn(s.q, f.electric);
        const double eV = __dmul_rn(cV, exp(__ddiv_rn(radius_of(s), -f.electric_radius)));
        Fx = __dadd_rn(Fx, __dmul_rn(eV, s.x));
        Fy = __dadd_rn(Fy, __dmul_rn(eV, s.y));
    }
    if (fl & kGravitational) Fy = __dadd_rn(Fy, __dmul_rn(s.m, f.gravity));
    if (fl & kVertElectric) {
        const double cV = __dmul_rn(s.q, f.vert_electric);
        Fy = __dadd_rn(Fy, __dmul_rn(cV, exp(__ddiv_rn(s.y, f.vert_decay))));
    }
}

// The per-particle epilogue of one RK stage for particle i, given the
// shielded-Coulomb pair sum (fpx, fpy) at the stage positions:
//  - sums the enabled forces in the reference driver's order
//    (driver.cpp:372-402): Confinement, ConfinementVoid, Drag, Driving,
//    Magnetic, RectConfinement, Rotational, ShieldedCoulomb, Thermal,
//    ThermalLocalized, TimeVaryingDrag, TimeVaryingThermal, Electric,
//    Gravitational, VertElectric, at the stage's force time;
//  - stage increments k = (dt*Fx)/m, l = dt*Vx_stage (Runge_Kutta4.cpp:32-104);
//  - the next stage's CacheOperator values (CacheOperator.cpp:28-73);
//  - after stage 4 the combine v += (k1 + (2*(k2+k3) + k4))/6
//    (Runge_Kutta4.cpp:107-133, 147-151); for RK2 (order 2) stage 2 ends
//    the step with v += k2, x += l2 (Runge_Kutta2.cpp:68-75).
// Every FP64 operation is an explicit round-to-nearest intrinsic so nothing
// is contracted into an FMA: given the same forces the state update is bit
// for bit the reference's.  The forces other than Confinement, Drag,
// RectConfinement, ShieldedCoulomb and Thermal sit behind one flag test.
__device__ __forceinline__ void stage_epilogue(const StageParams &P, int i, double fpx,
                                               double fpy, double2 therm) {
    const CloudDev &c = P.c;
    const int s = (P.mode == kModeForceOnly) ? 1 : P.stage;
    const int b = (P.mode == kModeForceOnly) ? P.fo_buf : (s - 1) & 1;
    const double xs = c.px[b][i], ys = c.py[b][i];
    const double vxs = (s == 1) ? c.vx[i] : c.vxc[i];
    const double vys = (s == 1) ? c.vy[i] : c.vyc[i];
    const double q = c.q[i], m = c.m[i];
    const long long fl = P.f.flags;
    double Fx = 0.0, Fy = 0.0;
    if (fl & ~kBasicForces) {
        const ParticleAt pt{xs, ys, vxs, vys, q, m};
        const double t = (fl & kTimeForces) ? stage_time(P) : 0.0;
        add_forces_before_pairs(P.f, pt, t, Fx, Fy);
        if (fl & kShieldedCoulomb) {
            Fx = __dadd_rn(Fx, fpx);
            Fy = __dadd_rn(Fy, fpy);
        }
        if (fl & kThermal) {
            Fx = __dadd_rn(Fx, therm.x);
            Fy = __dadd_rn(Fy, therm.y);
        }
        add_forces_after_pairs(P.f, pt, t, (uint32_t)c.orig[i], stage_step_index(P), P.therm_stage, Fx, Fy);
    } else {
        if (fl & kConfinement) {
            const double cq = __dmul_rn(q, P.f.confine);
            Fx = __dadd_rn(Fx, __dmul_rn(cq, xs));
            Fy = __dadd_rn(Fy, __dmul_rn(cq, ys));
        }
        if (fl & kDrag) {
            const double d = __dmul_rn(m, -P.f.gamma);
            Fx = __dadd_rn(Fx, __dmul_rn(d, vxs));
            Fy = __dadd_rn(Fy, __dmul_rn(d, vys));
        }
        if (fl & kRectConfinement) {
            Fx = __dadd_rn(Fx, __dmul_rn(__dmul_rn(q, P.f.confine_x), xs));
            Fy = __dadd_rn(Fy, __dmul_rn(__dmul_rn(q, P.f.confine_y), ys));
        }
        if (fl & kShieldedCoulomb) {
            Fx = __dadd_rn(Fx, fpx);
            Fy = __dadd_rn(Fy, fpy);
        }
        if (fl & kThermal) {
            Fx = __dadd_rn(Fx, therm.x);
            Fy = __dadd_rn(Fy, therm.y);
        }
    }
    if (P.mode == kModeForceOnly) {  // outputs in the caller's order
        P.fx_out[c.orig[i]] = Fx;
        P.fy_out[c.orig[i]] = Fy;
        return;
    }
    const double dt = stage_dt(P);
    const double k = __ddiv_rn(__dmul_rn(dt, Fx), m);
    const double l = __dmul_rn(dt, vxs);
    const double mm = __ddiv_rn(__dmul_rn(dt, Fy), m);
    const double nn = __dmul_rn(dt, vys);
    const double x = c.x[i], y = c.y[i], vx = c.vx[i], vy = c.vy[i];
    double nx, ny, nvx = 0.0, nvy = 0.0;
    const bool last = (s == P.order);
    if (last && s == 2) {  // Runge_Kutta2: x += l2, Vx += k2
        const double xn = __dadd_rn(x, l), yn = __dadd_rn(y, nn);
        c.vx[i] = __dadd_rn(vx, k);
        c.x[i] = xn;
        c.vy[i] = __dadd_rn(vy, mm);
        c.y[i] = yn;
        nx = xn;
        ny = yn;
    } else if (s == 1 || s == 2) {
        if (s == 1) {
            c.a1[0][i] = k; c.a1[1][i] = l; c.a1[2][i] = mm; c.a1[3][i] = nn;
        } else {
            c.a23[0][i] = k; c.a23[1][i] = l; c.a23[2][i] = mm; c.a23[3][i] = nn;
        }
        // operation2 / operation3: cache = 0.5*tidbit + base
        nx = __dadd_rn(__dmul_rn(0.5, l), x);
        ny = __dadd_rn(__dmul_rn(0.5, nn), y);
        nvx = __dadd_rn(__dmul_rn(0.5, k), vx);
        nvy = __dadd_rn(__dmul_rn(0.5, mm), vy);
    } else if (s == 3) {
        c.a23[0][i] = __dadd_rn(c.a23[0][i], k);
        c.a23[1][i] = __dadd_rn(c.a23[1][i], l);
        c.a23[2][i] = __dadd_rn(c.a23[2][i], mm);
        c.a23[3][i] = __dadd_rn(c.a23[3][i], nn);
        // operation4: cache = base + tidbit
        nx = __dadd_rn(x, l);
        ny = __dadd_rn(y, nn);
        nvx = __dadd_rn(vx, k);
        nvy = __dadd_rn(vy, mm);
    } else {
        // da(a1, a2, a3, a4) = (a1 + ((a2 + a3)*2 + a4)) / 6
        const double dvx = __ddiv_rn(__dadd_rn(c.a1[0][i], __dadd_rn(__dmul_rn(c.a23[0][i], 2.0), k)), 6.0);
        const double dx = __ddiv_rn(__dadd_rn(c.a1[1][i], __dadd_rn(__dmul_rn(c.a23[1][i], 2.0), l)), 6.0);
        const double dvy = __ddiv_rn(__dadd_rn(c.a1[2][i], __dadd_rn(__dmul_rn(c.a23[2][i], 2.0), mm)), 6.0);
        const double dy = __ddiv_rn(__dadd_rn(c.a1[3][i], __dadd_rn(__dmul_rn(c.a23[3][i], 2.0), nn)), 6.0);
        const double xn = __dadd_rn(x, dx), yn = __dadd_rn(y, dy);
        c.vx[i] = __dadd_rn(vx, dvx);
        c.x[i] = xn;
        c.vy[i] = __dadd_rn(vy, dvy);
        c.y[i] = yn;
        nx = xn;
        ny = yn;
    }
    write_stage_position(c, b ^ 1, i, nx, ny);
    if (!last) {
        c.vxc[i] = nvx;
        c.vyc[i] = nvy;
    }
    if (!isfinite(nx) || !isfinite(ny)) atomicOr(c.err, 1);
}

}  // namespace dm
