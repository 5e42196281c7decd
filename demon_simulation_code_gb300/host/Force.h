/**
 * Force.h -- the abstract force and the force flags (Force.h:15-91 in the
 * reference).
 *
 * As in the reference, force1..4(currentTime) ADD the force at the inputs of
 * RK substep 1..4 into cloud->forceX / forceY (substep 1: x, y, Vx, Vy;
 * substeps 2-4: the CacheOperator's xCache, yCache, VxCache, VyCache), and
 * writeForce / readForce store the force's FORCES flag and parameters in
 * the output file's primary header.
 *
 * GB300 addition: addDeviceParams() folds the force into the parameter
 * block of the fused device stage kernel (dm_force_params), through which
 * Runge_Kutta4 evaluates every force of the ForceArray in one launch.  A
 * force that cannot be fused (a user-defined one, or a second shielded
 * Coulomb force with another kappa) returns false and Runge_Kutta4 refuses
 * the ForceArray.
 */
#ifndef FORCE_H
#define FORCE_H

#include <cstdint>
#include <vector>

#include "Cloud.h"

class Force {
public:
    Cloud *const cloud;  //!< Cloud object

    Force(Cloud *const C) : cloud(C) {}
    virtual ~Force() {}

    virtual void force1(const double currentTime) = 0;  // rk substep 1
    virtual void force2(const double currentTime) = 0;  // rk substep 2
    virtual void force3(const double currentTime) = 0;  // rk substep 3
    virtual void force4(const double currentTime) = 0;  // rk substep 4

    virtual void writeForce(fitsfile *const file, int *const error) const = 0;
    virtual void readForce(fitsfile *const file, int *const error) = 0;

    /// Adds this force to `p` (flags and constants); false if it cannot be
    /// expressed there (given what `p` already holds).
    virtual bool addDeviceParams(dm_force_params &p) const {
        (void)p;
        return false;
    }
};

typedef std::vector<Force *> ForceArray;  //!< Vector of Force objects
typedef long force_flags;                 //!< bit-packed FORCES keyword

enum ForceFlag : force_flags {
    ConfinementForceFlag = 1,
    DragForceFlag = 2,
    ShieldedCoulombForceFlag = 4,
    GravitationalForceFlag = 8,
    ThermalForceFlag = 16,
    ThermalForceLocalizedFlag = 32,
    DrivingForceFlag = 64,
    RotationalForceFlag = 128,
    TimeVaryingDragForceFlag = 256,
    TimeVaryingThermalForceFlag = 512,
    MagneticForceFlag = 1024,
    ConfinementForceVoidFlag = 2048,
    ElectricForceFlag = 4096,
    RectConfinementForceFlag = 8192,
    VertElectricForceFlag = 16384
};

/**
 * A force evaluated on the GPU.  force1..4 evaluate this force alone on the
 * cloud's scratch device copy at the substep's inputs and add the result
 * into forceX / forceY (one upload, one launch, one download each: the
 * per-force API is for checks and for composing with host code; the fused
 * Runge_Kutta4 path does not use it).
 */
class DeviceForce : public Force {
public:
    DeviceForce(Cloud *const C) : Force(C) {}
    void force1(const double currentTime) override { evaluate(1, currentTime); }
    void force2(const double currentTime) override { evaluate(2, currentTime); }
    void force3(const double currentTime) override { evaluate(3, currentTime); }
    void force4(const double currentTime) override { evaluate(4, currentTime); }

    /// Pair arithmetic of the per-force evaluations (DM_FP64 or DM_FP32C).
    static int precision;

protected:
    /// RK step index of the per-force thermal kicks; advanced after force4.
    uint64_t step = 0;
    void evaluate(int stage, double currentTime);
    /// FORCES |= flag in the primary header.
    static void addFlag(fitsfile *const file, force_flags flag, int *const error);
};

#endif  // FORCE_H
