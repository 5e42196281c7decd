/**
 * Runge_Kutta4.h -- fourth-order Runge-Kutta with the CacheOperator
 * (Runge_Kutta4.h, Runge_Kutta4.cpp:23-137), run on the GPU.
 *
 * moveParticles(endTime) advances while currentTime < endTime, as the
 * reference does, but every step -- the adaptive dt test, four fused force +
 * substep launches, the final combine -- runs on the device copy of the
 * cloud (CUDA-graph-captured where dt is fixed).  The ForceArray is folded
 * into one parameter block (Force::addDeviceParams); x, y, Vx, Vy, charge
 * and mass are uploaded at the start of the call and x, y, Vx, Vy
 * downloaded at its end, so the caller's Cloud is current on return (the
 * reference's driver writes it out next, driver.cpp:448-449).
 *
 * Thermal kicks are keyed by the device's step counter, which carries over
 * from one call to the next.
 */
#ifndef RUNGA_KUTTA4_H
#define RUNGA_KUTTA4_H

#include "Integrator.h"

class Runge_Kutta4 : public Integrator {
public:
    Runge_Kutta4(Cloud *const C, const ForceArray &FA, const double timeStep, const double startTime);
    ~Runge_Kutta4() {}
    void moveParticles(const double endTime) override;

    /// Pair arithmetic: DM_FP64 (default) or DM_FP32C.
    void setPrecision(int precision) { precision_ = precision; }
    /// false: fixed dt = timeStep (no modifyTimeStep), as in the fixed-step
    /// benchmarks; true (default): the reference's adaptive dt.
    void setAdaptiveTimeStep(bool on) { adaptive_ = on; }
    /// RK4 steps taken so far.
    long long stepsTaken() const { return steps_; }

private:
    int precision_ = DM_FP64;
    bool adaptive_ = true;
    long long steps_ = 0;
    dm_force_params last_{};  // parameters the device copy holds
    bool have_last_ = false;
};

#endif  // RUNGA_KUTTA4_H
