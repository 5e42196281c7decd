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

/**
 * The device-stepped integrators' shared machinery (no reference
 * counterpart: the reference's Runge_Kutta2 and Runge_Kutta4 each loop on
 * the host).  moveParticles(endTime) of the subclasses runs their order's
 * stages on the device.
 */
class DeviceIntegrator : public Integrator {
public:
    DeviceIntegrator(Cloud *const C, const ForceArray &FA, const double timeStep, const double startTime, int order)
        : Integrator(C, FA, timeStep, startTime), order_(order) {}
    void moveParticles(const double endTime) override;

    /// Pair arithmetic: DM_FP64 (default) or DM_FP32C.
    void setPrecision(int precision) { precision_ = precision; }
    /// false: fixed dt = timeStep (no modifyTimeStep), as in the fixed-step
    /// benchmarks; true (default): the reference's adaptive dt.
    void setAdaptiveTimeStep(bool on) { adaptive_ = on; }
    /// Steps taken so far.
    long long stepsTaken() const { return steps_; }

private:
    int order_;
    int precision_ = DM_FP64;
    bool adaptive_ = true;
    long long steps_ = 0;
    dm_force_params last_{};  // parameters the device copy holds
    bool have_last_ = false;
};

class Runge_Kutta4 : public DeviceIntegrator {
public:
    Runge_Kutta4(Cloud *const C, const ForceArray &FA, const double timeStep, const double startTime)
        : DeviceIntegrator(C, FA, timeStep, startTime, 4) {}
    ~Runge_Kutta4() {}
};

#endif  // RUNGA_KUTTA4_H
