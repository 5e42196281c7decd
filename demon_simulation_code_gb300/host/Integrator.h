/**
 * Integrator.h -- the abstract time integrator (Integrator.h:17-38): cloud,
 * forces, initial time step, current time, the CacheOperator, and the
 * adaptive time-step test (Integrator.cpp:68-182).
 */
#ifndef INTEGRATOR_H
#define INTEGRATOR_H

#include <array>

#include "Cloud.h"
#include "Force.h"
#include "Operator.h"

class Integrator {
public:
    Integrator(Cloud *const C, const ForceArray &FA, const double timeStep, double startTime);
    virtual ~Integrator();
    double currentTime;
    virtual void moveParticles(const double endTime) = 0;

protected:
    Cloud *const cloud;
    const ForceArray &forces;
    const double init_dt;
    const std::array<Operator *const, 1> operations;

    /// The reference's dt reduction: dt / 10^k and distance / 10^k for the
    /// smallest k with every checked pair (the FP32 separations the
    /// reference visits, Integrator.cpp:90-131) farther apart than the
    /// reduced distance.  The separations come from the device copy of the
    /// cloud's current host positions; needs n % 4 == 0 (the reference reads
    /// past the arrays otherwise).  Throws where the reference would loop
    /// forever (two particles at one point).
    const double modifyTimeStep(float currentDist, double currentTimeStep) const;
};

#endif  // INTEGRATOR_H
