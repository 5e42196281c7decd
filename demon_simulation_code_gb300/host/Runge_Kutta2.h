/**
 * Runge_Kutta2.h -- second-order Runge-Kutta, the midpoint method
 * (Runge_Kutta2.h, Runge_Kutta2.cpp:23-78), run on the GPU like
 * Runge_Kutta4: stage 1 at (x, Vx, t), CacheOperator::operation2 to the
 * midpoint, stage 2 there at t + dt/2, then Vx += k2, x += l2; adaptive dt
 * as the reference's (modifyTimeStep before every step).
 */
#ifndef RUNGA_KUTTA2_H
#define RUNGA_KUTTA2_H

#include "Runge_Kutta4.h"

class Runge_Kutta2 : public DeviceIntegrator {
public:
    Runge_Kutta2(Cloud *const C, const ForceArray &FA, const double timeStep, const double startTime)
        : DeviceIntegrator(C, FA, timeStep, startTime, 2) {}
    ~Runge_Kutta2() {}
};

#endif  // RUNGA_KUTTA2_H
