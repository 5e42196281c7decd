/**
 * CacheOperator.h -- the RK4 substep inputs (CacheOperator.cpp:18-73):
 *   substep 2: cache = base + tidbit_1 / 2, substep 3: base + tidbit_2 / 2,
 *   substep 4: base + tidbit_3, for x (l), y (n), Vx (k), Vy (m).
 * On the host arrays of the cloud; the device step computes the same values
 * in its stage kernels.
 */
#ifndef CACHEOPERATOR_H
#define CACHEOPERATOR_H

#include "Operator.h"

class CacheOperator : public Operator {
public:
    CacheOperator(Cloud *const C) : Operator(C) {}
    ~CacheOperator() {}
    void operation1(const double currentTime) override;
    void operation2(const double currentTime) override;
    void operation3(const double currentTime) override;
    void operation4(const double currentTime) override;
};

#endif  // CACHEOPERATOR_H
