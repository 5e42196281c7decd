/**
 * Operator.h -- an operation applied between RK substeps (Operator.h:14-47).
 */
#ifndef OPERATOR_H
#define OPERATOR_H

#include "Cloud.h"

class Operator {
public:
    Cloud *const cloud;  //!< the dust cloud
    Operator(Cloud *const C) : cloud(C) {}
    virtual ~Operator() {}
    virtual void operation1(const double currentTime) = 0;
    virtual void operation2(const double currentTime) = 0;
    virtual void operation3(const double currentTime) = 0;
    virtual void operation4(const double currentTime) = 0;
};

#endif  // OPERATOR_H
