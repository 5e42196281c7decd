/**
 * ConfinementForce.h -- radial confinement F = q * confine * (x, y)
 * (ConfinementForce.h / ConfinementForce.cpp:13-54 in the reference).
 */
#ifndef CONFINEMENTFORCE_H
#define CONFINEMENTFORCE_H

#include "Force.h"

class ConfinementForce : public DeviceForce {
public:
    ConfinementForce(Cloud *const C, double confineConst) : DeviceForce(C), confine(confineConst) {}
    ~ConfinementForce() {}
    void writeForce(fitsfile *const file, int *const error) const override;
    void readForce(fitsfile *const file, int *const error) override;
    bool addDeviceParams(dm_force_params &p) const override;

protected:
    double confine;  //!< strength of the confinement [V/m^2]
};

#endif  // CONFINEMENTFORCE_H
