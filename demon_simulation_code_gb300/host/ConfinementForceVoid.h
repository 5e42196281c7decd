/**
 * ConfinementForceVoid.h -- the confinement force plus a central void,
 * F += q*(-decay)*exp(-decay*r)/r*(x, y) (ConfinementForceVoid.h,
 * ConfinementForceVoid.cpp:13-55).  Its FITS entry sets both the
 * ConfinementForce and the ConfinementForceVoid flags, as the reference's.
 */
#ifndef CONFINEMENTFORCEVOID_H
#define CONFINEMENTFORCEVOID_H

#include "ConfinementForce.h"

class ConfinementForceVoid : public ConfinementForce {
public:
    ConfinementForceVoid(Cloud *const C, double confineConst, double voidDecay)
        : ConfinementForce(C, confineConst), decay(voidDecay) {}
    ~ConfinementForceVoid() {}
    void writeForce(fitsfile *const file, int *const error) const override;
    void readForce(fitsfile *const file, int *const error) override;
    bool addDeviceParams(dm_force_params &p) const override;

private:
    double decay;  //!< decay constant of the void [m^-1]
};

#endif  // CONFINEMENTFORCEVOID_H
