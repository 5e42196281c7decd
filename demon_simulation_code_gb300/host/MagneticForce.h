/**
 * MagneticForce.h -- F = q*(v x B) for B along z, on the substep's
 * velocities: F += q*B*(vy, -vx) (MagneticForce.h, MagneticForce.cpp:13-54).
 */
#ifndef MAGNETICFORCE_H
#define MAGNETICFORCE_H

#include "Force.h"

class MagneticForce : public DeviceForce {
public:
    MagneticForce(Cloud *const C, const double magneticField) : DeviceForce(C), BField(magneticField) {}
    ~MagneticForce() {}
    void writeForce(fitsfile *const file, int *const error) const override;
    void readForce(fitsfile *const file, int *const error) override;
    bool addDeviceParams(dm_force_params &p) const override;

private:
    double BField;  //!< [T]
};

#endif  // MAGNETICFORCE_H
