/**
 * RotationalForce.h -- a shear layer: for rmin < r < rmax,
 * F += c*(-y, x)/r (RotationalForce.h, RotationalForce.cpp:13-66).
 */
#ifndef ROTATIONALFORCE_H
#define ROTATIONALFORCE_H

#include "Force.h"

class RotationalForce : public DeviceForce {
public:
    RotationalForce(Cloud *const C, const double rmin, const double rmax, const double rotConst)
        : DeviceForce(C), innerRad(rmin), outerRad(rmax), rotationalConst(rotConst) {}
    ~RotationalForce() {}
    void writeForce(fitsfile *const file, int *const error) const override;
    void readForce(fitsfile *const file, int *const error) override;
    bool addDeviceParams(dm_force_params &p) const override;

private:
    double innerRad;         //!< [m]
    double outerRad;         //!< [m]
    double rotationalConst;  //!< [N]
};

#endif  // ROTATIONALFORCE_H
