/**
 * GravitationalForce.h -- F_y += m*g (GravitationalForce.h,
 * GravitationalForce.cpp:13-50; the sign is the caller's g).
 */
#ifndef GRAVITATIONALFORCE_H
#define GRAVITATIONALFORCE_H

#include "Force.h"

class GravitationalForce : public DeviceForce {
public:
    GravitationalForce(Cloud *const C, const double gravitationalField)
        : DeviceForce(C), gravitational(gravitationalField) {}
    ~GravitationalForce() {}
    void writeForce(fitsfile *const file, int *const error) const override;
    void readForce(fitsfile *const file, int *const error) override;
    bool addDeviceParams(dm_force_params &p) const override;

private:
    double gravitational;  //!< [m/s^2]
};

#endif  // GRAVITATIONALFORCE_H
