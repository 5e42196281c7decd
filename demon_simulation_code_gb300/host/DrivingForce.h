/**
 * DrivingForce.h -- a travelling sinusoidal drive along x,
 * F_x = amplitude*sin(x*2pi/2mm - t*2pi*10Hz)*exp((d - d)/dampConst) with
 * d = x - shift (DrivingForce.h, DrivingForce.cpp:14-61).  As in the
 * reference the stored driveConst is -dampConst, and that is the value of its
 * FITS key.
 */
#ifndef DRIVINGFORCE_H
#define DRIVINGFORCE_H

#include "Force.h"

class DrivingForce : public DeviceForce {
public:
    DrivingForce(Cloud *const C, const double dampConst, const double amp, const double drivingShift)
        : DeviceForce(C), amplitude(amp), driveConst(-dampConst), shift(drivingShift) {}
    ~DrivingForce() {}
    void writeForce(fitsfile *const file, int *const error) const override;
    void readForce(fitsfile *const file, int *const error) override;
    bool addDeviceParams(dm_force_params &p) const override;

private:
    double amplitude;   //!< [N]
    double driveConst;  //!< -dampConst [m^2]
    double shift;       //!< [m]
};

#endif  // DRIVINGFORCE_H
