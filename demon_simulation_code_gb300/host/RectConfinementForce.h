/**
 * RectConfinementForce.h -- F = (q * confineX * x, q * confineY * y)
 * (RectConfinementForce.h / RectConfinementForce.cpp:13-59).
 */
#ifndef RECTCONFINEMENTFORCE_H
#define RECTCONFINEMENTFORCE_H

#include "Force.h"

class RectConfinementForce : public DeviceForce {
public:
    RectConfinementForce(Cloud *const C, double confineConstX, double confineConstY)
        : DeviceForce(C), confineX(confineConstX), confineY(confineConstY) {}
    ~RectConfinementForce() {}
    void writeForce(fitsfile *const file, int *const error) const override;
    void readForce(fitsfile *const file, int *const error) override;
    bool addDeviceParams(dm_force_params &p) const override;

private:
    double confineX;  //!< x-direction strength [V/m^2]
    double confineY;  //!< y-direction strength [V/m^2]
};

#endif  // RECTCONFINEMENTFORCE_H
