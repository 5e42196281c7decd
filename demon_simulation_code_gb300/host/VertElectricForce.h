/**
 * VertElectricForce.h -- F_y += q*E*exp(y/d) (VertElectricForce.h,
 * VertElectricForce.cpp:13-53).
 */
#ifndef VERTELECTRICFORCE_H
#define VERTELECTRICFORCE_H

#include "Force.h"

class VertElectricForce : public DeviceForce {
public:
    VertElectricForce(Cloud *const C, double vertElectricField, double vertDecay)
        : DeviceForce(C), vertElectric(vertElectricField), vertDec(vertDecay) {}
    ~VertElectricForce() {}
    void writeForce(fitsfile *const file, int *const error) const override;
    void readForce(fitsfile *const file, int *const error) override;
    bool addDeviceParams(dm_force_params &p) const override;

private:
    double vertElectric;  //!< [V/m^2]
    double vertDec;       //!< [m]
};

#endif  // VERTELECTRICFORCE_H
