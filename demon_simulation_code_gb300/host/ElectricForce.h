/**
 * ElectricForce.h -- a radial field F = q*E*exp(r/(-R))*(x, y)
 * (ElectricForce.h, ElectricForce.cpp:13-62).
 */
#ifndef ELECTRICFORCE_H
#define ELECTRICFORCE_H

#include "Force.h"

class ElectricForce : public DeviceForce {
public:
    ElectricForce(Cloud *const C, double electricField, double plasmaRad)
        : DeviceForce(C), electric(electricField), radius(plasmaRad) {}
    ~ElectricForce() {}
    void writeForce(fitsfile *const file, int *const error) const override;
    void readForce(fitsfile *const file, int *const error) override;
    bool addDeviceParams(dm_force_params &p) const override;

private:
    double electric;  //!< [V/m^2]
    double radius;    //!< [m]
};

#endif  // ELECTRICFORCE_H
