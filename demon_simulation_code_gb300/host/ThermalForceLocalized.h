/**
 * ThermalForceLocalized.h -- thermal kicks of scale heatVal1 inside
 * r < heatingRadius and heatVal2 outside, new ones at every RK substep
 * (ThermalForceLocalized.h, ThermalForceLocalized.cpp:14-133).  The draws
 * come from the counter-based generator of ThermalForce (stream substep +
 * 16, so both forces can be on together); mode 0 is the reference's
 * uniform-magnitude form, mode 1 Gaussian.
 */
#ifndef THERMALFORCELOCALIZED_H
#define THERMALFORCELOCALIZED_H

#include "Force.h"

class ThermalForceLocalized : public DeviceForce {
public:
    ThermalForceLocalized(Cloud *const C, const double thermRed1, const double thermRed2,
                          const double specifiedRadius, const int mode = 0, const uint64_t seed = 0)
        : DeviceForce(C), heatingRadius(specifiedRadius), heatVal1(thermRed1), heatVal2(thermRed2), mode(mode),
          seed(seed) {}
    ~ThermalForceLocalized() {}
    void writeForce(fitsfile *const file, int *const error) const override;
    void readForce(fitsfile *const file, int *const error) override;
    bool addDeviceParams(dm_force_params &p) const override;

private:
    double heatingRadius;  //!< [m]
    double heatVal1;       //!< inside [N]
    double heatVal2;       //!< outside [N]
    int mode;
    uint64_t seed;
};

#endif  // THERMALFORCELOCALIZED_H
