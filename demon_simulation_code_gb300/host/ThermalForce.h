/**
 * ThermalForce.h -- random thermal kicks, new ones at every RK substep
 * (ThermalForce.h, ThermalForce.cpp:42-140).
 *
 * The reference draws heatVal * U(0,1) * (cos t, sin t), t ~ U(0, 2 pi),
 * from a clock-seeded Mersenne Twister.  Here the draws come from a
 * counter-based generator (Philox4x32-10 keyed by `seed`, counter =
 * particle, RK step, substep), so runs are reproducible and every particle
 * draws independently on the device.  mode 0 is the reference's form; mode 1
 * draws Gaussian kicks N(0, heatVal^2) per axis.
 */
#ifndef THERMALFORCE_H
#define THERMALFORCE_H

#include "Force.h"

class ThermalForce : public DeviceForce {
public:
    ThermalForce(Cloud *const C, const double redFactor, const int mode = 0, const uint64_t seed = 0)
        : DeviceForce(C), heatVal(redFactor), mode(mode), seed(seed) {}
    ~ThermalForce() {}
    void writeForce(fitsfile *const file, int *const error) const override;
    void readForce(fitsfile *const file, int *const error) override;
    bool addDeviceParams(dm_force_params &p) const override;

protected:
    double heatVal;  //!< strength of the thermal force [N]
    int mode;        //!< 0: reference form, 1: Gaussian
    uint64_t seed;   //!< generator key
};

#endif  // THERMALFORCE_H
