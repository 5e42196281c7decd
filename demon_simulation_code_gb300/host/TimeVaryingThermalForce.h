/**
 * TimeVaryingThermalForce.h -- ThermalForce with heatVal = scale*t + offset
 * at every substep's time (TimeVaryingThermalForce.h,
 * TimeVaryingThermalForce.cpp:14-42); draws on stream substep + 32.  Its
 * FITS entry sets both the ThermalForce and the TimeVaryingThermalForce
 * flags, as the reference's.
 */
#ifndef TIMEVARYINGTHERMALFORCE_H
#define TIMEVARYINGTHERMALFORCE_H

#include "ThermalForce.h"

class TimeVaryingThermalForce : public ThermalForce {
public:
    TimeVaryingThermalForce(Cloud *const C, const double scale, const double offset, const int mode = 0,
                            const uint64_t seed = 0)
        : ThermalForce(C, offset, mode, seed), heatValScale(scale), heatValOffset(offset) {}
    ~TimeVaryingThermalForce() {}
    void writeForce(fitsfile *const file, int *const error) const override;
    void readForce(fitsfile *const file, int *const error) override;
    bool addDeviceParams(dm_force_params &p) const override;

private:
    double heatValScale;   //!< [N/s]
    double heatValOffset;  //!< [N]
};

#endif  // TIMEVARYINGTHERMALFORCE_H
