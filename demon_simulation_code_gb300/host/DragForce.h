/**
 * DragForce.h -- Epstein drag F = dragConst * m * v with dragConst = -gamma,
 * on the substep's velocities (DragForce.h:16-17, DragForce.cpp:13-55).
 */
#ifndef DRAGFORCE_H
#define DRAGFORCE_H

#include "Force.h"

class DragForce : public DeviceForce {
public:
    DragForce(Cloud *const myCloud, const double gamma) : DeviceForce(myCloud), dragConst(-gamma) {}
    ~DragForce() {}
    void writeForce(fitsfile *const file, int *const error) const override;
    void readForce(fitsfile *const file, int *const error) override;
    bool addDeviceParams(dm_force_params &p) const override;

protected:
    double dragConst;  //!< -gamma [Hz]
};

#endif  // DRAGFORCE_H
