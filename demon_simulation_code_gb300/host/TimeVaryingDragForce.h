/**
 * TimeVaryingDragForce.h -- DragForce with dragConst = -(scale*t + offset)
 * at every substep's time (TimeVaryingDragForce.h,
 * TimeVaryingDragForce.cpp:13-40).  Its FITS entry sets both the DragForce
 * and the TimeVaryingDragForce flags, as the reference's.
 */
#ifndef TIMEVARYINGDRAGFORCE_H
#define TIMEVARYINGDRAGFORCE_H

#include "DragForce.h"

class TimeVaryingDragForce : public DragForce {
public:
    TimeVaryingDragForce(Cloud *const C, const double scale, const double offset)
        : DragForce(C, -offset), scaleConst(scale), offsetConst(offset) {}
    ~TimeVaryingDragForce() {}
    void writeForce(fitsfile *const file, int *const error) const override;
    void readForce(fitsfile *const file, int *const error) override;
    bool addDeviceParams(dm_force_params &p) const override;

private:
    double scaleConst;   //!< [Hz/s]
    double offsetConst;  //!< [Hz]
};

#endif  // TIMEVARYINGDRAGFORCE_H
