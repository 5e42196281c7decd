/**
 * ShieldedCoulombForce.h -- the Yukawa pair force
 *   F_ij = q_i q_j / (4 pi eps0) (1 + kappa r) e^{-kappa r} (r_i - r_j) / r^3
 * for pairs with kappa r < 10 (ShieldedCoulombForce.h,
 * ShieldedCoulombForce.cpp:37-237).  On the device this is the all-pairs
 * tiled kernel; the SIMD and lock machinery of the reference has no
 * counterpart.
 */
#ifndef SHIELDEDCOULOMBFORCE_H
#define SHIELDEDCOULOMBFORCE_H

#include "Force.h"

class ShieldedCoulombForce : public DeviceForce {
public:
    ShieldedCoulombForce(Cloud *const C, const double shieldingConstant)
        : DeviceForce(C), shielding(shieldingConstant) {}
    ~ShieldedCoulombForce() {}
    void writeForce(fitsfile *const file, int *const error) const override;
    void readForce(fitsfile *const file, int *const error) override;
    bool addDeviceParams(dm_force_params &p) const override;

private:
    double shielding;  //!< inverse shielding length kappa [1/m]
};

#endif  // SHIELDEDCOULOMBFORCE_H
