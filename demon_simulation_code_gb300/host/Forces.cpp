/**
 * Forces.cpp -- the GPU-backed forces: per-force substep evaluation, FITS
 * keys, and their parameters in the fused device kernel.
 *
 * FITS keys follow the reference's writeForce/readForce: FORCES (bitmask,
 * e.g. ConfinementForce.cpp:60-84), confineConst, confineConstX/Y,
 * dragConst, shieldingConstant, heatingValue.  The reference's other forces
 * are in OtherForces.cpp.
 */
#include <vector>

#include "ConfinementForce.h"
#include "Device.h"
#include "DragForce.h"
#include "RectConfinementForce.h"
#include "ShieldedCoulombForce.h"
#include "ThermalForce.h"

namespace F = demon_gb300::fits;

int DeviceForce::precision = DM_FP64;

void DeviceForce::evaluate(int stage, double currentTime) {
    dm_force_params p{};
    if (!addDeviceParams(p))
        throw demon_gb300::Error(DM_ERR_UNSUPPORTED, "force cannot be evaluated on the device");
    dm_ctx *ctx = demon_gb300::context();
    dm_cloud *s = cloud->deviceScratch();
    const bool base = (stage == 1);
    demon_gb300::check(dm_cloud_set_charge_mass(s, cloud->charge, cloud->mass), ctx, "dm_cloud_set_charge_mass");
    demon_gb300::check(dm_cloud_upload(s, base ? cloud->x : cloud->xCache, base ? cloud->y : cloud->yCache,
                                       base ? cloud->Vx : cloud->VxCache, base ? cloud->Vy : cloud->VyCache),
                       ctx, "dm_cloud_upload");
    demon_gb300::check(dm_cloud_set_forces(s, &p), ctx, "dm_cloud_set_forces");
    demon_gb300::check(dm_cloud_set_step_counter(s, step), ctx, "dm_cloud_set_step_counter");
    demon_gb300::check(dm_cloud_set_time(s, currentTime), ctx, "dm_cloud_set_time");
    std::vector<double> fx((size_t)cloud->n), fy((size_t)cloud->n);
    demon_gb300::check(dm_cloud_eval_forces_stage(s, precision, stage, fx.data(), fy.data()), ctx,
                       "dm_cloud_eval_forces_stage");
    for (cloud_index i = 0; i < cloud->n; i++) {
        cloud->forceX[i] += fx[(size_t)i];
        cloud->forceY[i] += fy[(size_t)i];
    }
    if (stage == 4) step++;
}

void DeviceForce::addFlag(fitsfile *const file, force_flags flag, int *const error) {
    if (*error) return;
    int st = 0;
    long flags = F::read_key_long(file, "FORCES", st);
    if (st) flags = 0;
    F::write_key_long(file, "FORCES", flags | flag, "Force configuration", *error);
}

// --- ConfinementForce ------------------------------------------------------

void ConfinementForce::writeForce(fitsfile *const file, int *const error) const {
    addFlag(file, ConfinementForceFlag, error);
    F::write_key_dbl(file, "confineConst", confine, "[V/m^2] (ConfinementForce)", *error);
}

void ConfinementForce::readForce(fitsfile *const file, int *const error) {
    confine = F::read_key_dbl(file, "confineConst", *error);
}

bool ConfinementForce::addDeviceParams(dm_force_params &p) const {
    // the device's ConfinementForceVoid term uses the same constant
    if ((p.flags & DM_CONFINEMENT_VOID_FORCE) && !(p.flags & DM_CONFINEMENT_FORCE) && p.confine != confine)
        return false;
    p.confine = (p.flags & DM_CONFINEMENT_FORCE) ? p.confine + confine : confine;
    p.flags |= DM_CONFINEMENT_FORCE;
    return true;
}

// --- RectConfinementForce --------------------------------------------------

void RectConfinementForce::writeForce(fitsfile *const file, int *const error) const {
    addFlag(file, RectConfinementForceFlag, error);
    F::write_key_dbl(file, "confineConstX", confineX, "[V/m^2] (RectConfinementForce)", *error);
    F::write_key_dbl(file, "confineConstY", confineY, "[V/m^2] (RectConfinementForce)", *error);
}

void RectConfinementForce::readForce(fitsfile *const file, int *const error) {
    confineX = F::read_key_dbl(file, "confineConstX", *error);
    confineY = F::read_key_dbl(file, "confineConstY", *error);
}

bool RectConfinementForce::addDeviceParams(dm_force_params &p) const {
    const bool had = (p.flags & DM_RECT_CONFINEMENT_FORCE) != 0;
    p.confine_x = had ? p.confine_x + confineX : confineX;
    p.confine_y = had ? p.confine_y + confineY : confineY;
    p.flags |= DM_RECT_CONFINEMENT_FORCE;
    return true;
}

// --- DragForce -------------------------------------------------------------

void DragForce::writeForce(fitsfile *const file, int *const error) const {
    addFlag(file, DragForceFlag, error);
    F::write_key_dbl(file, "dragConst", dragConst, "[Hz] (DragForce)", *error);
}

void DragForce::readForce(fitsfile *const file, int *const error) {
    dragConst = F::read_key_dbl(file, "dragConst", *error);
}

bool DragForce::addDeviceParams(dm_force_params &p) const {
    p.gamma = (p.flags & DM_DRAG_FORCE) ? p.gamma - dragConst : -dragConst;
    p.flags |= DM_DRAG_FORCE;
    return true;
}

// --- ShieldedCoulombForce --------------------------------------------------

void ShieldedCoulombForce::writeForce(fitsfile *const file, int *const error) const {
    addFlag(file, ShieldedCoulombForceFlag, error);
    F::write_key_dbl(file, "shieldingConstant", shielding, "[m^-1] (ShieldedCoulombForce)", *error);
}

void ShieldedCoulombForce::readForce(fitsfile *const file, int *const error) {
    shielding = F::read_key_dbl(file, "shieldingConstant", *error);
}

bool ShieldedCoulombForce::addDeviceParams(dm_force_params &p) const {
    if (p.flags & DM_SHIELDED_COULOMB_FORCE) return false;  // one pair force per kernel
    p.flags |= DM_SHIELDED_COULOMB_FORCE;
    p.shielding = shielding;
    return true;
}

// --- ThermalForce ----------------------------------------------------------

void ThermalForce::writeForce(fitsfile *const file, int *const error) const {
    addFlag(file, ThermalForceFlag, error);
    F::write_key_dbl(file, "heatingValue", heatVal, "[N] (ThermalForce)", *error);
}

void ThermalForce::readForce(fitsfile *const file, int *const error) {
    heatVal = F::read_key_dbl(file, "heatingValue", *error);
}

bool ThermalForce::addDeviceParams(dm_force_params &p) const {
    if (p.flags & DM_THERMAL_FORCE) return false;
    // every thermal force draws with one generator key and form
    if ((p.flags & (DM_THERMAL_LOCALIZED_FORCE | DM_TIME_VARYING_THERMAL_FORCE)) &&
        (p.thermal_mode != mode || p.seed != seed))
        return false;
    p.flags |= DM_THERMAL_FORCE;
    p.heat = heatVal;
    p.thermal_mode = mode;
    p.seed = seed;
    return true;
}
