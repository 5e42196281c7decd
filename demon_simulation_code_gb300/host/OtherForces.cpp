/**
 * OtherForces.cpp -- the reference's forces beyond confinement, drag, the
 * shielded Coulomb pair force and ThermalForce: FITS keys and their
 * parameters in the fused device kernel.
 *
 * FITS keys and FORCES bits follow each force's writeForce/readForce in the
 * reference (e.g. DrivingForce.cpp:63-109).  A force whose parameters cannot
 * share the device parameter block with what is already there (a second
 * force of the same kind) returns false from addDeviceParams, and
 * Runge_Kutta4 refuses the ForceArray.
 */
#include "ConfinementForceVoid.h"
#include "Device.h"
#include "DrivingForce.h"
#include "ElectricForce.h"
#include "GravitationalForce.h"
#include "MagneticForce.h"
#include "RotationalForce.h"
#include "ThermalForceLocalized.h"
#include "TimeVaryingDragForce.h"
#include "TimeVaryingThermalForce.h"
#include "VertElectricForce.h"

namespace F = demon_gb300::fits;

namespace {

// Thermal draws of every thermal force share one generator key and form.
bool add_thermal_key(dm_force_params &p, int mode, uint64_t seed) {
    if (p.flags & (DM_THERMAL_FORCE | DM_THERMAL_LOCALIZED_FORCE | DM_TIME_VARYING_THERMAL_FORCE))
        if (p.thermal_mode != mode || p.seed != seed) return false;
    p.thermal_mode = mode;
    p.seed = seed;
    return true;
}

}  // namespace

// --- ConfinementForceVoid (ConfinementForceVoid.cpp:57-88) ----------------

void ConfinementForceVoid::writeForce(fitsfile *const file, int *const error) const {
    ConfinementForce::writeForce(file, error);
    addFlag(file, ConfinementForceFlag | ConfinementForceVoidFlag, error);
    F::write_key_dbl(file, "decay", decay, "[m^-1] (ConfinementForceVoid)", *error);
}

void ConfinementForceVoid::readForce(fitsfile *const file, int *const error) {
    ConfinementForce::readForce(file, error);
    decay = F::read_key_dbl(file, "decay", *error);
}

bool ConfinementForceVoid::addDeviceParams(dm_force_params &p) const {
    if (p.flags & DM_CONFINEMENT_VOID_FORCE) return false;
    // its confinement term shares the constant with a ConfinementForce
    if ((p.flags & DM_CONFINEMENT_FORCE) && p.confine != confine) return false;
    p.confine = confine;
    p.void_decay = decay;
    p.flags |= DM_CONFINEMENT_VOID_FORCE;
    return true;
}

// --- DrivingForce (DrivingForce.cpp:63-109) -------------------------------

void DrivingForce::writeForce(fitsfile *const file, int *const error) const {
    addFlag(file, DrivingForceFlag, error);
    F::write_key_dbl(file, "drivingAmplitude", amplitude, "[N] (DrivingForce)", *error);
    F::write_key_dbl(file, "drivingConst", driveConst, "[m^2] (DrivingForce)", *error);
    F::write_key_dbl(file, "drivingShift", shift, "[m] (DrivingForce)", *error);
}

void DrivingForce::readForce(fitsfile *const file, int *const error) {
    amplitude = F::read_key_dbl(file, "drivingAmplitude", *error);
    driveConst = F::read_key_dbl(file, "drivingConst", *error);
    shift = F::read_key_dbl(file, "drivingShift", *error);
}

bool DrivingForce::addDeviceParams(dm_force_params &p) const {
    if (p.flags & DM_DRIVING_FORCE) return false;
    p.drive_const = -driveConst;
    p.drive_amplitude = amplitude;
    p.drive_shift = shift;
    p.flags |= DM_DRIVING_FORCE;
    return true;
}

// --- MagneticForce (MagneticForce.cpp:56-95) ------------------------------

void MagneticForce::writeForce(fitsfile *const file, int *const error) const {
    addFlag(file, MagneticForceFlag, error);
    F::write_key_dbl(file, "magneticField", BField, "[T] (MagneticForce)", *error);
}

void MagneticForce::readForce(fitsfile *const file, int *const error) {
    BField = F::read_key_dbl(file, "magneticField", *error);
}

bool MagneticForce::addDeviceParams(dm_force_params &p) const {
    if (p.flags & DM_MAGNETIC_FORCE) return false;
    p.magnetic = BField;
    p.flags |= DM_MAGNETIC_FORCE;
    return true;
}

// --- RotationalForce (RotationalForce.cpp:68-114) -------------------------

void RotationalForce::writeForce(fitsfile *const file, int *const error) const {
    addFlag(file, RotationalForceFlag, error);
    F::write_key_dbl(file, "rotationalConst", rotationalConst, "[N] (RotationalForce)", *error);
    F::write_key_dbl(file, "innerRadius", innerRad, "[m] (RotationalForce)", *error);
    F::write_key_dbl(file, "outerRadius", outerRad, "[m] (RotationalForce)", *error);
}

void RotationalForce::readForce(fitsfile *const file, int *const error) {
    rotationalConst = F::read_key_dbl(file, "rotationalConst", *error);
    innerRad = F::read_key_dbl(file, "innerRadius", *error);
    outerRad = F::read_key_dbl(file, "outerRadius", *error);
}

bool RotationalForce::addDeviceParams(dm_force_params &p) const {
    if (p.flags & DM_ROTATIONAL_FORCE) return false;
    p.rot_rmin = innerRad;
    p.rot_rmax = outerRad;
    p.rot_const = rotationalConst;
    p.flags |= DM_ROTATIONAL_FORCE;
    return true;
}

// --- ThermalForceLocalized (ThermalForceLocalized.cpp:151-197) ------------

void ThermalForceLocalized::writeForce(fitsfile *const file, int *const error) const {
    addFlag(file, ThermalForceLocalizedFlag, error);
    F::write_key_dbl(file, "heatingValue1", heatVal1, "[N] (ThermalForceLocalized)", *error);
    F::write_key_dbl(file, "heatingValue2", heatVal2, "[N] (ThermalForceLocalized)", *error);
    F::write_key_dbl(file, "heatingRadius", heatingRadius, "[m] (ThermalForceLocalized)", *error);
}

void ThermalForceLocalized::readForce(fitsfile *const file, int *const error) {
    heatVal1 = F::read_key_dbl(file, "heatingValue1", *error);
    heatVal2 = F::read_key_dbl(file, "heatingValue2", *error);
    heatingRadius = F::read_key_dbl(file, "heatingRadius", *error);
}

bool ThermalForceLocalized::addDeviceParams(dm_force_params &p) const {
    if ((p.flags & DM_THERMAL_LOCALIZED_FORCE) || !add_thermal_key(p, mode, seed)) return false;
    p.heat_in = heatVal1;
    p.heat_out = heatVal2;
    p.heat_radius = heatingRadius;
    p.flags |= DM_THERMAL_LOCALIZED_FORCE;
    return true;
}

// --- TimeVaryingDragForce (TimeVaryingDragForce.cpp:42-77) ----------------

void TimeVaryingDragForce::writeForce(fitsfile *const file, int *const error) const {
    DragForce::writeForce(file, error);
    addFlag(file, DragForceFlag | TimeVaryingDragForceFlag, error);
    F::write_key_dbl(file, "TVDragScaleConst", scaleConst, "[Hz/s] (TimeVaryingDragForce)", *error);
    F::write_key_dbl(file, "TVDragOffsetConst", offsetConst, "[Hz] (TimeVaryingDragForce)", *error);
}

void TimeVaryingDragForce::readForce(fitsfile *const file, int *const error) {
    DragForce::readForce(file, error);
    scaleConst = F::read_key_dbl(file, "TVDragScaleConst", *error);
    offsetConst = F::read_key_dbl(file, "TVDragOffsetConst", *error);
}

bool TimeVaryingDragForce::addDeviceParams(dm_force_params &p) const {
    if (p.flags & DM_TIME_VARYING_DRAG_FORCE) return false;
    p.drag_scale = scaleConst;
    p.drag_offset = offsetConst;
    p.flags |= DM_TIME_VARYING_DRAG_FORCE;
    return true;
}

// --- TimeVaryingThermalForce (TimeVaryingThermalForce.cpp:44-79) ----------

void TimeVaryingThermalForce::writeForce(fitsfile *const file, int *const error) const {
    ThermalForce::writeForce(file, error);
    addFlag(file, ThermalForceFlag | TimeVaryingThermalForceFlag, error);
    F::write_key_dbl(file, "heatingValueScale", heatValScale, "[N/s] (TimeVaryingThermalForce)", *error);
    F::write_key_dbl(file, "heatingValueOffset", heatValOffset, "[N] (TimeVaryingThermalForce)", *error);
}

void TimeVaryingThermalForce::readForce(fitsfile *const file, int *const error) {
    ThermalForce::readForce(file, error);
    heatValScale = F::read_key_dbl(file, "heatingValueScale", *error);
    heatValOffset = F::read_key_dbl(file, "heatingValueOffset", *error);
}

bool TimeVaryingThermalForce::addDeviceParams(dm_force_params &p) const {
    if ((p.flags & DM_TIME_VARYING_THERMAL_FORCE) || !add_thermal_key(p, mode, seed)) return false;
    p.heat_scale = heatValScale;
    p.heat_offset = heatValOffset;
    p.flags |= DM_TIME_VARYING_THERMAL_FORCE;
    return true;
}

// --- ElectricForce (ElectricForce.cpp:64-106) -----------------------------

void ElectricForce::writeForce(fitsfile *const file, int *const error) const {
    addFlag(file, ElectricForceFlag, error);
    F::write_key_dbl(file, "ElectricFieldStrength", electric, "[V/m^2] (ElectricForce)", *error);
    F::write_key_dbl(file, "plasmaRadius", radius, "[m] (ElectricForce)", *error);
}

void ElectricForce::readForce(fitsfile *const file, int *const error) {
    electric = F::read_key_dbl(file, "electricFieldStrength", *error);
    radius = F::read_key_dbl(file, "plasmaRadius", *error);
}

bool ElectricForce::addDeviceParams(dm_force_params &p) const {
    if (p.flags & DM_ELECTRIC_FORCE) return false;
    p.electric = electric;
    p.electric_radius = radius;
    p.flags |= DM_ELECTRIC_FORCE;
    return true;
}

// --- GravitationalForce (GravitationalForce.cpp:52-92) --------------------

void GravitationalForce::writeForce(fitsfile *const file, int *const error) const {
    addFlag(file, GravitationalForceFlag, error);
    F::write_key_dbl(file, "GravitationalFieldStrength", gravitational, "[m/s^2] (GravitationalForce)",
                     *error);
}

void GravitationalForce::readForce(fitsfile *const file, int *const error) {
    gravitational = F::read_key_dbl(file, "gravitationalFieldStrength", *error);
}

bool GravitationalForce::addDeviceParams(dm_force_params &p) const {
    if (p.flags & DM_GRAVITATIONAL_FORCE) return false;
    p.gravity = gravitational;
    p.flags |= DM_GRAVITATIONAL_FORCE;
    return true;
}

// --- VertElectricForce (VertElectricForce.cpp:55-98) ----------------------

void VertElectricForce::writeForce(fitsfile *const file, int *const error) const {
    addFlag(file, VertElectricForceFlag, error);
    F::write_key_dbl(file, "VertElectricFieldStrength", vertElectric, "[V/m^2] (VertElectricForce)", *error);
    F::write_key_dbl(file, "verticalDecay", vertDec, "[m] (VertElectricForce)", *error);
}

void VertElectricForce::readForce(fitsfile *const file, int *const error) {
    vertElectric = F::read_key_dbl(file, "vertElectricFieldStrength", *error);
    vertDec = F::read_key_dbl(file, "verticalDecay", *error);
}

bool VertElectricForce::addDeviceParams(dm_force_params &p) const {
    if (p.flags & DM_VERT_ELECTRIC_FORCE) return false;
    p.vert_electric = vertElectric;
    p.vert_decay = vertDec;
    p.flags |= DM_VERT_ELECTRIC_FORCE;
    return true;
}
