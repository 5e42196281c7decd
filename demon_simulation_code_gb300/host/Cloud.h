/**
 * Cloud.h -- the dust cloud, with the reference's public interface
 * (Cloud.h:16-87): particle count, raw FP64 arrays owned by the cloud, the
 * Runge-Kutta tidbit arrays, the stage caches, the physical constants and
 * the grid / file initialisers.
 *
 * GB300 layout: the host arrays are the caller's view.  Runge_Kutta4 keeps a
 * device copy of the cloud (structure-of-arrays in HBM) for the whole run,
 * uploads x, y, Vx, Vy, charge and mass at the start of each
 * moveParticles() and downloads x, y, Vx, Vy at its end, so the host arrays
 * are current whenever control is back with the caller.  The k/l/m/n tidbits
 * and the caches are filled only by host-side calls (CacheOperator and the
 * per-force force1..4 evaluations); the device step keeps its own.
 *
 * Differences from the reference:
 *  - the caches are plain double[n] (the reference packs them in SIMD
 *    vectors of n/2);
 *  - any n >= 1 is accepted (the reference needs even n, SIMD pairs);
 *  - output uses this library's FITS subset (FitsLite.h).
 */
#ifndef CLOUD_H
#define CLOUD_H

#include "Device.h"  // demon_gb300::Error, thrown by the device-backed calls
#include "FitsLite.h"
#include "RandomNumbers.h"
#include "demon_gb300.h"

typedef int cloud_index;  //!< Parallel.h:19 (OpenMP builds)

class Cloud {
public:
    Cloud(const cloud_index numPar);
    ~Cloud();

    const cloud_index n;                                    //!< Number of particles
    double *const x, *const y, *const Vx, *const Vy;       //!< current positions and velocities
    double *const charge, *const mass;                     //!< particle charges [C] and masses [kg]
    double *const k1, *const k2, *const k3, *const k4;     //!< velocity-x RK tidbits
    double *const l1, *const l2, *const l3, *const l4;     //!< position-x RK tidbits
    double *const m1, *const m2, *const m3, *const m4;     //!< velocity-y RK tidbits
    double *const n1, *const n2, *const n3, *const n4;     //!< position-y RK tidbits
    double *const forceX, *const forceY;                   //!< force on particles
    double *const xCache, *const yCache, *const VxCache, *const VyCache;  //!< stage 2-4 inputs
    RandomNumbers rands;  //!< for charge / mass initialisation

    static double interParticleSpacing;       //!< grid spacing [m]
    static const double electronCharge;       //!< [C]
    static const double epsilon0;             //!< [F/m]
    static const double particleRadius;       //!< [m]
    static double dustParticleMassDensity;    //!< [kg/m^3]
    static double justX, justY;               //!< grid centre offset [m]
    static double velX, velY;                 //!< initial velocity [m/s]

    void writeCloudSetup(fitsfile *const file, int &error) const;
    void writeTimeStep(fitsfile *const file, int &error, double currentTime) const;

    static Cloud *const initializeGrid(const cloud_index numParticles, cloud_index row_x_particles,
                                       cloud_index row_y_particles, const double rMean, const double rSigma,
                                       const double qMean, const double qSigma);
    static Cloud *const initializeFromFile(fitsfile *const file, int &error, double *const currentTime);

    /// Device copy used by Runge_Kutta4 (created on first use).
    dm_cloud *deviceState();
    /// Second device copy used by the per-force force1..4 evaluations, so
    /// that they never disturb the integrator's state.
    dm_cloud *deviceScratch();

private:
    void initCharge(const double qMean, const double qSigma);
    void initMass(const double rMean, const double rSigma);
    dm_cloud *state_ = nullptr;
    dm_cloud *scratch_ = nullptr;
    Cloud(const Cloud &) = delete;
    Cloud &operator=(const Cloud &) = delete;
};

#endif  // CLOUD_H
