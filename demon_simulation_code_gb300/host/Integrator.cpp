/**
 * Integrator.cpp -- base integrator state and the adaptive dt test.
 */
#include "Integrator.h"

#include "CacheOperator.h"
#include "Device.h"

Integrator::Integrator(Cloud *const C, const ForceArray &FA, const double timeStep, double startTime)
    : currentTime(startTime), cloud(C), forces(FA), init_dt(timeStep), operations{{new CacheOperator(C)}} {}

Integrator::~Integrator() {
    for (Operator *const op : operations) delete op;
}

const double Integrator::modifyTimeStep(float currentDist, double currentTimeStep) const {
    dm_ctx *ctx = demon_gb300::context();
    dm_cloud *d = cloud->deviceScratch();
    demon_gb300::check(dm_cloud_upload(d, cloud->x, cloud->y, cloud->Vx, cloud->Vy), ctx, "dm_cloud_upload");
    float minDist = 0.0f;
    double dt0 = 0.0;
    demon_gb300::check(dm_cloud_modify_timestep(d, currentTimeStep, &minDist, &dt0), ctx,
                       "dm_cloud_modify_timestep");
    // tryToReduceTimeStep (Integrator.cpp:144-155): while a checked pair is
    // within the distance, distance /= 10 (FP32) and dt /= 10
    float dist = currentDist;
    double dt = currentTimeStep;
    for (int k = 0; minDist <= dist; k++) {
        if (k > 64 || !(minDist > 0.0f))
            throw demon_gb300::Error(DM_ERR_NUMERIC, "modifyTimeStep: two particles share a position");
        dist /= 10.0f;
        dt /= 10.0f;
    }
    return dt;
}
