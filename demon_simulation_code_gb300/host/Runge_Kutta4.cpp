/**
 * Runge_Kutta4.cpp -- the device-stepped moveParticles of Runge_Kutta4 and
 * Runge_Kutta2.
 */
#include "Runge_Kutta4.h"

#include <cstring>
#include <string>
#include <typeinfo>

#include "Device.h"

void DeviceIntegrator::moveParticles(const double endTime) {
    if (!(currentTime < endTime)) return;
    dm_force_params p{};
    for (const Force *f : forces)
        if (!f->addDeviceParams(p))
            throw demon_gb300::Error(DM_ERR_UNSUPPORTED, std::string("moveParticles: ") + typeid(*f).name() +
                                                             " cannot run in the fused device step");
    dm_ctx *ctx = demon_gb300::context();
    dm_cloud *d = cloud->deviceState();
    demon_gb300::check(dm_cloud_set_charge_mass(d, cloud->charge, cloud->mass), ctx, "dm_cloud_set_charge_mass");
    demon_gb300::check(dm_cloud_upload(d, cloud->x, cloud->y, cloud->Vx, cloud->Vy), ctx, "dm_cloud_upload");
    if (!have_last_ || std::memcmp(&p, &last_, sizeof p) != 0) {  // new parameters drop captured graphs
        demon_gb300::check(dm_cloud_set_forces(d, &p), ctx, "dm_cloud_set_forces");
        last_ = p;
        have_last_ = true;
    }
    demon_gb300::check(dm_cloud_set_integrator(d, order_), ctx, "dm_cloud_set_integrator");
    int steps = 0;
    demon_gb300::check(dm_cloud_move_particles(d, endTime, init_dt, precision_, adaptive_ ? 1 : 0, &currentTime,
                                               &steps),
                       ctx, "dm_cloud_move_particles");
    steps_ += steps;
    demon_gb300::check(dm_cloud_download(d, cloud->x, cloud->y, cloud->Vx, cloud->Vy), ctx, "dm_cloud_download");
}
