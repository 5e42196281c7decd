// host_api_check.cpp -- drives the C++ host classes the way the reference's
// own code does, for tests/test_gpu_host.py.
//
//   host_api_check <in.bin> <out.bin> <mode> <nsteps> <dt> <precision> [basic|other]
//
// in.bin: int32 n, then x, y, vx, vy, q, m (n doubles each).  Forces
// "basic": Confinement(1e4), Drag(3), ShieldedCoulomb(5e3), Thermal(1e-16,
// mode 1, seed 5), from t = 0.  Forces "other": the reference's other
// forces around ShieldedCoulomb(5e3), from t = 0.3.  mode "fused":
// Runge_Kutta4::moveParticles with a fixed dt for nsteps steps.  mode
// "host": the same steps written out as the reference's
// Runge_Kutta4::moveParticles loop (Runge_Kutta4.cpp:23-137) over the
// per-force force1..4 calls and CacheOperator::operation1..4.  out.bin: x,
// y, vx, vy after the steps (n doubles each).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "CacheOperator.h"
#include "ConfinementForce.h"
#include "ConfinementForceVoid.h"
#include "DragForce.h"
#include "DrivingForce.h"
#include "ElectricForce.h"
#include "GravitationalForce.h"
#include "MagneticForce.h"
#include "RotationalForce.h"
#include "Runge_Kutta4.h"
#include "ShieldedCoulombForce.h"
#include "ThermalForce.h"
#include "ThermalForceLocalized.h"
#include "TimeVaryingDragForce.h"
#include "TimeVaryingThermalForce.h"
#include "VertElectricForce.h"

namespace {

void host_rk4(Cloud *c, const ForceArray &forces, CacheOperator &op, double t0, double dt, int nsteps) {
    const int n = c->n;
    double t = t0;
    double *K[4] = {c->k1, c->k2, c->k3, c->k4}, *L[4] = {c->l1, c->l2, c->l3, c->l4};
    double *M[4] = {c->m1, c->m2, c->m3, c->m4}, *N[4] = {c->n1, c->n2, c->n3, c->n4};
    for (int s = 0; s < nsteps; s++) {
        for (int k = 0; k < 4; k++) {
            const double tk = (k == 0) ? t : (k == 3 ? t + dt : t + dt / 2.0);
            if (k == 0) op.operation1(tk);
            if (k == 1) op.operation2(tk);
            if (k == 2) op.operation3(tk);
            if (k == 3) op.operation4(tk);
            for (Force *f : forces) {
                if (k == 0) f->force1(tk);
                if (k == 1) f->force2(tk);
                if (k == 2) f->force3(tk);
                if (k == 3) f->force4(tk);
            }
            const double *vx = (k == 0) ? c->Vx : c->VxCache;
            const double *vy = (k == 0) ? c->Vy : c->VyCache;
            for (int i = 0; i < n; i++) {
                K[k][i] = (dt * c->forceX[i]) / c->mass[i];
                L[k][i] = dt * vx[i];
                M[k][i] = (dt * c->forceY[i]) / c->mass[i];
                N[k][i] = dt * vy[i];
                c->forceX[i] = 0.0;
                c->forceY[i] = 0.0;
            }
        }
        // Runge_Kutta4.cpp:147-151: (a1 + (a2 + a3) * 2 + a4) / 6
        auto da = [](double a1, double a2, double a3, double a4) { return (a1 + ((a2 + a3) * 2.0 + a4)) / 6.0; };
        for (int i = 0; i < n; i++) {
            c->Vx[i] += da(c->k1[i], c->k2[i], c->k3[i], c->k4[i]);
            c->x[i] += da(c->l1[i], c->l2[i], c->l3[i], c->l4[i]);
            c->Vy[i] += da(c->m1[i], c->m2[i], c->m3[i], c->m4[i]);
            c->y[i] += da(c->n1[i], c->n2[i], c->n3[i], c->n4[i]);
        }
        t += dt;
    }
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 7 && argc != 8) {
        std::fprintf(stderr, "usage: %s in.bin out.bin fused|host nsteps dt fp64|fp32c [basic|other]\n", argv[0]);
        return 2;
    }
    const bool other = argc == 8 && std::string(argv[7]) == "other";
    FILE *in = std::fopen(argv[1], "rb");
    int n = 0;
    if (!in || std::fread(&n, sizeof n, 1, in) != 1 || n < 1) return 2;
    Cloud cloud(n);
    for (double *a : {cloud.x, cloud.y, cloud.Vx, cloud.Vy, cloud.charge, cloud.mass})
        if (std::fread(a, sizeof(double), (size_t)n, in) != (size_t)n) return 2;
    std::fclose(in);
    const std::string mode = argv[3];
    const int nsteps = std::atoi(argv[4]);
    const double dt = std::atof(argv[5]);
    const int prec = std::string(argv[6]) == "fp32c" ? DM_FP32C : DM_FP64;

    ConfinementForce conf(&cloud, 1e4);
    DragForce drag(&cloud, 3.0);
    ShieldedCoulombForce coul(&cloud, 5e3);
    ThermalForce therm(&cloud, 1e-16, 1, 5);
    // the reference's other forces, in driver.cpp:372-402 order
    ConfinementForceVoid cvoid(&cloud, 1e4, 400.0);
    DrivingForce drive(&cloud, 1e-5, 1e-15, 5e-4);
    MagneticForce mag(&cloud, 0.5);
    RotationalForce rot(&cloud, 2e-4, 1e-3, 1e-15);
    ThermalForceLocalized tloc(&cloud, 1e-16, 3e-16, 5e-4, 1, 5);
    TimeVaryingDragForce tvdrag(&cloud, -1.0, 3.0);
    TimeVaryingThermalForce tvtherm(&cloud, 1e-16, 1e-16, 1, 5);
    ElectricForce elec(&cloud, 1e3, 2e-3);
    GravitationalForce grav(&cloud, -1.0);
    VertElectricForce velec(&cloud, 1.0, 2e-3);
    const ForceArray forces = other ? ForceArray{&cvoid, &drive, &mag, &rot, &coul, &tloc, &tvdrag, &tvtherm,
                                                 &elec, &grav, &velec}
                                    : ForceArray{&conf, &drag, &coul, &therm};
    const double t0 = other ? 0.3 : 0.0;
    try {
        if (mode == "fused") {
            Runge_Kutta4 I(&cloud, forces, dt, t0);
            I.setAdaptiveTimeStep(false);
            I.setPrecision(prec);
            I.moveParticles(t0 + (nsteps - 0.5) * dt);
            if (I.stepsTaken() != nsteps) {
                std::fprintf(stderr, "took %lld steps\n", I.stepsTaken());
                return 3;
            }
        } else {
            DeviceForce::precision = prec;
            CacheOperator op(&cloud);
            host_rk4(&cloud, forces, op, t0, dt, nsteps);
        }
    } catch (const demon_gb300::Error &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 4;
    }
    FILE *out = std::fopen(argv[2], "wb");
    if (!out) return 2;
    for (double *a : {cloud.x, cloud.y, cloud.Vx, cloud.Vy}) std::fwrite(a, sizeof(double), (size_t)n, out);
    std::fclose(out);
    return 0;
}
