/**
 * Cloud.cpp -- host cloud: arrays, grid initialisation (Cloud.cpp:95-135),
 * charge / mass draws (Cloud.cpp:56-81), FITS setup / time-step output and
 * restart (Cloud.cpp:146-271), and the device copies.
 */
#include "Cloud.h"

#include <cmath>
#include <string>
#include <vector>

#include "Device.h"

const double Cloud::electronCharge = -1.602E-19;
const double Cloud::epsilon0 = 8.8541878E-12;
const double Cloud::particleRadius = 1.45E-6;
// The reference's driver defines these (driver.cpp:122-127); weak defaults
// here let a driver that defines them again link unchanged.
__attribute__((weak)) double Cloud::interParticleSpacing = 0.003;
__attribute__((weak)) double Cloud::dustParticleMassDensity = 2200.0;
__attribute__((weak)) double Cloud::justX = 0.0;
__attribute__((weak)) double Cloud::justY = 0.0;
__attribute__((weak)) double Cloud::velX = 0.0;
__attribute__((weak)) double Cloud::velY = 0.0;

Cloud::Cloud(const cloud_index numPar)
    : n(numPar),
      x(new double[n]()), y(new double[n]()), Vx(new double[n]()), Vy(new double[n]()),
      charge(new double[n]()), mass(new double[n]()),
      k1(new double[n]()), k2(new double[n]()), k3(new double[n]()), k4(new double[n]()),
      l1(new double[n]()), l2(new double[n]()), l3(new double[n]()), l4(new double[n]()),
      m1(new double[n]()), m2(new double[n]()), m3(new double[n]()), m4(new double[n]()),
      n1(new double[n]()), n2(new double[n]()), n3(new double[n]()), n4(new double[n]()),
      forceX(new double[n]()), forceY(new double[n]()),
      xCache(new double[n]()), yCache(new double[n]()), VxCache(new double[n]()), VyCache(new double[n]()) {}

Cloud::~Cloud() {
    if (state_) dm_cloud_destroy(state_);
    if (scratch_) dm_cloud_destroy(scratch_);
    for (double *p : {x, y, Vx, Vy, charge, mass, k1, k2, k3, k4, l1, l2, l3, l4, m1, m2, m3, m4, n1, n2, n3, n4,
                      forceX, forceY, xCache, yCache, VxCache, VyCache})
        delete[] p;
}

void Cloud::initCharge(const double qMean, const double qSigma) {
    std::normal_distribution<double> dist(qMean, qSigma);
    for (cloud_index i = 0; i < n; i++) charge[i] = rands.gaussian(dist) * electronCharge;
}

void Cloud::initMass(const double rMean, const double rSigma) {
    const double particleMassConstant = (4.0 / 3.0) * M_PI * dustParticleMassDensity;
    std::normal_distribution<double> dist(rMean, rSigma);
    for (cloud_index i = 0; i < n; i++) {
        const double r = rands.gaussian(dist);
        mass[i] = particleMassConstant * r * r * r;
    }
}

Cloud *const Cloud::initializeGrid(const cloud_index numParticles, cloud_index row_x_particles,
                                   cloud_index row_y_particles, const double rMean, const double rSigma,
                                   const double qMean, const double qSigma) {
    Cloud *const cloud = new Cloud(numParticles);
    // as square a grid as divides numParticles, unless the rows are given
    if (row_y_particles == 0) {
        row_x_particles = (cloud_index)std::floor(std::sqrt((double)numParticles));
        if (row_x_particles < 1) row_x_particles = 1;
        while (numParticles % row_x_particles != 0) ++row_x_particles;
        row_y_particles = numParticles / row_x_particles;
    }
    const double halfX = ((double)row_x_particles - 1.0) / 2.0 * interParticleSpacing;
    const double halfY = ((double)row_y_particles - 1.0) / 2.0 * interParticleSpacing;
    cloud->initCharge(qMean, qSigma);
    cloud->initMass(rMean, rSigma);
    for (cloud_index i = 0; i < row_x_particles; i++)
        for (cloud_index j = 0; j < row_y_particles; j++) {
            const cloud_index p = i * row_y_particles + j;
            if (p >= numParticles) continue;
            cloud->x[p] = halfX - (i * interParticleSpacing) + justX;
            cloud->y[p] = halfY - (j * interParticleSpacing) + justY;
        }
    for (cloud_index p = 0; p < numParticles; p++) {
        cloud->Vx[p] = velX;
        cloud->Vy[p] = velY;
    }
    return cloud;
}

namespace {
std::vector<demon_gb300::fits::Column> time_step_columns(long n) {
    return {{"TIME", 1, "s"},
            {"X_POSITION", n, "m"},
            {"Y_POSITION", n, "m"},
            {"X_VELOCITY", n, "m/s"},
            {"Y_VELOCITY", n, "m/s"}};
}
}  // namespace

void Cloud::writeCloudSetup(fitsfile *const file, int &error) const {
    namespace F = demon_gb300::fits;
    F::create_table(file, "CLOUD", {{"MASS", 1, "kg"}, {"CHARGE", 1, "C"}}, error);
    F::append_rows(file, "CLOUD", n, {mass, charge}, error);
    F::create_table(file, "TIME_STEP", time_step_columns(n), error);
    const double t0 = 0.0;
    F::append_rows(file, "TIME_STEP", 1, {&t0, x, y, Vx, Vy}, error);
    F::flush(file, error);
}

void Cloud::writeTimeStep(fitsfile *const file, int &error, double currentTime) const {
    namespace F = demon_gb300::fits;
    F::append_rows(file, "TIME_STEP", 1, {&currentTime, x, y, Vx, Vy}, error);
    F::flush(file, error);
}

Cloud *const Cloud::initializeFromFile(fitsfile *const file, int &error, double *const currentTime) {
    namespace F = demon_gb300::fits;
    const long numParticles = F::num_rows(file, "CLOUD", error);
    if (error) return nullptr;
    Cloud *const cloud = new Cloud((cloud_index)numParticles);
    std::vector<double> m = F::read_column(file, "CLOUD", 0, error);
    std::vector<double> q = F::read_column(file, "CLOUD", 1, error);
    const long rows = F::num_rows(file, "TIME_STEP", error);
    if (!error && rows < 1) error = F::BAD_ROW_NUM;
    std::vector<double> cols[5];
    for (int c = 0; c < 5 && !error; c++) cols[c] = F::read_cell(file, "TIME_STEP", c, rows - 1, error);
    if (!error && ((long)m.size() != numParticles || (long)q.size() != numParticles ||
                   (long)cols[1].size() != numParticles))
        error = F::NOT_BTABLE;
    if (error) {
        delete cloud;
        return nullptr;
    }
    for (long i = 0; i < numParticles; i++) {
        cloud->mass[i] = m[i];
        cloud->charge[i] = q[i];
        cloud->x[i] = cols[1][i];
        cloud->y[i] = cols[2][i];
        cloud->Vx[i] = cols[3][i];
        cloud->Vy[i] = cols[4][i];
    }
    if (currentTime) *currentTime = cols[0][0];
    return cloud;
}

dm_cloud *Cloud::deviceState() {
    if (!state_) {
        dm_ctx *ctx = demon_gb300::context();
        demon_gb300::check(dm_cloud_create(ctx, n, x, y, Vx, Vy, charge, mass, &state_), ctx, "dm_cloud_create");
    }
    return state_;
}

dm_cloud *Cloud::deviceScratch() {
    if (!scratch_) {
        dm_ctx *ctx = demon_gb300::context();
        demon_gb300::check(dm_cloud_create(ctx, n, x, y, Vx, Vy, charge, mass, &scratch_), ctx, "dm_cloud_create");
    }
    return scratch_;
}
