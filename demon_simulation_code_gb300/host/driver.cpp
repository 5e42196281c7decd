/**
 * driver.cpp -- the `demon_gb300` program: DEMON's command line and
 * Params.cfg (driver.cpp:135-1030 in the reference) for the forces this
 * library runs on the GPU, the same force set-up, output loop and time
 * accounting (driver.cpp:315-475), with the integration on the device.
 *
 * Forces: Confinement (unless -R), Drag and ShieldedCoulomb always, as in
 * the reference (driver.cpp:320-325); -R RectConfinement, -T Thermal.  The
 * reference's other forces (-B -D -E -F -G -L -S -v -V -w) and its RK2
 * integrator (-I) are refused with a message.
 *
 * Options beyond the reference's:
 *   --precision fp64|fp32c   pair arithmetic (default fp64)
 *   --fixed-dt               skip the adaptive dt test (the reference always
 *                            runs it)
 *   --seed S                 seed of the charge/mass draws and the thermal
 *                            generator (default: random)
 *   --thermal-mode 0|1       0: the reference's uniform-magnitude kick,
 *                            1: Gaussian N(0, thermRed^2) per axis
 *   --device D               CUDA device (default $DEMON_GB300_DEVICE or 0)
 *   --dry-run                set up and write the initial file, no steps
 */
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "Cloud.h"
#include "ConfinementForce.h"
#include "Device.h"
#include "DragForce.h"
#include "RectConfinementForce.h"
#include "Runge_Kutta4.h"
#include "ShieldedCoulombForce.h"
#include "ThermalForce.h"

namespace {

struct Settings {
    bool mach = false;
    double startTime = 0.0;
    double dataTimeStep = 0.01;
    double simTimeStep = 0.01 / 100.0;
    double endTime = 5.0;
    double confinementConst = 100;
    double confinementConstX = 100;
    double confinementConstY = 1000;
    double shieldingConstant = 2E4;
    double dragGamma = 10.0;
    double thermRed = 1E-14;
    double machSpeed = 0.2;
    double massFactor = 100;
    double qMean = 6000.0;
    double qSigma = 100.0;
    double rMean = 1.45E-6;
    double rSigma = 0.0;
    force_flags usedForces = 0;
    cloud_index numParticles = 4;
    cloud_index row_x_particles = 4;
    cloud_index row_y_particles = 0;
    std::string continueFile, finalsFile, outputFile = "data.fits";
    int precision = DM_FP64;
    bool adaptive = true;
    uint64_t seed = 0;
    int thermalMode = 0;
    int device = -1;
    bool dryRun = false;
};

[[noreturn]] void fail(const std::string &msg) {
    std::cerr << "demon_gb300: " << msg << std::endl;
    std::exit(1);
}

void refuseForce(char letter) {
    fail(std::string("force option -") + letter +
         " is not available in this build (GPU forces: Confinement, RectConfinement, Drag, "
         "ShieldedCoulomb, Thermal)");
}

bool isNumber(const char *s) {
    if (!s || !*s) return false;
    char *end = nullptr;
    std::strtod(s, &end);
    return end && *end == '\0';
}

void help() {
    std::cout << "demon_gb300 -- DEMON's RK4 dusty-plasma simulation on a GB300\n\n"
              << " -c file.fits           continue run from file (appends)\n"
              << " -C 100.0               confinementConst [V/m^2]\n"
              << " -d 2200                dust density [kg/m^3]\n"
              << " -e 5.0                 end time [s]\n"
              << " -f file.fits           start from the final state of a file\n"
              << " -g 10.0                dragGamma [Hz]\n"
              << " -h                     this help\n"
              << " -i 0.003               initial inter-particle spacing [m]\n"
              << " -k 0 0                 initial x;y velocity [m/s]\n"
              << " -M 0.2 100             Mach cone: bullet velocity [m/s], mass factor\n"
              << " -n 4 4                 number of particles [, particles per x row]\n"
              << " -o 0.01                data output time step [s]\n"
              << " -O data.fits           output file\n"
              << " -P Params.cfg          read parameters from file\n"
              << " -p 0 0                 cloud centre x;y [m]\n"
              << " -q 6000.0 100.0        charge mean and sigma [electron charges]\n"
              << " -R 100.0 1000.0        RectConfinementForce confineConstX,Y [V/m^2]\n"
              << " -r 1.45E-6 0.0         particle radius mean and sigma [m]\n"
              << " -s 2E4                 shielding constant [1/m]\n"
              << " -t 0.0001              simulation time step [s]\n"
              << " -T 1E-14               ThermalForce reduction factor [N]\n"
              << " --precision fp64|fp32c, --fixed-dt, --seed S, --thermal-mode 0|1,\n"
              << " --device D, --dry-run\n";
}

// Params.cfg: "name value" pairs (driver.cpp:626-826).
void readParams(const std::string &path, Settings &s) {
    std::ifstream in(path);
    if (!in) fail("cannot read parameter file " + path);
    std::string name, value;
    while (in >> name >> value) {
        const double v = std::atof(value.c_str());
        if (name == "numParticles") s.numParticles = (cloud_index)v;
        else if (name == "startTime") s.startTime = v;
        else if (name == "dataTimeStep") s.dataTimeStep = v;
        else if (name == "simTimeStep") s.simTimeStep = v;
        else if (name == "spacing") Cloud::interParticleSpacing = v;
        else if (name == "endTime") s.endTime = v;
        else if (name == "confinementConst") s.confinementConst = v;
        else if (name == "confinementConstX") s.confinementConstX = v;
        else if (name == "confinementConstY") s.confinementConstY = v;
        else if (name == "shieldingConstant") s.shieldingConstant = v;
        else if (name == "dragGamma") s.dragGamma = v;
        else if (name == "thermRed") s.thermRed = v;
        else if (name == "machSpeed") s.machSpeed = v;
        else if (name == "massFactor") s.massFactor = v;
        else if (name == "qMean") s.qMean = v;
        else if (name == "qSigma") s.qSigma = v;
        else if (name == "rMean") s.rMean = v;
        else if (name == "rSigma") s.rSigma = v;
        else if (name == "justifyX") Cloud::justX = v;
        else if (name == "justifyY") Cloud::justY = v;
        else if (name == "massDensity") Cloud::dustParticleMassDensity = v;
        else if (name == "velocityX") Cloud::velX = v;
        else if (name == "velocityY") Cloud::velY = v;
        else if (name == "forceFlags") {
            // comma-separated letters, e.g. "R,T," (driver.cpp:756-822)
            size_t start = 0;
            while (start < value.size()) {
                size_t comma = value.find(',', start);
                const std::string f = value.substr(start, comma == std::string::npos ? std::string::npos
                                                                                      : comma - start);
                if (f == "R") s.usedForces |= RectConfinementForceFlag;
                else if (f == "T") s.usedForces |= ThermalForceFlag;
                else if (!f.empty()) refuseForce(f[0]);
                if (comma == std::string::npos) break;
                start = comma + 1;
            }
        }
        // the remaining keys parameterise forces this build does not run;
        // they are accepted and ignored unless their force is requested
    }
}

void parseArgs(int argc, char **argv, Settings &s) {
    auto need = [&](int &i, int k) {
        for (int j = 1; j <= k; j++)
            if (i + j >= argc) fail(std::string("option ") + argv[i] + " needs " + std::to_string(k) + " value(s)");
    };
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        if (a == "--precision") {
            need(i, 1);
            const std::string v = argv[++i];
            if (v == "fp64") s.precision = DM_FP64;
            else if (v == "fp32c") s.precision = DM_FP32C;
            else fail("--precision takes fp64 or fp32c");
        } else if (a == "--fixed-dt") {
            s.adaptive = false;
        } else if (a == "--seed") {
            need(i, 1);
            s.seed = std::strtoull(argv[++i], nullptr, 10);
        } else if (a == "--thermal-mode") {
            need(i, 1);
            s.thermalMode = std::atoi(argv[++i]);
        } else if (a == "--device") {
            need(i, 1);
            s.device = std::atoi(argv[++i]);
        } else if (a == "--dry-run") {
            s.dryRun = true;
        } else if (a.size() == 2 && a[0] == '-') {
            switch (a[1]) {
            case 'P': need(i, 1); readParams(argv[++i], s); break;
            case 'O': need(i, 1); s.outputFile = argv[++i]; break;
            case 'c': need(i, 1); s.continueFile = argv[++i]; break;
            case 'f': need(i, 1); s.finalsFile = argv[++i]; break;
            case 'n':
                need(i, 1);
                s.numParticles = (cloud_index)std::atoi(argv[++i]);
                if (i + 1 < argc && isNumber(argv[i + 1])) {
                    s.row_x_particles = (cloud_index)std::atoi(argv[++i]);
                    s.row_y_particles = s.row_x_particles > 0 ? s.numParticles / s.row_x_particles : 0;
                }
                break;
            case 'C': need(i, 1); s.confinementConst = std::atof(argv[++i]); break;
            case 'e': need(i, 1); s.endTime = std::atof(argv[++i]); break;
            case 'g': need(i, 1); s.dragGamma = std::atof(argv[++i]); break;
            case 'h': help(); std::exit(0);
            case 'I': fail("-I (Runge_Kutta2) is not available in this build");
            case 'M':
                need(i, 2);
                s.mach = true;
                s.machSpeed = std::atof(argv[++i]);
                s.massFactor = std::atof(argv[++i]);
                break;
            case 'o': need(i, 1); s.dataTimeStep = std::atof(argv[++i]); break;
            case 'q': need(i, 2); s.qMean = std::atof(argv[++i]); s.qSigma = std::atof(argv[++i]); break;
            case 'r': need(i, 2); s.rMean = std::atof(argv[++i]); s.rSigma = std::atof(argv[++i]); break;
            case 'R':
                need(i, 2);
                s.usedForces |= RectConfinementForceFlag;
                s.confinementConstX = std::atof(argv[++i]);
                s.confinementConstY = std::atof(argv[++i]);
                break;
            case 's': need(i, 1); s.shieldingConstant = std::atof(argv[++i]); break;
            case 't': need(i, 1); s.simTimeStep = std::atof(argv[++i]); break;
            case 'T': need(i, 1); s.usedForces |= ThermalForceFlag; s.thermRed = std::atof(argv[++i]); break;
            case 'd': need(i, 1); Cloud::dustParticleMassDensity = std::atof(argv[++i]); break;
            case 'i': need(i, 1); Cloud::interParticleSpacing = std::atof(argv[++i]); break;
            case 'p': need(i, 2); Cloud::justX = std::atof(argv[++i]); Cloud::justY = std::atof(argv[++i]); break;
            case 'k': need(i, 2); Cloud::velX = std::atof(argv[++i]); Cloud::velY = std::atof(argv[++i]); break;
            case 'B': case 'D': case 'E': case 'F': case 'G': case 'L': case 'S': case 'v': case 'V': case 'w':
                refuseForce(a[1]);
            default: fail("unknown option " + a + " (-h for help)");
            }
        } else {
            fail("unknown argument " + a + " (-h for help)");
        }
    }
}

}  // namespace

int main(int argc, char **argv) {
    const auto start = std::chrono::steady_clock::now();
    Settings s;
    parseArgs(argc, argv, s);
    RandomNumbers::seed = s.seed;
    if (s.device >= 0) demon_gb300::context(s.device);  // make it the process's device
    if (!(s.usedForces & RectConfinementForceFlag)) s.usedForces |= ConfinementForceFlag;
    s.usedForces |= DragForceFlag | ShieldedCoulombForceFlag;

    namespace F = demon_gb300::fits;
    int error = 0;
    fitsfile *file = nullptr;
    Cloud *cloud = nullptr;
    if (!s.continueFile.empty()) {
        file = F::open(s.continueFile, true, error);
        if (!error) s.usedForces = F::read_key_long(file, "FORCES", error);
        if (!error) cloud = Cloud::initializeFromFile(file, error, &s.startTime);
    } else if (!s.finalsFile.empty()) {
        fitsfile *in = F::open(s.finalsFile, false, error);
        if (!error) cloud = Cloud::initializeFromFile(in, error, nullptr);
        if (in) F::close(in, error);
    } else {
        if (s.numParticles < 1) fail("need at least one particle");
        cloud = Cloud::initializeGrid(s.numParticles, s.row_x_particles, s.row_y_particles, s.rMean, s.rSigma,
                                      s.qMean, s.qSigma);
    }
    if (error) fail("FITS error " + std::to_string(error) + " reading the input file");
    if (s.continueFile.empty()) file = F::create(s.outputFile, error);
    if (error) fail("FITS error " + std::to_string(error) + " creating " + s.outputFile);

    const force_flags known = ConfinementForceFlag | DragForceFlag | ShieldedCoulombForceFlag | ThermalForceFlag |
                              RectConfinementForceFlag;
    if (s.usedForces & ~known) fail("the input file uses forces this build does not run");

    // driver.cpp:372-402 order
    ForceArray forces;
    if (s.usedForces & ConfinementForceFlag) forces.push_back(new ConfinementForce(cloud, s.confinementConst));
    if (s.usedForces & DragForceFlag) forces.push_back(new DragForce(cloud, s.dragGamma));
    if (s.usedForces & RectConfinementForceFlag)
        forces.push_back(new RectConfinementForce(cloud, s.confinementConstX, s.confinementConstY));
    if (s.usedForces & ShieldedCoulombForceFlag) forces.push_back(new ShieldedCoulombForce(cloud, s.shieldingConstant));
    if (s.usedForces & ThermalForceFlag) forces.push_back(new ThermalForce(cloud, s.thermRed, s.thermalMode, s.seed));

    if (!s.continueFile.empty()) {
        for (Force *const f : forces) f->readForce(file, &error);
    } else {
        for (Force *const f : forces) f->writeForce(file, &error);
        cloud->writeCloudSetup(file, error);
    }
    if (error) fail("FITS error " + std::to_string(error) + " writing the set-up");

    if (s.mach) {  // driver.cpp:420-427
        cloud->x[0] = -0.75 * std::sqrt((double)cloud->n) * Cloud::interParticleSpacing;
        cloud->y[0] = 0.0;
        cloud->Vx[0] = s.machSpeed;
        cloud->Vy[0] = 0.0;
        cloud->mass[0] *= s.massFactor;
    }

    int rc = 0;
    try {
        Runge_Kutta4 I(cloud, forces, s.simTimeStep, s.startTime);
        I.setPrecision(s.precision);
        I.setAdaptiveTimeStep(s.adaptive);
        double t = s.startTime;
        while (!s.dryRun && t < s.endTime) {
            std::cout << "\rCurrent Time: " << I.currentTime << "s (" << I.currentTime / s.endTime * 100.0
                      << "% Complete)" << std::flush;
            I.moveParticles(t += s.dataTimeStep);
            cloud->writeTimeStep(file, error, I.currentTime);
            if (error) fail("FITS error " + std::to_string(error) + " writing a time step");
        }
        if (!s.dryRun) std::cout << "\r" << I.stepsTaken() << " RK4 steps to t = " << I.currentTime << " s";
    } catch (const demon_gb300::Error &e) {
        std::cerr << "\ndemon_gb300: " << e.what() << std::endl;
        rc = 1;
    }
    F::close(file, error);
    for (Force *const f : forces) delete f;
    delete cloud;
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    std::cout << "\nTime elapsed: " << secs << " s" << std::endl;
    return rc ? rc : (error ? 1 : 0);
}
