/**
 * driver.cpp -- the `demon_gb300` program: DEMON's command line and
 * Params.cfg (driver.cpp:135-1030 in the reference) for the forces this
 * library runs on the GPU, the same force set-up, output loop and time
 * accounting (driver.cpp:315-475), with the integration on the device.
 *
 * Forces, as in the reference (driver.cpp:320-326, 372-402): Drag unless
 * -D, Confinement unless -R or -V, ShieldedCoulomb always; -B Magnetic,
 * -D TimeVaryingDrag, -E Electric, -F VertElectric, -G Gravitational,
 * -L ThermalLocalized, -R RectConfinement, -S Rotational, -T Thermal,
 * -v TimeVaryingThermal, -V ConfinementVoid, -w Driving, with the
 * reference's conflict checks (driver.cpp:483-511).  -I selects the
 * Runge_Kutta2 integrator (driver.cpp:904-907, 437-438).
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
#include <initializer_list>
#include <iostream>
#include <string>
#include <vector>

#include "Cloud.h"
#include "ConfinementForce.h"
#include "ConfinementForceVoid.h"
#include "Device.h"
#include "DragForce.h"
#include "DrivingForce.h"
#include "ElectricForce.h"
#include "GravitationalForce.h"
#include "MagneticForce.h"
#include "RectConfinementForce.h"
#include "RotationalForce.h"
#include "Runge_Kutta2.h"
#include "Runge_Kutta4.h"
#include "ShieldedCoulombForce.h"
#include "ThermalForce.h"
#include "ThermalForceLocalized.h"
#include "TimeVaryingDragForce.h"
#include "TimeVaryingThermalForce.h"
#include "VertElectricForce.h"

namespace {

// Defaults of the reference (driver.cpp:61-121).
struct Settings {
    bool mach = false;
    bool rk4 = true;
    double voidDecay = 0.4;
    double magneticFieldStrength = 1.0;
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
    double thermRed1 = 1E-14;
    double thermScale = 1E-14;
    double thermOffset = 0.0;
    double heatRadius = 0.001;
    double driveConst = 0.00001;
    double waveAmplitude = 1E-13;
    double waveShift = 0.007;
    double machSpeed = 0.2;
    double massFactor = 100;
    double qMean = 6000.0;
    double qSigma = 100.0;
    double rMean = 1.45E-6;
    double rSigma = 0.0;
    double rmin = 0.003 * 5.0;  // spacing*5 with the driver's spacing 0.003
    double rmax = 0.003 * 10.0;
    double rotConst = 1E-15;
    double dragScale = -1.0;
    double electricFieldStrength = 0;
    double plasmaRadius = 1;
    double vertElectricFieldStrength = 0;
    double verticalDecay = 1;
    double gravitationalFieldStrength = 0;
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

// checkForce (driver.cpp:483-511): the first flag must not be set yet and
// none of the others may be; then the first is set.
void checkForce(Settings &s, char option, force_flags flag, const char *others = "",
                std::initializer_list<force_flags> otherFlags = {}) {
    if (s.usedForces & flag) fail(std::string("option -") + option + " already set");
    size_t k = 0;
    for (force_flags f : otherFlags) {
        if (s.usedForces & f) fail(std::string("option -") + option + " conflicts with option -" + others[k]);
        k++;
    }
    s.usedForces |= flag;
}

// The thermal options exclude one another (driver.cpp:908-915, 958-972).
void checkThermal(Settings &s, char option) {
    switch (option) {
    case 'T': checkForce(s, 'T', ThermalForceFlag, "Lv", {ThermalForceLocalizedFlag, TimeVaryingThermalForceFlag}); break;
    case 'L': checkForce(s, 'L', ThermalForceLocalizedFlag, "Tv", {ThermalForceFlag, TimeVaryingThermalForceFlag}); break;
    default: checkForce(s, 'v', TimeVaryingThermalForceFlag, "LT", {ThermalForceLocalizedFlag, ThermalForceFlag}); break;
    }
}

// The force letter of a forceFlags entry or command-line option.
void useForce(Settings &s, char letter) {
    switch (letter) {
    case 'B': checkForce(s, 'B', MagneticForceFlag); break;
    case 'D': checkForce(s, 'D', TimeVaryingDragForceFlag); break;
    case 'E': checkForce(s, 'E', ElectricForceFlag); break;
    case 'F': checkForce(s, 'F', VertElectricForceFlag); break;
    case 'G': checkForce(s, 'G', GravitationalForceFlag); break;
    case 'R': checkForce(s, 'R', RectConfinementForceFlag); break;
    case 'S': checkForce(s, 'S', RotationalForceFlag); break;
    case 'V': checkForce(s, 'V', ConfinementForceVoidFlag); break;
    case 'w': checkForce(s, 'w', DrivingForceFlag); break;
    case 'T': case 'L': case 'v': checkThermal(s, letter); break;
    default: break;  // the reference ignores other entries
    }
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
              << " -I                     use the second-order Runge-Kutta integrator\n"
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
              << " -B 1.0                 MagneticForce field [T]\n"
              << " -D -1.0 10.0           TimeVaryingDragForce scale [Hz/s], offset [Hz]\n"
              << " -E 0 1                 ElectricForce field [V/m^2], plasma radius [m]\n"
              << " -F 0 1                 VertElectricForce field [V/m^2], decay [m]\n"
              << " -G 0                   GravitationalForce field [m/s^2]\n"
              << " -L 0.001 1E-14 1E-14   ThermalForceLocalized radius [m], inner, outer [N]\n"
              << " -S 1E-15 0.015 0.03    RotationalForce strength [N], rmin, rmax [m]\n"
              << " -v 1E-14 0             TimeVaryingThermalForce scale [N/s], offset [N]\n"
              << " -V 0.4                 ConfinementForceVoid decay [1/m]\n"
              << " -w 1E-13 0.007 1E-5    DrivingForce amplitude [N], shift [m], driving constant\n"
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
        else if (name == "thermRed1") s.thermRed1 = v;
        else if (name == "thermScale") s.thermScale = v;
        else if (name == "thermOffset") s.thermOffset = v;
        else if (name == "heatRadius") s.heatRadius = v;
        else if (name == "driveConst") s.driveConst = v;
        else if (name == "waveAmplitude") s.waveAmplitude = v;
        else if (name == "waveShift") s.waveShift = v;
        else if (name == "voidDecay") s.voidDecay = v;
        else if (name == "magneticFieldStrength") s.magneticFieldStrength = v;
        else if (name == "rmin") s.rmin = v;
        else if (name == "rmax") s.rmax = v;
        else if (name == "rotConst") s.rotConst = v;
        else if (name == "dragScale") s.dragScale = v;
        else if (name == "electricFieldStrength") s.electricFieldStrength = v;
        else if (name == "plasmaRadius") s.plasmaRadius = v;
        else if (name == "vertElectricFieldStrength") s.vertElectricFieldStrength = v;
        else if (name == "verticalDecay") s.verticalDecay = v;
        else if (name == "gravitationalFieldStrength") s.gravitationalFieldStrength = v;
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
            // comma-terminated letters, e.g. "B,D," (driver.cpp:761-822): as in
            // the reference an entry counts only while more than one
            // character is left, so a last letter without its comma is dropped
            std::string rest = value;
            while (rest.size() > 1) {
                const size_t comma = rest.find(',');
                const std::string f = rest.substr(0, comma);
                if (f.size() == 1) useForce(s, f[0]);
                if (comma == std::string::npos) break;
                rest = rest.substr(comma + 1);
            }
        }
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
            case 'I': s.rk4 = false; break;
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
                useForce(s, 'R');
                s.confinementConstX = std::atof(argv[++i]);
                s.confinementConstY = std::atof(argv[++i]);
                break;
            case 's': need(i, 1); s.shieldingConstant = std::atof(argv[++i]); break;
            case 't': need(i, 1); s.simTimeStep = std::atof(argv[++i]); break;
            case 'T': need(i, 1); useForce(s, 'T'); s.thermRed = std::atof(argv[++i]); break;
            case 'd': need(i, 1); Cloud::dustParticleMassDensity = std::atof(argv[++i]); break;
            case 'i': need(i, 1); Cloud::interParticleSpacing = std::atof(argv[++i]); break;
            case 'p': need(i, 2); Cloud::justX = std::atof(argv[++i]); Cloud::justY = std::atof(argv[++i]); break;
            case 'k': need(i, 2); Cloud::velX = std::atof(argv[++i]); Cloud::velY = std::atof(argv[++i]); break;
            // the other forces' options (driver.cpp:878-1003)
            case 'B': need(i, 1); useForce(s, 'B'); s.magneticFieldStrength = std::atof(argv[++i]); break;
            case 'D':
                need(i, 2);
                useForce(s, 'D');
                s.dragScale = std::atof(argv[++i]);
                s.dragGamma = std::atof(argv[++i]);
                break;
            case 'E':
                need(i, 2);
                useForce(s, 'E');
                s.electricFieldStrength = std::atof(argv[++i]);
                s.plasmaRadius = std::atof(argv[++i]);
                break;
            case 'F':
                need(i, 2);
                useForce(s, 'F');
                s.vertElectricFieldStrength = std::atof(argv[++i]);
                s.verticalDecay = std::atof(argv[++i]);
                break;
            case 'G': need(i, 1); useForce(s, 'G'); s.gravitationalFieldStrength = std::atof(argv[++i]); break;
            case 'L':
                need(i, 3);
                useForce(s, 'L');
                s.heatRadius = std::atof(argv[++i]);
                s.thermRed = std::atof(argv[++i]);
                s.thermRed1 = std::atof(argv[++i]);
                break;
            case 'S':
                need(i, 3);
                useForce(s, 'S');
                s.rotConst = std::atof(argv[++i]);
                s.rmin = std::atof(argv[++i]);
                s.rmax = std::atof(argv[++i]);
                break;
            case 'v':
                need(i, 2);
                useForce(s, 'v');
                s.thermScale = std::atof(argv[++i]);
                s.thermOffset = std::atof(argv[++i]);
                break;
            case 'V': need(i, 1); useForce(s, 'V'); s.voidDecay = std::atof(argv[++i]); break;
            case 'w':
                need(i, 3);
                useForce(s, 'w');
                s.waveAmplitude = std::atof(argv[++i]);
                s.waveShift = std::atof(argv[++i]);
                s.driveConst = std::atof(argv[++i]);
                break;
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
    // driver.cpp:322-326
    if (!(s.usedForces & TimeVaryingDragForceFlag)) s.usedForces |= DragForceFlag;
    if (!(s.usedForces & RectConfinementForceFlag) && !(s.usedForces & ConfinementForceVoidFlag))
        s.usedForces |= ConfinementForceFlag;
    s.usedForces |= ShieldedCoulombForceFlag;

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

    if (s.usedForces & ~(force_flags)32767) fail("the input file sets unknown force flags");

    // driver.cpp:372-402, same order and constructor arguments; a continued
    // file's FORCES picks them, so a file written with -D, -V or -v (which
    // also set the Drag, Confinement or Thermal bit, TimeVaryingDragForce.cpp:51,
    // ConfinementForceVoid.cpp:66, TimeVaryingThermalForce.cpp:53) continues
    // with both forces, as in the reference
    const force_flags u = s.usedForces;
    ForceArray forces;
    if (u & ConfinementForceFlag) forces.push_back(new ConfinementForce(cloud, s.confinementConst));
    if (u & ConfinementForceVoidFlag)
        forces.push_back(new ConfinementForceVoid(cloud, s.confinementConst, s.voidDecay));
    if (u & DragForceFlag) forces.push_back(new DragForce(cloud, s.dragGamma));
    if (u & DrivingForceFlag) forces.push_back(new DrivingForce(cloud, s.driveConst, s.waveAmplitude, s.waveShift));
    if (u & MagneticForceFlag) forces.push_back(new MagneticForce(cloud, s.magneticFieldStrength));
    if (u & RectConfinementForceFlag)
        forces.push_back(new RectConfinementForce(cloud, s.confinementConstX, s.confinementConstY));
    if (u & RotationalForceFlag) forces.push_back(new RotationalForce(cloud, s.rmin, s.rmax, s.rotConst));
    if (u & ShieldedCoulombForceFlag) forces.push_back(new ShieldedCoulombForce(cloud, s.shieldingConstant));
    if (u & ThermalForceFlag) forces.push_back(new ThermalForce(cloud, s.thermRed, s.thermalMode, s.seed));
    if (u & ThermalForceLocalizedFlag)
        forces.push_back(new ThermalForceLocalized(cloud, s.thermRed, s.thermRed1, s.heatRadius, s.thermalMode, s.seed));
    if (u & TimeVaryingDragForceFlag) forces.push_back(new TimeVaryingDragForce(cloud, s.dragScale, s.dragGamma));
    if (u & TimeVaryingThermalForceFlag)
        forces.push_back(new TimeVaryingThermalForce(cloud, s.thermScale, s.thermOffset, s.thermalMode, s.seed));
    if (u & ElectricForceFlag) forces.push_back(new ElectricForce(cloud, s.electricFieldStrength, s.plasmaRadius));
    if (u & GravitationalForceFlag) forces.push_back(new GravitationalForce(cloud, s.gravitationalFieldStrength));
    if (u & VertElectricForceFlag)
        forces.push_back(new VertElectricForce(cloud, s.vertElectricFieldStrength, s.verticalDecay));

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
        // driver.cpp:437-438
        Runge_Kutta4 rk4(cloud, forces, s.simTimeStep, s.startTime);
        Runge_Kutta2 rk2(cloud, forces, s.simTimeStep, s.startTime);
        DeviceIntegrator &I = s.rk4 ? static_cast<DeviceIntegrator &>(rk4) : rk2;
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
        if (!s.dryRun)
            std::cout << "\r" << I.stepsTaken() << (s.rk4 ? " RK4" : " RK2") << " steps to t = " << I.currentTime << " s";
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
