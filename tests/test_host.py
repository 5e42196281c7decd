"""The C++ host classes and the demon_gb300 driver, without a GPU: build,
Params.cfg and command-line handling, the FITS output of the set-up, and the
force options' checks (--dry-run stops before the first device call)."""
import os
import subprocess

import numpy as np
import pytest

from fitsread import read_fits

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def host_build():
    from demon_simulation_code_gb300 import build

    return build.build_host()


def run(driver, *args, cwd):
    return subprocess.run([driver, *args], cwd=cwd, capture_output=True, text=True, timeout=120)


def test_host_library_exports_the_reference_classes(host_build):
    lib, _ = host_build
    syms = subprocess.run(["nm", "-DC", "--defined-only", lib], capture_output=True, text=True).stdout
    for s in ("Cloud::initializeGrid", "Cloud::writeTimeStep", "Cloud::initializeFromFile",
              "DeviceIntegrator::moveParticles", "Integrator::modifyTimeStep", "CacheOperator::operation2",
              "DeviceForce::evaluate", "ShieldedCoulombForce::writeForce", "ThermalForce::addDeviceParams"):
        assert s in syms, s


def test_params_cfg_sets_up_the_cloud_and_file(host_build, tmp_path):
    _, driver = host_build
    (tmp_path / "Params.cfg").write_text(
        "numParticles 36\nspacing 0.0004\nconfinementConstX 150\nconfinementConstY 250\n"
        "shieldingConstant 30000\ndragGamma 4.0\nthermRed 2E-14\nqMean 5000.0\nqSigma 0.0\n"
        "rMean 2.0E-6\nrSigma 0.0\nmassDensity 1000\njustifyX 0.001\njustifyY -0.002\n"
        "velocityX 0.5\nvelocityY 0.25\nmagneticFieldStrength 1.0\nforceFlags R,T,\n")
    r = run(driver, "-P", "Params.cfg", "-O", "out.fits", "--seed", "9", "--dry-run", cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    keys, tables = read_fits(str(tmp_path / "out.fits"))
    # Drag | ShieldedCoulomb | Thermal | RectConfinement (no radial confinement with -R)
    assert keys["FORCES"] == 2 | 4 | 16 | 8192
    assert keys["CONFINECONSTX"] == 150.0 and keys["CONFINECONSTY"] == 250.0
    assert keys["SHIELDINGCONSTANT"] == 30000.0 and keys["DRAGCONST"] == -4.0
    assert keys["HEATINGVALUE"] == 2e-14 and "CONFINECONST" not in keys
    mass = tables["CLOUD"]["MASS"].ravel()
    charge = tables["CLOUD"]["CHARGE"].ravel()
    assert np.allclose(mass, 4.0 / 3.0 * np.pi * 1000 * (2e-6) ** 3, rtol=1e-15, atol=0)
    assert np.allclose(charge, 5000.0 * -1.602e-19, rtol=1e-15, atol=0)
    ts = tables["TIME_STEP"]
    assert ts["TIME"].shape == (1, 1) and ts["TIME"][0, 0] == 0.0
    x, y = ts["X_POSITION"][0], ts["Y_POSITION"][0]
    # 6 x 6 grid, spacing 4e-4, centred on (justifyX, justifyY) (Cloud.cpp:114-126)
    assert np.allclose(np.sort(np.unique(np.round(x, 12))), 0.001 + 4e-4 * (np.arange(6) - 2.5), atol=1e-15)
    assert np.allclose(np.sort(np.unique(np.round(y, 12))), -0.002 + 4e-4 * (np.arange(6) - 2.5), atol=1e-15)
    assert np.all(ts["X_VELOCITY"] == 0.5) and np.all(ts["Y_VELOCITY"] == 0.25)


def test_command_line_overrides_and_defaults(host_build, tmp_path):
    _, driver = host_build
    r = run(driver, "-n", "16", "-C", "123", "-s", "4e4", "-g", "2.5", "-O", "d.fits", "--dry-run", cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    keys, tables = read_fits(str(tmp_path / "d.fits"))
    assert keys["FORCES"] == 1 | 2 | 4
    assert keys["CONFINECONST"] == 123.0 and keys["SHIELDINGCONSTANT"] == 4e4 and keys["DRAGCONST"] == -2.5
    assert tables["CLOUD"]["MASS"].shape == (16, 1)


def test_driver_accepts_rk2(host_build, tmp_path):
    _, driver = host_build
    r = run(driver, "-n", "8", "-I", "-O", "i.fits", "--dry-run", cwd=tmp_path)
    assert r.returncode == 0, r.stderr


def test_every_force_option_sets_its_flag_and_keys(host_build, tmp_path):
    """The reference's force options (driver.cpp:878-1003) and the FITS keys
    of each force's writeForce."""
    _, driver = host_build
    r = run(driver, "-n", "16", "-B", "0.5", "-D", "-2.0", "7.0", "-E", "3.0", "0.02", "-F", "4.0", "0.03",
            "-G", "-9.8", "-L", "0.002", "1e-14", "3e-14", "-S", "2e-15", "0.001", "0.004", "-V", "0.6",
            "-w", "2e-13", "0.005", "2e-5", "-O", "f.fits", "--dry-run", cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    keys, _ = read_fits(str(tmp_path / "f.fits"))
    # -D replaces Drag but its file entry sets the Drag bit too; -V replaces
    # Confinement likewise (TimeVaryingDragForce.cpp:51, ConfinementForceVoid.cpp:66)
    assert keys["FORCES"] == 1 | 2 | 4 | 8 | 32 | 64 | 128 | 256 | 1024 | 2048 | 4096 | 16384
    assert keys["MAGNETICFIELD"] == 0.5
    assert keys["TVDRAGSCALECONST"] == -2.0 and keys["TVDRAGOFFSETCONST"] == 7.0
    assert keys["DRAGCONST"] == 7.0  # DragForce(C, -offset): dragConst = offset (TimeVaryingDragForce.h:16-17)
    assert keys["ELECTRICFIELDSTRENGTH"] == 3.0 and keys["PLASMARADIUS"] == 0.02
    assert keys["VERTELECTRICFIELDSTRENGTH"] == 4.0 and keys["VERTICALDECAY"] == 0.03
    assert keys["GRAVITATIONALFIELDSTRENGTH"] == -9.8
    assert keys["HEATINGVALUE1"] == 1e-14 and keys["HEATINGVALUE2"] == 3e-14 and keys["HEATINGRADIUS"] == 0.002
    assert keys["ROTATIONALCONST"] == 2e-15 and keys["INNERRADIUS"] == 0.001 and keys["OUTERRADIUS"] == 0.004
    assert keys["DECAY"] == 0.6 and "CONFINECONST" in keys
    # the stored driving constant is minus the option's value (DrivingForce.h:17-18)
    assert keys["DRIVINGAMPLITUDE"] == 2e-13 and keys["DRIVINGSHIFT"] == 0.005 and keys["DRIVINGCONST"] == -2e-5


def test_time_varying_thermal_option(host_build, tmp_path):
    _, driver = host_build
    r = run(driver, "-n", "8", "-v", "2e-14", "1e-15", "-O", "v.fits", "--dry-run", cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    keys, _ = read_fits(str(tmp_path / "v.fits"))
    assert keys["FORCES"] == 1 | 2 | 4 | 16 | 512
    assert keys["HEATINGVALUESCALE"] == 2e-14 and keys["HEATINGVALUEOFFSET"] == 1e-15
    assert keys["HEATINGVALUE"] == 1e-15


@pytest.mark.parametrize("args,msg", [(["-T", "1e-14", "-L", "0.001", "1e-14", "1e-14"], "conflicts"),
                                      (["-v", "1", "0", "-T", "1e-14"], "conflicts"),
                                      (["-B", "1", "-B", "2"], "already set")])
def test_force_option_conflicts_as_the_reference(host_build, tmp_path, args, msg):
    _, driver = host_build
    r = run(driver, *args, "--dry-run", cwd=tmp_path)
    assert r.returncode == 1 and msg in r.stderr


def test_params_force_flags_parse_like_the_reference(host_build, tmp_path):
    """forceFlags entries are comma-terminated; as in the reference
    (driver.cpp:764-769) a last letter without its comma is not read."""
    _, driver = host_build
    (tmp_path / "p.cfg").write_text("numParticles 8\nrotConst 3e-15\nrmin 0.002\nrmax 0.005\n"
                                    "forceFlags R,S,G\n")
    r = run(driver, "-P", "p.cfg", "-O", "p.fits", "--dry-run", cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    keys, _ = read_fits(str(tmp_path / "p.fits"))
    assert keys["FORCES"] == 2 | 4 | 128 | 8192
    assert keys["ROTATIONALCONST"] == 3e-15 and keys["INNERRADIUS"] == 0.002 and keys["OUTERRADIUS"] == 0.005


def test_continue_reads_back_the_file(host_build, tmp_path):
    _, driver = host_build
    assert run(driver, "-n", "8", "-T", "1e-14", "-O", "c.fits", "--dry-run", cwd=tmp_path).returncode == 0
    before = (tmp_path / "c.fits").read_bytes()
    r = run(driver, "-c", "c.fits", "--dry-run", cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "c.fits").read_bytes() == before
    # every force's keys read back
    assert run(driver, "-n", "8", "-B", "2", "-S", "1e-15", "0.001", "0.002", "-D", "-1", "3", "-w", "1e-13",
               "0.001", "1e-5", "-O", "d.fits", "--dry-run", cwd=tmp_path).returncode == 0
    before = (tmp_path / "d.fits").read_bytes()
    r = run(driver, "-c", "d.fits", "--dry-run", cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "d.fits").read_bytes() == before


def test_host_api_check_compiles(host_build, tmp_path):
    from demon_simulation_code_gb300 import build

    exe = tmp_path / "host_api_check"
    cmd = ["g++", *build.HOST_FLAGS, "-o", str(exe), os.path.join(HERE, "host_api_check.cpp"),
           "-L" + build.PKG, "-ldemon_gb300_host", "-ldemon_gb300", "-Wl,-rpath," + build.PKG]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
