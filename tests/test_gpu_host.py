"""The C++ host classes and the demon_gb300 driver on the GPU (needs a GB300).

* the driver's output file against the oracle replaying the reference's
  driver loop (driver.cpp:442-450: moveParticles(startTime += dataTimeStep),
  adaptive dt, writeTimeStep) from the file's own initial row, and the same
  for a run continued with -c;
* a host-stepped RK4 written over the reference's per-force force1..4 calls
  and CacheOperator (tests/host_api_check.cpp) against the fused device
  Runge_Kutta4."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from fitsread import read_fits
from demon_simulation_code_gb300 import workloads as W

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def host_build():
    from demon_simulation_code_gb300 import build

    return build.build_host()


def run(driver, *args, cwd):
    r = subprocess.run([driver, *args], cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


def replay(oracle_lib, params, state, q, m, t0, end, data_dt, init_dt, rk2=False):
    """The reference's output loop on the oracle: rows (time, x, y, vx, vy)."""
    x, y, vx, vy = state
    move = oracle_lib.rk2_move_particles if rk2 else oracle_lib.rk4_move_particles
    rows = []
    te, t = t0, t0
    while te < end:
        te += data_dt
        x, y, vx, vy, _, t = move(x, y, vx, vy, q, m, params, init_dt, t, te)
        rows.append((t, x, y, vx, vy))
    return rows


def check_rows(ts, first, rows, tol=1e-12):
    for k, (t, x, y, vx, vy) in enumerate(rows):
        r = first + k
        assert ts["TIME"][r, 0] == t, (r, ts["TIME"][r, 0], t)
        for name, ref in (("X_POSITION", x), ("Y_POSITION", y), ("X_VELOCITY", vx), ("Y_VELOCITY", vy)):
            got = ts[name][r]
            err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300)
            assert err <= tol, (r, name, err)


ARGS = ["-n", "64", "-i", "3e-4", "-C", "1e4", "-g", "3", "-t", "1e-4", "-o", "0.00053", "--seed", "3"]


def test_driver_output_matches_oracle(host_build, oracle_lib, tmp_path):
    _, driver = host_build
    run(driver, *ARGS, "-e", "0.002", "-O", "run.fits", cwd=tmp_path)
    keys, tables = read_fits(str(tmp_path / "run.fits"))
    assert keys["FORCES"] == 1 | 2 | 4
    q, m = tables["CLOUD"]["CHARGE"].ravel(), tables["CLOUD"]["MASS"].ravel()
    ts = tables["TIME_STEP"]
    p = oracle.make_params(flags=1 | 2 | 4, shielding=2e4, confine=1e4, gamma=3.0)
    state = [ts[k][0] for k in ("X_POSITION", "Y_POSITION", "X_VELOCITY", "Y_VELOCITY")]
    rows = replay(oracle_lib, p, state, q, m, 0.0, 0.002, 0.00053, 1e-4)
    assert len(rows) == ts["TIME"].shape[0] - 1 == 4
    check_rows(ts, 1, rows)


def test_driver_rk2_matches_oracle(host_build, oracle_lib, tmp_path):
    _, driver = host_build
    run(driver, *ARGS, "-I", "-w", "1e-15", "5e-4", "1e-5", "-e", "0.002", "-O", "rk2.fits", cwd=tmp_path)
    keys, tables = read_fits(str(tmp_path / "rk2.fits"))
    assert keys["FORCES"] == 1 | 2 | 4 | 64
    q, m = tables["CLOUD"]["CHARGE"].ravel(), tables["CLOUD"]["MASS"].ravel()
    ts = tables["TIME_STEP"]
    p = oracle.make_params(flags=1 | 2 | 4 | 64, shielding=2e4, confine=1e4, gamma=3.0, drive_amplitude=1e-15,
                           drive_shift=5e-4, drive_const=1e-5)
    state = [ts[k][0] for k in ("X_POSITION", "Y_POSITION", "X_VELOCITY", "Y_VELOCITY")]
    rows = replay(oracle_lib, p, state, q, m, 0.0, 0.002, 0.00053, 1e-4, rk2=True)
    assert len(rows) == ts["TIME"].shape[0] - 1 == 4
    check_rows(ts, 1, rows)


def test_driver_other_forces_match_oracle(host_build, oracle_lib, tmp_path):
    """The reference's other force options through the driver, replayed on
    the oracle with the same forces and the stage times of each step."""
    _, driver = host_build
    run(driver, *ARGS, "-V", "400", "-B", "0.5", "-D", "-1", "3", "-w", "1e-15", "5e-4", "1e-5", "-S", "1e-15",
        "2e-4", "1e-3", "-G", "-1", "-E", "1e3", "2e-3", "-F", "1", "2e-3", "-e", "0.0016", "-O", "o.fits",
        cwd=tmp_path)
    keys, tables = read_fits(str(tmp_path / "o.fits"))
    flags = 4 | 8 | 64 | 128 | 256 | 1024 | 2048 | 4096 | 16384
    assert keys["FORCES"] == flags | 1 | 2  # -V and -D also set the Confinement and Drag bits
    q, m = tables["CLOUD"]["CHARGE"].ravel(), tables["CLOUD"]["MASS"].ravel()
    ts = tables["TIME_STEP"]
    p = oracle.make_params(flags=flags, shielding=2e4, confine=1e4, void_decay=400.0, magnetic=0.5,
                           drag_scale=-1.0, drag_offset=3.0, drive_amplitude=1e-15, drive_shift=5e-4,
                           drive_const=1e-5, rot_const=1e-15, rot_rmin=2e-4, rot_rmax=1e-3, gravity=-1.0,
                           electric=1e3, electric_radius=2e-3, vert_electric=1.0, vert_decay=2e-3)
    state = [ts[k][0] for k in ("X_POSITION", "Y_POSITION", "X_VELOCITY", "Y_VELOCITY")]
    rows = replay(oracle_lib, p, state, q, m, 0.0, 0.0016, 0.00053, 1e-4)
    assert len(rows) == ts["TIME"].shape[0] - 1 == 4
    check_rows(ts, 1, rows)


def test_driver_continue_appends_like_the_reference(host_build, oracle_lib, tmp_path):
    _, driver = host_build
    run(driver, *ARGS, "-e", "0.001", "-O", "c.fits", cwd=tmp_path)
    _, t1 = read_fits(str(tmp_path / "c.fits"))
    run(driver, "-c", "c.fits", "-o", "0.00053", "-t", "1e-4", "-e", "0.002", cwd=tmp_path)
    _, t2 = read_fits(str(tmp_path / "c.fits"))
    ts1, ts2 = t1["TIME_STEP"], t2["TIME_STEP"]
    n1 = ts1["TIME"].shape[0]
    for k in ts1:
        assert np.array_equal(ts2[k][:n1], ts1[k])  # earlier rows untouched
    q, m = t2["CLOUD"]["CHARGE"].ravel(), t2["CLOUD"]["MASS"].ravel()
    p = oracle.make_params(flags=1 | 2 | 4, shielding=2e4, confine=1e4, gamma=3.0)
    state = [ts1[k][n1 - 1] for k in ("X_POSITION", "Y_POSITION", "X_VELOCITY", "Y_VELOCITY")]
    rows = replay(oracle_lib, p, state, q, m, ts1["TIME"][n1 - 1, 0], 0.002, 0.00053, 1e-4)
    assert len(rows) == ts2["TIME"].shape[0] - n1 > 0
    check_rows(ts2, n1, rows)


@pytest.fixture(scope="module")
def api_check(host_build, tmp_path_factory):
    from demon_simulation_code_gb300 import build

    exe = str(tmp_path_factory.mktemp("hostapi") / "host_api_check")
    cmd = ["g++", *build.HOST_FLAGS, "-o", exe, os.path.join(HERE, "host_api_check.cpp"),
           "-L" + build.PKG, "-ldemon_gb300_host", "-ldemon_gb300", "-Wl,-rpath," + build.PKG]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("forces", ["basic", "other"])
@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_per_force_calls_match_the_fused_step(api_check, tmp_path, prec, forces):
    c = W.calm_cloud(96)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([c.n], dtype=np.int32).tofile(f)
        for a in (c.x, c.y, c.vx, c.vy, c.q, c.m):
            np.asarray(a, dtype=np.float64).tofile(f)
    out = {}
    for mode in ("fused", "host"):
        o = tmp_path / f"{mode}.bin"
        r = subprocess.run([api_check, str(inp), str(o), mode, "8", "1e-4", prec, forces], capture_output=True,
                           text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        out[mode] = np.fromfile(o, dtype=np.float64).reshape(4, c.n)
    f, h = out["fused"], out["host"]
    disp = np.abs(f[0] - c.x).max()
    assert disp > 0
    if prec == "fp64":
        for k in range(4):
            assert np.linalg.norm(f[k] - h[k]) <= 1e-12 * np.linalg.norm(f[k]), k
    else:
        assert np.abs(f[0] - h[0]).max() <= 1e-5 * disp
        assert np.abs(f[1] - h[1]).max() <= 1e-5 * np.abs(f[1] - c.y).max()
