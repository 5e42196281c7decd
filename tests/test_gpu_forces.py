"""The reference's other per-particle forces on the CUDA path (needs a GB300):
ConfinementForceVoid, DrivingForce, MagneticForce, RotationalForce,
ThermalForceLocalized, TimeVaryingDragForce, TimeVaryingThermalForce,
ElectricForce, GravitationalForce, VertElectricForce, and the force time
that the time-dependent ones read.

They are evaluated in FP64 in the stage epilogue whatever the pair precision,
so alone they agree with the reference's fixtures to libm last-bit
differences (CUDA's exp/sin against glibc's): tolerance 1e-13 relative.
Mixed with the pair force they take the pair force's tolerance (FP64 1e-12,
FP32C 1e-6).  The counter-based thermal kicks are bit-identical to the
oracle's.
"""
import os

import numpy as np
import pytest

import oracle
from demon_simulation_code_gb300 import DeviceBatch, DeviceCloud, workloads as W

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL = {"fp64": 1e-12, "fp32c": 1e-6}
OTHER = W.OTHER_FORCES
SINGLE = ["gravitational", "driving", "rotational", "tv_drag", "magnetic", "void", "electric",
          "vert_electric"]


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def params(flags, **kw):
    d = dict(flags=flags, shielding=2e4, confine=1e8, confine_x=1e8, confine_y=2e8, gamma=3.0, **OTHER)
    d.update(kw)
    return d


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
@pytest.mark.parametrize("name", SINGLE + ["mix_a", "mix_b"])
def test_other_forces_vs_reference_golden(gpu_ctx, name, prec):
    g = golden("forces_other_t")
    c = DeviceCloud(gpu_ctx, g["x"], g["y"], g["vx"], g["vy"], g["q"], g["m"],
                    params(int(g[name + "_flags"])))
    c.set_time(float(g["t"]))
    fx, fy = c.eval_forces(prec)
    tol = 1e-13 if name in SINGLE else TOL[prec]
    assert rel(fx, g[name + "_fx"]) <= tol and rel(fy, g[name + "_fy"]) <= tol, name
    if name == "rotational":  # acts inside the annulus only, as the reference
        np.testing.assert_array_equal(fx == 0.0, g[name + "_fx"] == 0.0)
    if name == "gravitational":
        np.testing.assert_array_equal(fy, g[name + "_fy"])


def test_force_time_is_read_by_the_time_dependent_forces(gpu_ctx, oracle_lib):
    g = golden("forces_other_t")
    c = DeviceCloud(gpu_ctx, g["x"], g["y"], g["vx"], g["vy"], g["q"], g["m"], params(64 | 256))
    for t in (0.0, 0.25, 1.75):
        c.set_time(t)
        assert c.get_time() == t
        fx, fy = c.eval_forces("fp64")
        rx, ry = oracle_lib.forces(g["x"], g["y"], g["vx"], g["vy"], g["q"], g["m"],
                                   oracle.make_params(**params(64 | 256)), t=t)
        assert rel(fx, rx) <= 1e-13 and rel(fy, ry) <= 1e-13, t


@pytest.mark.parametrize("flags", [32, 512, 16 | 32 | 512])
@pytest.mark.parametrize("mode", [0, 1])
def test_other_thermal_kicks_bit_identical_to_oracle(gpu_ctx, oracle_lib, flags, mode):
    n = 3001
    rng = np.random.default_rng(4)
    x, y = W.uniform_disk(rng, n, 2e-2)
    p = params(flags, heat=1e-14, thermal_mode=mode, seed=99)
    c = DeviceCloud(gpu_ctx, x, y, np.zeros(n), np.zeros(n), np.full(n, W.Q_DUST), np.full(n, W.M_DUST), p)
    c.set_step_counter(41)
    c.set_time(0.3)
    fx, fy = c.eval_forces("fp64")
    rx, ry = oracle_lib.forces(x, y, np.zeros(n), np.zeros(n), np.full(n, W.Q_DUST), np.full(n, W.M_DUST),
                               oracle.make_params(**p), step=41, stage=1, t=0.3)
    np.testing.assert_array_equal(fx, rx)
    np.testing.assert_array_equal(fy, ry)


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_rk4_with_force_time_vs_reference_golden(gpu_ctx, prec):
    g = golden("rk4_fixed_time_n64")
    p = dict(flags=int(g["flags"]), shielding=float(g["kappa"]), confine=float(g["confine"]), **OTHER)
    c = DeviceCloud(gpu_ctx, g["x"], g["y"], g["vx"], g["vy"], g["q"], g["m"], p)
    t1 = c.step(int(g["steps"]), float(g["dt"]), prec, t=float(g["t0"]))
    tol = 1e-12 if prec == "fp64" else 1e-7
    for a, k in zip(c.download(), ("x1", "y1", "vx1", "vy1")):
        assert rel(a, g[k]) <= tol, (k, rel(a, g[k]))
    t = float(g["t0"])
    for _ in range(int(g["steps"])):
        t += float(g["dt"])
    assert t1 == t and c.get_time() == t


def test_force_time_continues_across_calls_and_move_particles(gpu_ctx, oracle_lib):
    c0 = W.calm_cloud(256, 1e-2, 5)
    flags = 1 | 2 | 4 | 64 | 256 | 512 | 1024 | 2048 | 4096 | 8 | 16384 | 128 | 32
    p = dict(c0.params(), flags=flags, heat=1e-15, seed=3, **OTHER)
    ref = oracle_lib.rk4_fixed(c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, oracle.make_params(**p), 1e-4, 30,
                               t0=0.5)
    a = DeviceCloud(gpu_ctx, c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, p)
    a.set_time(0.5)
    a.step(10, 1e-4, "fp64")
    a.step(20, 1e-4, "fp64")  # continues from the cloud's force time
    b = DeviceCloud(gpu_ctx, c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, p)
    t, steps = b.move_particles(0.5 + 29.5e-4, 1e-4, 0.5, "fp64")
    assert steps == 30 and b.get_time() == t
    for u, v, r in zip(a.download(), b.download(), ref):
        assert np.array_equal(u, v)
        assert rel(u, r) <= 1e-12


def test_batch_with_other_forces_vs_oracle(gpu_ctx, oracle_lib):
    clouds = []
    for k, n in enumerate([96, 700, 1500]):
        c = W.calm_cloud(n, 1e-2 * np.sqrt(n / 512), 20 + k)
        c.flags = c.flags | [64 | 256, 1024 | 128 | 2048, 4096 | 8 | 16384][k]
        c.extra = dict(OTHER, drive_amplitude=1e-13 * (1 + k))
        c.heat, c.seed = 1e-15, 5
        clouds.append(c)
    B = DeviceBatch(gpu_ctx, clouds)
    B.set_time(0.125)
    B.step(8, 1e-4, "fp32c")
    assert B.get_time() == pytest.approx(0.125 + 8e-4, rel=0, abs=1e-15)
    xs = B.download()
    off = 0
    for c in clouds:
        ref = oracle_lib.rk4_fixed(c.x, c.y, c.vx, c.vy, c.q, c.m, oracle.make_params(**c.params()), 1e-4, 8,
                                   t0=0.125)
        for a, r, tol in zip(xs, ref, (1e-7, 1e-7, 1e-5, 1e-5)):
            assert rel(a[off:off + c.n], r) <= tol
        off += c.n


def test_unknown_flag_bits_rejected(gpu_ctx):
    from demon_simulation_code_gb300 import DemonError

    n = 8
    z = np.zeros(n)
    c = DeviceCloud(gpu_ctx, np.arange(n) * 1e-3, z, z, z, np.full(n, W.Q_DUST), np.full(n, W.M_DUST))
    with pytest.raises(DemonError):
        c.set_forces(params(1 << 15))
    c.set_forces(params(32767 & ~(16 | 32 | 512)))
