"""Runge_Kutta2 (the midpoint method, Runge_Kutta2.cpp:23-78) on the CUDA
path (needs a GB300): fixed-dt steps against the oracle, the adaptive
moveParticles against the reference's own run, the batch, and the step
counter and force time it advances.  Tolerances as for RK4: FP64 1e-12
relative, FP32C 1e-7 on positions and 1e-5 on velocities."""
import os

import numpy as np
import pytest

import oracle
from demon_simulation_code_gb300 import DeviceBatch, DeviceCloud, workloads as W

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
OTHER = W.OTHER_FORCES


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
@pytest.mark.parametrize("nsteps", [5, 40])  # direct launches; CUDA-graph replays + remainder
def test_rk2_fixed_steps_vs_oracle(gpu_ctx, oracle_lib, prec, nsteps):
    c0 = W.calm_cloud(512, 1e-2, 7)
    p = dict(c0.params(), flags=1 | 2 | 4 | 16 | 64 | 256 | 1024, heat=1e-15, seed=4, **OTHER)
    ref = oracle_lib.rk2_fixed(c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, oracle.make_params(**p), 1e-4, nsteps,
                               step0=3, t0=0.25)
    c = DeviceCloud(gpu_ctx, c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, p)
    c.set_integrator(2)
    c.set_step_counter(3)
    t1 = c.step(nsteps, 1e-4, prec, t=0.25)
    assert c.get_step_counter() == 3 + nsteps
    t = 0.25
    for _ in range(nsteps):
        t += 1e-4
    assert t1 == t and c.get_time() == t
    tols = (1e-12,) * 4 if prec == "fp64" else (1e-7, 1e-7, 1e-5, 1e-5)
    for a, r, tol in zip(c.download(), ref, tols):
        assert rel(a, r) <= tol


def test_rk2_adaptive_vs_reference_golden(gpu_ctx):
    g = dict(np.load(os.path.join(GOLDEN, "rk2_move_adaptive_disk512.npz")))
    c = DeviceCloud(gpu_ctx, g["x"], g["y"], g["vx"], g["vy"], g["q"], g["m"],
                    dict(flags=int(g["flags"]), shielding=2e4, confine=1e8, gamma=3.0, **OTHER))
    c.set_integrator(2)
    t, steps = c.move_particles(float(g["end"]), float(g["dt"]), float(g["t0"]), "fp64", adaptive=True)
    assert steps == int(g["steps"]) and t == float(g["t1"])
    for a, k in zip(c.download(), ("x1", "y1", "vx1", "vy1")):
        assert rel(a, g[k]) <= 1e-12, k


def test_rk2_and_rk4_differ_and_switch_back(gpu_ctx, oracle_lib):
    c0 = W.calm_cloud(256, 1e-2, 9)
    p = c0.params()
    a = DeviceCloud(gpu_ctx, c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, p)
    a.set_integrator(2)
    a.step(20, 1e-4, "fp64")
    a.set_integrator(4)
    a.step(20, 1e-4, "fp64")
    x, y, vx, vy = oracle_lib.rk2_fixed(c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, oracle.make_params(**p), 1e-4, 20)
    ref = oracle_lib.rk4_fixed(x, y, vx, vy, c0.q, c0.m, oracle.make_params(**p), 1e-4, 20, step0=20, t0=20e-4)
    for u, r in zip(a.download(), ref):
        assert rel(u, r) <= 1e-12
    b = oracle_lib.rk4_fixed(c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, oracle.make_params(**p), 1e-4, 40)
    assert rel(ref[2], b[2]) > 1e-9  # the integrators are not the same
    with pytest.raises(Exception):
        a.set_integrator(3)


def test_batch_rk2_matches_single_clouds(gpu_ctx):
    clouds = [W.calm_cloud(n, 4e-4 * np.sqrt(n) + 1e-3, 60 + k) for k, n in enumerate((64, 300, 513))]
    b = DeviceBatch(gpu_ctx, clouds)
    b.set_integrator(2)
    b.step(20, 1e-4)
    bx, by, _, _ = b.download()
    for c, gx, gy in zip(clouds, b.split(bx), b.split(by)):
        s = DeviceCloud.from_cloud(gpu_ctx, c)
        s.set_integrator(2)
        s.step(20, 1e-4, "fp32c")
        sx, sy, _, _ = s.download()
        R = max(np.max(np.hypot(c.x, c.y)), 1e-6)
        assert np.max(np.hypot(gx - sx, gy - sy)) / R < 1e-6, c.n
