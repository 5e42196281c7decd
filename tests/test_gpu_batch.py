"""Batched clouds (one persistent launch per stage) vs the oracle and vs the
single-cloud path (needs a GB300)."""
import numpy as np
import pytest

import oracle
from demon_simulation_code_gb300 import DeviceBatch, DeviceCloud, workloads as W

pytestmark = pytest.mark.gpu


def e_F(fx, fy, rx, ry):
    return np.sqrt(np.sum((fx - rx) ** 2 + (fy - ry) ** 2) / np.sum(rx**2 + ry**2))


def small_batch(nclouds=12, seed=5):
    w = W.batch256(seed=seed, nclouds=nclouds, nmin=1, nmax=700)
    return w.clouds


def test_batch_forces_vs_oracle_per_cloud(gpu_ctx, oracle_lib):
    clouds = small_batch()
    b = DeviceBatch(gpu_ctx, clouds)
    fx, fy = b.eval_forces("fp32c")
    for c, gx, gy in zip(clouds, b.split(fx), b.split(fy)):
        rx, ry = oracle_lib.forces(c.x, c.y, c.vx, c.vy, c.q, c.m, oracle.make_params(**c.params()))
        if c.n > 1 and np.any(rx != 0):
            assert e_F(gx, gy, rx, ry) <= 1e-6, c.n


def test_every_batch_variant_matches_the_oracle(gpu_ctx, oracle_lib):
    """Each batch variant (culling ones included) on clouds that are sparse
    enough for the box test to skip groups."""
    from demon_simulation_code_gb300 import _lib

    clouds = W.batch256(seed=7, nclouds=10, nmin=30, nmax=3000).clouds
    refs = [oracle_lib.forces(c.x, c.y, c.vx, c.vy, c.q, c.m, oracle.make_params(**c.params())) for c in clouds]
    total = sum(c.n * c.n for c in clouds)
    for name in _lib.batch_variants():
        b = DeviceBatch(gpu_ctx, clouds)  # a fresh state per variant (the check steps it)
        b.set_kernel(name)
        e0 = b.evaluated_pairs()
        fx, fy = b.eval_forces("fp32c")
        swept = b.evaluated_pairs() - e0
        for c, gx, gy, (rx, ry) in zip(clouds, b.split(fx), b.split(fy), refs):
            assert e_F(gx, gy, rx, ry) <= 1e-6, (name, c.n)
        if name.endswith(",cull>"):
            print(name, "swept", swept / total)
            assert 0 < swept < total
        b.step(2, 1e-4)
        assert np.all(np.isfinite(b.download()[0]))
        b.close()


def test_batch_steps_match_single_cloud_steps(gpu_ctx):
    """Each cloud of a batch integrates like the same cloud stepped alone."""
    # well-conditioned clouds (minimum separation), uneven sizes and kappa
    clouds = []
    for k, n in enumerate((7, 64, 129, 300, 513, 31)):
        c = W.calm_cloud(n, 4e-4 * np.sqrt(n) + 1e-3, 40 + k)
        c.shielding = 4e3 + 500.0 * k
        clouds.append(c)
    b = DeviceBatch(gpu_ctx, clouds)
    b.step(20, 1e-4)
    bx, by, _, _ = b.download()
    for c, gx, gy in zip(clouds, b.split(bx), b.split(by)):
        s = DeviceCloud.from_cloud(gpu_ctx, c)
        s.step(20, 1e-4, "fp32c")
        sx, sy, _, _ = s.download()
        R = max(np.max(np.hypot(c.x, c.y)), 1e-6)
        assert np.max(np.hypot(gx - sx, gy - sy)) / R < 1e-6, c.n


def test_batch256_workload_runs_graph_captured(gpu_ctx):
    w = W.batch256()
    b = DeviceBatch(gpu_ctx, w.clouds)
    name, nitems, grid = b.info()
    assert name.startswith("batch_fp32c<") and nitems >= 256 and grid >= 152
    b.step(20, w.dt)  # 16-step CUDA graph + direct steps
    x, y, vx, vy = b.download()
    assert np.all(np.isfinite(x)) and np.all(np.isfinite(vy))
