"""Particles thrown far out of the cloud (needs a GB300).

A particle far from the rest of its 32-particle group (thrown out of the
cloud within a substep) stretches its group's box, and the culling test
must still find every pair within the cutoff.  These cases put such
particles in the input state -- singles metres out, close pairs of them far
away (they interact only with each other), and some just outside the
cloud's edge (they interact with edge particles) -- and check every culling
kernel variant against the oracle (the fraction of pairs swept is
printed)."""
import numpy as np
import pytest

import oracle
from demon_simulation_code_gb300 import DeviceCloud, _lib, workloads as W

pytestmark = pytest.mark.gpu


def e_F(fx, fy, rx, ry):
    return np.sqrt(np.sum((fx - rx) ** 2 + (fy - ry) ** 2) / np.sum(rx**2 + ry**2))


def outlier_cloud(n=4096, seed=21):
    c = W.disk_cloud(n, 5e-3, seed)  # kappa = 2e4: cutoff radius 5e-4 m
    rng = np.random.default_rng(seed + 1)
    idx = rng.choice(n, 112, replace=False)
    ang = rng.uniform(0, 2 * np.pi, 112)
    far = rng.uniform(0.5, 5.0, 112)
    # singles metres out
    c.x[idx[:48]] = far[:48] * np.cos(ang[:48])
    c.y[idx[:48]] = far[:48] * np.sin(ang[:48])
    # 16 close pairs metres out: 2e-4 m apart, inside the cutoff of each other
    for k in range(16):
        a, b = idx[48 + 2 * k], idx[49 + 2 * k]
        c.x[a] = far[48 + k] * np.cos(ang[48 + k])
        c.y[a] = far[48 + k] * np.sin(ang[48 + k])
        c.x[b] = c.x[a] + 2e-4 * np.cos(ang[80 + k])
        c.y[b] = c.y[a] + 2e-4 * np.sin(ang[80 + k])
    # just outside the disk's edge, within the cutoff of edge particles
    r_edge = 5e-3 + rng.uniform(1e-4, 4e-4, 32)
    c.x[idx[80:]] = r_edge * np.cos(ang[80:])
    c.y[idx[80:]] = r_edge * np.sin(ang[80:])
    return c


def test_every_culling_variant_with_outliers_matches_the_oracle(gpu_ctx, oracle_lib):
    c0 = outlier_cloud()
    rx, ry = oracle_lib.forces(c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, oracle.make_params(**c0.params()))
    pairs = c0.n * (c0.n - 1)
    names = [v for v in _lib.kernel_variants() if v.endswith(",cull>")]
    assert names
    for name in names:
        for split in (0, 3):
            c = DeviceCloud.from_cloud(gpu_ctx, c0)
            try:
                c.set_kernel(name, split)
            except _lib.DemonError:
                c.close()
                continue  # a cluster shape this GPU cannot schedule
            e0 = c.evaluated_pairs()
            fx, fy = c.eval_forces("fp32c")
            swept = (c.evaluated_pairs() - e0) / pairs
            err = e_F(fx, fy, rx, ry)
            print(name, split, "e_F %.2e swept %.3f" % (err, swept))
            assert err <= 1e-6, (name, split, err)
            assert np.all(np.isfinite(fx)) and np.all(np.isfinite(fy))
            assert 0.0 < swept <= 1.0, (name, split, swept)
            c.close()


def test_steps_with_outliers_track_fp64(gpu_ctx):
    """Two RK4 steps (re-sorted, boxes rebuilt by every stage) FP32C vs FP64
    on the outlier cloud: the same trajectory to FP32C force accuracy."""
    c0 = outlier_cloud(seed=33)
    a = DeviceCloud.from_cloud(gpu_ctx, c0)
    b = DeviceCloud.from_cloud(gpu_ctx, c0)
    a.step(2, 1e-5, "fp32c")
    b.step(2, 1e-5, "fp64")
    xa, ya, _, _ = a.download()
    xb, yb, _, _ = b.download()
    moved = np.hypot(xb - c0.x, yb - c0.y)
    assert np.max(np.hypot(xa - xb, ya - yb)) <= 1e-5 * np.max(moved) + 1e-15
