"""Parity at the configurations' own sizes (needs a GB300).

* batch256 (256 clouds, N ~ U{64..4096}, per-cloud kappa/q/k_c): after a
  CUDA-graph replay of 16 steps, every cloud's FP32C forces at the state the
  graph reached against the oracle's FP64 forces of that state.
* disk512 (N = 512, FP64, 1000 steps of 1e-4 s, outputs every 100): the
  GPU's FP64 run against the oracle's.  This configuration is chaotic (close
  pairs are thrown out within tens of steps): a one-ulp change of one
  coordinate grows past the cloud's radius by step 50 in the oracle itself,
  so the two runs are gated where they can agree -- the first steps, and at
  every output a short segment from the GPU's own state -- and the divergence
  at each output is printed, not gated.
"""
import os

import numpy as np
import pytest

import oracle
from demon_simulation_code_gb300 import DeviceBatch, DeviceCloud, workloads as W

pytestmark = pytest.mark.gpu


def e_F(fx, fy, rx, ry):
    return np.sqrt(np.sum((fx - rx) ** 2 + (fy - ry) ** 2) / np.sum(rx**2 + ry**2))


def _threads():
    return max(1, len(os.sched_getaffinity(0)))


def test_batch256_every_cloud_vs_oracle_after_a_graph_replay(gpu_ctx, oracle_lib):
    w = W.batch256()
    b = DeviceBatch(gpu_ctx, w.clouds)
    b.step(16, w.dt)  # one replay of the 16-step CUDA graph
    x, y, vx, vy = b.download()
    fx, fy = b.eval_forces("fp32c")
    worst = 0.0
    parts = [b.split(a) for a in (x, y, vx, vy, fx, fy)]
    for c, cx, cy, cvx, cvy, gx, gy in zip(w.clouds, *parts):
        assert np.all(np.isfinite(cx)) and np.all(np.isfinite(cy))
        rx, ry = oracle_lib.forces(cx, cy, cvx, cvy, c.q, c.m, oracle.make_params(**c.params()),
                                   nthreads=_threads())
        e = e_F(gx, gy, rx, ry)
        worst = max(worst, e)
        assert e <= 1e-6, (c.n, e)
    print(f"batch256 after 16 graph-replayed steps: worst per-cloud e_F = {worst:.3e} over {len(w.clouds)} clouds")


def test_disk512_1000_step_fp64_run_against_the_oracle(gpu_ctx, oracle_lib):
    w = W.disk512()
    c = w.clouds[0]
    p = oracle.make_params(**c.params())
    R = float(np.max(np.hypot(c.x, c.y)))
    g = DeviceCloud.from_cloud(gpu_ctx, c)
    # the first steps, before the dynamics amplify last-bit differences
    g.step(5, w.dt, "fp64")
    ref = oracle_lib.rk4_fixed(c.x, c.y, c.vx, c.vy, c.q, c.m, p, w.dt, 5)
    gs = g.download()
    assert np.max(np.hypot(gs[0] - ref[0], gs[1] - ref[1])) / R <= 1e-12
    rows = []
    done = 5
    for k in range(1, 11):
        g.step(100 * k - done, w.dt, "fp64")  # graph-captured steps
        ref = oracle_lib.rk4_fixed(*ref, c.q, c.m, p, w.dt, 100 * k - done, step0=done, t0=done * w.dt)
        done = 100 * k
        gs = g.download()
        assert all(np.all(np.isfinite(a)) for a in gs)
        dev = np.hypot(gs[0] - ref[0], gs[1] - ref[1]) / R
        # local agreement: two steps from the GPU's own state, on both
        probe = DeviceCloud.from_cloud(gpu_ctx, c)
        probe.upload(*gs)
        probe.set_step_counter(done)
        probe.step(2, w.dt, "fp64", t=done * w.dt)
        a = probe.download()
        o = oracle_lib.rk4_fixed(*gs, c.q, c.m, p, w.dt, 2, step0=done, t0=done * w.dt)
        scale = max(np.max(np.hypot(gs[0], gs[1])), R)
        local = np.max(np.hypot(a[0] - o[0], a[1] - o[1])) / scale
        probe.close()
        rows.append((done, float(dev.max()), float(np.sqrt(np.mean(dev**2))), local))
        assert local <= 1e-10, (done, local)
    print("disk512 FP64 GPU vs oracle at each output (step, max |dp|/R, rms |dp|/R, 2-step local):")
    for r in rows:
        print("  %5d  %.3e  %.3e  %.2e" % r)
