"""Generates tests/golden/*.npz from the reference's OWN code.

Runs the reference sources compiled by oracle/Makefile (`make ref`,
serial build, so the summation order is the reference's single-thread
order) on seeded inputs and records inputs and outputs.  Needs the
reference checkout named by the environment variable DEMON_REF_DIR (read at
build time only) and an x86-64 host.

    DEMON_REF_DIR=<reference checkout> python tests/golden/make_golden.py [fixture names]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from demon_simulation_code_gb300 import workloads as W  # noqa: E402

Q = W.Q_DUST
M = W.M_DUST

OTHER_FORCES = W.OTHER_FORCES
THERMAL_HEAT = 1e-14  # ThermalForce heatVal of the kick fixture [N]
# ForceFlag bits of the forces the fixtures exercise one at a time (Force.h:75-91)
EACH_FORCE = {"gravitational": 8, "driving": 64, "rotational": 128, "tv_drag": 256,
              "magnetic": 1024, "void": 2048, "electric": 4096, "vert_electric": 16384}


def disk(n, R, seed, vscale=0.0):
    rng = np.random.default_rng(seed)
    x, y = W.uniform_disk(rng, n, R)
    vx = rng.normal(0.0, vscale, n) if vscale else np.zeros(n)
    vy = rng.normal(0.0, vscale, n) if vscale else np.zeros(n)
    return x, y, vx, vy


def main():
    oracle.build(ref=True)
    ref = oracle.Reference()
    out = {}
    # 1. ShieldedCoulombForce::force1 alone
    cases = [
        ("pair_n2", 2, 1e-4, 2e4, 10),
        ("pair_n4", 4, 3e-4, 2e4, 11),
        ("pair_n64_dense", 64, 2e-4, 2e4, 12),      # many pairs inside the cutoff
        ("pair_n256_k1e2", 256, 5e-3, 1e2, 13),     # every pair inside the cutoff
        ("pair_disk512", 512, 5e-3, 2e4, 0),        # the N=512 disk workload
    ]
    for name, n, R, kappa, seed in cases:
        if name == "pair_disk512":
            c = W.disk512().clouds[0]
            x, y, q = c.x, c.y, c.q
        else:
            x, y, _, _ = disk(n, R, seed)
            q = np.random.default_rng(seed + 100).normal(Q, abs(Q) * 0.05, n)
        fx, fy = ref.shielded_coulomb(x, y, q, kappa)
        out[name] = dict(x=x, y=y, q=q, kappa=np.float64(kappa), fx=fx, fy=fy)
    # 2. every non-thermal force in driver order (Confinement+Drag+Rect+Coulomb)
    x, y, vx, vy = disk(128, 1e-3, 20, vscale=1e-3)
    q = np.full(128, Q)
    m = np.full(128, M)
    for name, flags in [("forces_conf_drag_coul", 1 | 2 | 4), ("forces_rect_drag_coul", 8192 | 2 | 4)]:
        p = oracle.make_params(flags=flags, shielding=2e4, confine=1e8, confine_x=1e8,
                               confine_y=2e8, gamma=3.0)
        fx, fy = ref.forces(x, y, vx, vy, q, m, p)
        out[name] = dict(x=x, y=y, vx=vx, vy=vy, q=q, m=m, flags=np.int64(flags), fx=fx, fy=fy)
    # 3. fixed-dt RK4 (reference CacheOperator + forces, stage bookkeeping
    # restated) on a well-conditioned cloud (see workloads.calm_cloud)
    c = W.calm_cloud(64, 3e-3, 30)
    x, y, vx, vy, q, m = c.x, c.y, c.vx, c.vy, c.q, c.m
    p = oracle.make_params(**c.params())
    rx, ry, rvx, rvy = ref.rk4_fixed(x, y, vx, vy, q, m, p, 1e-4, 25)
    out["rk4_fixed_n64"] = dict(x=x, y=y, vx=vx, vy=vy, q=q, m=m, dt=np.float64(1e-4),
                                steps=np.int64(25), x1=rx, y1=ry, vx1=rvx, vy1=rvy,
                                kappa=np.float64(c.shielding), confine=np.float64(c.confine))
    # 4. the reference's own moveParticles (adaptive dt), disk512 workload
    c = W.disk512().clouds[0]
    p = oracle.make_params(flags=1 | 2 | 4, shielding=2e4, confine=1e8, gamma=3.0)
    rx, ry, rvx, rvy, steps, t1 = ref.rk4_move_particles(c.x, c.y, c.vx, c.vy, c.q, c.m, p,
                                                         1e-4, 0.0, 3e-4)
    out["move_adaptive_disk512"] = dict(x=c.x, y=c.y, vx=c.vx, vy=c.vy, q=c.q, m=c.m,
                                        dt=np.float64(1e-4), end=np.float64(3e-4),
                                        steps=np.int64(steps), t1=np.float64(t1),
                                        x1=rx, y1=ry, vx1=rvx, vy1=rvy)
    # 5. each of the reference's other deterministic forces alone, and two
    # mixes with the pair force, at a non-zero force time
    x, y, vx, vy = disk(256, 2e-2, 40, vscale=1e-3)
    q = np.random.default_rng(41).normal(Q, abs(Q) * 0.05, 256)
    m = np.full(256, M)
    t = 0.0123
    d = dict(x=x, y=y, vx=vx, vy=vy, q=q, m=m, t=np.float64(t))
    mixes = {"mix_a": 2048 | 2 | 64 | 1024 | 128 | 4, "mix_b": 1 | 256 | 4096 | 8 | 16384 | 8192 | 4}
    for name, flags in list(EACH_FORCE.items()) + list(mixes.items()):
        p = oracle.make_params(flags=flags, shielding=2e4, confine=1e8, confine_x=1e8, confine_y=2e8,
                               gamma=3.0, **OTHER_FORCES)
        d[name + "_fx"], d[name + "_fy"] = ref.forces(x, y, vx, vy, q, m, p, t=t)
        d[name + "_flags"] = np.int64(flags)
    out["forces_other_t"] = d
    # 6. fixed-dt RK4 from t0 = 0.05 with the time-dependent forces
    c = W.calm_cloud(64, 3e-3, 30)
    flags = 1 | 4 | 64 | 256 | 1024 | 128
    p = oracle.make_params(flags=flags, shielding=c.shielding, confine=c.confine, **OTHER_FORCES)
    rx, ry, rvx, rvy = ref.rk4_fixed(c.x, c.y, c.vx, c.vy, c.q, c.m, p, 1e-4, 25, t0=0.05)
    out["rk4_fixed_time_n64"] = dict(x=c.x, y=c.y, vx=c.vx, vy=c.vy, q=c.q, m=c.m, dt=np.float64(1e-4),
                                     steps=np.int64(25), t0=np.float64(0.05), flags=np.int64(flags),
                                     kappa=np.float64(c.shielding), confine=np.float64(c.confine),
                                     x1=rx, y1=ry, vx1=rvx, vy1=rvy)
    # 7. the reference's own Runge_Kutta2::moveParticles (adaptive dt) from
    # t0 = 0.1 with a time-dependent force, disk512 workload
    c = W.disk512().clouds[0]
    flags = 1 | 2 | 4 | 64 | 1024
    p = oracle.make_params(flags=flags, shielding=2e4, confine=1e8, gamma=3.0, **OTHER_FORCES)
    rx, ry, rvx, rvy, steps, t1 = ref.rk2_move_particles(c.x, c.y, c.vx, c.vy, c.q, c.m, p, 1e-4, 0.1,
                                                         0.1 + 5e-4)
    out["rk2_move_adaptive_disk512"] = dict(x=c.x, y=c.y, vx=c.vx, vy=c.vy, q=c.q, m=c.m, dt=np.float64(1e-4),
                                            t0=np.float64(0.1), end=np.float64(0.1 + 5e-4),
                                            flags=np.int64(flags), steps=np.int64(steps), t1=np.float64(t1),
                                            x1=rx, y1=ry, vx1=rvx, vy1=rvy)
    # 8. the three thermal forces' kicks from the reference itself (its
    # RandomNumbers is clock-seeded, so only their distribution is pinned):
    # ThermalForce (heatVal THERMAL_HEAT, ThermalForce.cpp:118-122),
    # ThermalForceLocalized and TimeVaryingThermalForce
    x, y, vx, vy = disk(4096, 2e-2, 50)
    q = np.full(4096, Q)
    m = np.full(4096, M)
    d = dict(x=x, y=y, thermal_heat=np.float64(THERMAL_HEAT))
    for name, flags, tt in [("thermal", 16, 0.0), ("localized", 32, 0.0), ("tv", 512, 0.5)]:
        p = oracle.make_params(flags=flags, heat=THERMAL_HEAT, **OTHER_FORCES)
        d[name + "_fx"], d[name + "_fy"] = ref.forces(x, y, vx, vy, q, m, p, t=tt, thermal=True)
        d[name + "_t"] = np.float64(tt)
    out["thermal_other_ref"] = d
    only = sys.argv[1:]
    for name, d in out.items():
        if only and name not in only:
            continue
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, {k: np.shape(v) for k, v in d.items()})


if __name__ == "__main__":
    main()
