"""The CPU oracle pinned against the reference (golden fixtures recorded from
the reference's own code, and the compiled reference itself when present)."""
import glob
import os

import numpy as np
import pytest

import oracle
from demon_simulation_code_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("name", ["pair_n2", "pair_n4", "pair_n64_dense", "pair_n256_k1e2",
                                  "pair_disk512"])
def test_pair_force_matches_reference_golden(oracle_lib, name):
    g = load(name)
    fx, fy = oracle_lib.shielded_coulomb(g["x"], g["y"], g["q"], float(g["kappa"]))
    # same visiting and accumulation order as the reference: equal up to the
    # last-bit differences of libm exp between machines
    np.testing.assert_allclose(fx, g["fx"], rtol=1e-13, atol=1e-13 * np.abs(g["fx"]).max())
    np.testing.assert_allclose(fy, g["fy"], rtol=1e-13, atol=1e-13 * np.abs(g["fy"]).max())
    assert np.any(g["fx"] != 0.0)


@pytest.mark.parametrize("name", ["forces_conf_drag_coul", "forces_rect_drag_coul"])
def test_all_forces_match_reference_golden(oracle_lib, name):
    g = load(name)
    p = oracle.make_params(flags=int(g["flags"]), shielding=2e4, confine=1e8, confine_x=1e8,
                           confine_y=2e8, gamma=3.0)
    fx, fy = oracle_lib.forces(g["x"], g["y"], g["vx"], g["vy"], g["q"], g["m"], p)
    assert rel(fx, g["fx"]) < 1e-14 and rel(fy, g["fy"]) < 1e-14


def test_rk4_fixed_matches_reference_golden(oracle_lib):
    g = load("rk4_fixed_n64")
    p = oracle.make_params(flags=1 | 2 | 4, shielding=float(g["kappa"]), confine=float(g["confine"]),
                           gamma=3.0)
    out = oracle_lib.rk4_fixed(g["x"], g["y"], g["vx"], g["vy"], g["q"], g["m"], p,
                               float(g["dt"]), int(g["steps"]))
    for a, k in zip(out, ("x1", "y1", "vx1", "vy1")):
        assert rel(a, g[k]) < 1e-13, k


def test_adaptive_move_particles_matches_reference_golden(oracle_lib):
    g = load("move_adaptive_disk512")
    p = oracle.make_params(flags=1 | 2 | 4, shielding=2e4, confine=1e8, gamma=3.0)
    x, y, vx, vy, steps, t1 = oracle_lib.rk4_move_particles(
        g["x"], g["y"], g["vx"], g["vy"], g["q"], g["m"], p, float(g["dt"]), 0.0, float(g["end"]))
    assert steps == int(g["steps"]) and t1 == float(g["t1"])
    for a, k in zip((x, y, vx, vy), ("x1", "y1", "vx1", "vy1")):
        assert rel(a, g[k]) < 1e-13, k


def test_oracle_bit_exact_against_compiled_reference(oracle_lib, ref_lib):
    rng = np.random.default_rng(7)
    for n, R, kappa in [(2, 1e-4, 2e4), (6, 2e-4, 2e4), (100, 3e-4, 2e4), (300, 5e-3, 1e2)]:
        x, y = W.uniform_disk(rng, n, R)
        q = rng.normal(W.Q_DUST, 1e-16, n)
        a = ref_lib.shielded_coulomb(x, y, q, kappa)
        b = oracle_lib.shielded_coulomb(x, y, q, kappa)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), (n, R, kappa)


def test_oracle_rk4_bit_exact_against_compiled_reference(oracle_lib, ref_lib):
    c = W.disk512().clouds[0]
    p = oracle.make_params(flags=1 | 2 | 4, shielding=2e4, confine=1e8, gamma=3.0)
    a = ref_lib.rk4_fixed(c.x, c.y, c.vx, c.vy, c.q, c.m, p, 1e-4, 10)
    b = oracle_lib.rk4_fixed(c.x, c.y, c.vx, c.vy, c.q, c.m, p, 1e-4, 10)
    assert all(np.array_equal(u, v) for u, v in zip(a, b))


def test_omp_pair_force_close_to_serial(oracle_lib):
    c = W.disk512().clouds[0]
    a = oracle_lib.shielded_coulomb(c.x, c.y, c.q, 2e4)
    b = oracle_lib.shielded_coulomb(c.x, c.y, c.q, 2e4, nthreads=4)
    assert rel(b[0], a[0]) < 1e-14 and rel(b[1], a[1]) < 1e-14


def test_odd_n_extension(oracle_lib):
    """Odd n (outside the reference's domain) equals the brute-force formula."""
    rng = np.random.default_rng(3)
    n = 37
    x, y = W.uniform_disk(rng, n, 3e-4)
    q = np.full(n, W.Q_DUST)
    fx, fy = oracle_lib.shielded_coulomb(x, y, q, 2e4)
    C = oracle_lib.coulomb()
    bx = np.zeros(n)
    by = np.zeros(n)
    for i in range(n):
        for j in range(n):
            if i == j:
                continue
            dx, dy = x[i] - x[j], y[i] - y[j]
            r = np.sqrt(dx * dx + dy * dy)
            a = r * 2e4
            if a < 10.0:
                f = C * q[i] * q[j] * (1 + a) * np.exp(-a) / r**3
                bx[i] += f * dx
                by[i] += f * dy
    assert rel(fx, bx) < 1e-13 and rel(fy, by) < 1e-13


def test_philox_known_answers(oracle_lib):
    # Philox4x32-10 known-answer vectors published with Random123
    assert oracle_lib.philox([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert oracle_lib.philox([0xffffffff] * 4, [0xffffffff] * 2) == [
        0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert oracle_lib.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                             [0xa4093822, 0x299f31d0]) == [0xd16cfe09, 0x94fdcceb, 0x5001e420,
                                                           0x24126ea1]


def test_thermal_statistics(oracle_lib):
    p = oracle.make_params(flags=16, heat=1e-14, thermal_mode=1, seed=1)
    tx, ty = oracle_lib.thermal(p, 20000, 5, 2)
    v = np.concatenate([tx, ty]) / 1e-14
    assert abs(v.mean()) < 0.03 and abs(v.std() - 1.0) < 0.03
    p0 = oracle.make_params(flags=16, heat=1e-14, thermal_mode=0, seed=1)
    tx, ty = oracle_lib.thermal(p0, 20000, 5, 2)
    mag = np.hypot(tx, ty) / 1e-14
    assert mag.max() <= 1.0 and abs(mag.mean() - 0.5) < 0.02


def test_modify_timestep_checked_pairs(oracle_lib):
    """Offset-3 pairs between 4-blocks are never checked (Integrator.cpp:117)."""
    n = 8
    x = np.arange(n) * 1.0e-2
    y = np.zeros(n)
    # put particle 0 (block 0, k=0) next to particle 5 (block 1, m=1): (k-m) mod 4 = 3
    x[5] = x[0] + 1e-6
    assert oracle_lib.checked_min_dist(x, y) > 1e-3
    assert oracle_lib.modify_timestep(x, y, 1e-4) == 1e-4
    # next to particle 4 (m=0): offset 0, checked
    x[5] = 5e-2
    x[4] = x[0] + 1e-6
    assert oracle_lib.checked_min_dist(x, y) < 2e-6
    assert oracle_lib.modify_timestep(x, y, 1e-4) == pytest.approx(1e-4 / 1e3)


# the reference's other forces (fixtures by tests/golden/make_golden.py)
OTHER_FORCES = W.OTHER_FORCES
OTHER_NAMES = ["gravitational", "driving", "rotational", "tv_drag", "magnetic", "void", "electric",
               "vert_electric", "mix_a", "mix_b"]


def other_params(flags):
    return oracle.make_params(flags=flags, shielding=2e4, confine=1e8, confine_x=1e8, confine_y=2e8,
                              gamma=3.0, **OTHER_FORCES)


@pytest.mark.parametrize("name", OTHER_NAMES)
def test_other_forces_match_reference_golden(oracle_lib, name):
    g = load("forces_other_t")
    p = other_params(int(g[name + "_flags"]))
    fx, fy = oracle_lib.forces(g["x"], g["y"], g["vx"], g["vy"], g["q"], g["m"], p, t=float(g["t"]))
    ex, ey = g[name + "_fx"], g[name + "_fy"]
    assert np.any(ex != 0.0) or np.any(ey != 0.0)
    # per-particle arithmetic in the reference's order: libm last-bit
    # differences between machines at most
    assert rel(fx, ex) < 1e-14 and rel(fy, ey) < 1e-14


def test_other_forces_exercise_their_branches():
    g = load("forces_other_t")
    r = np.hypot(g["x"], g["y"])
    inside = (r > OTHER_FORCES["rot_rmin"]) & (r < OTHER_FORCES["rot_rmax"])
    assert 0 < inside.sum() < len(r)
    # RotationalForce acts only inside its annulus
    assert np.all(g["rotational_fx"][~inside] == 0.0) and np.all(g["rotational_fx"][inside] != 0.0)
    # GravitationalForce is F_y = m*g, F_x = 0
    assert np.all(g["gravitational_fx"] == 0.0)
    np.testing.assert_array_equal(g["gravitational_fy"], g["m"] * OTHER_FORCES["gravity"])


def test_rk4_with_force_time_matches_reference_golden(oracle_lib):
    g = load("rk4_fixed_time_n64")
    p = oracle.make_params(flags=int(g["flags"]), shielding=float(g["kappa"]), confine=float(g["confine"]),
                           **OTHER_FORCES)
    out = oracle_lib.rk4_fixed(g["x"], g["y"], g["vx"], g["vy"], g["q"], g["m"], p, float(g["dt"]),
                               int(g["steps"]), t0=float(g["t0"]))
    for a, k in zip(out, ("x1", "y1", "vx1", "vy1")):
        assert rel(a, g[k]) < 1e-13, k
    # the stage times matter: starting the same steps at t0 = 0 ends elsewhere
    out0 = oracle_lib.rk4_fixed(g["x"], g["y"], g["vx"], g["vy"], g["q"], g["m"], p, float(g["dt"]),
                                int(g["steps"]))
    assert rel(out0[2], g["vx1"]) > 1e-6


def test_other_forces_bit_exact_against_compiled_reference(oracle_lib, ref_lib):
    rng = np.random.default_rng(9)
    n = 128
    x, y = W.uniform_disk(rng, n, 2e-2)
    vx, vy = rng.normal(0, 1e-3, n), rng.normal(0, 1e-3, n)
    q = rng.normal(W.Q_DUST, abs(W.Q_DUST) * 0.05, n)
    m = np.full(n, W.M_DUST)
    for flags in [8, 64, 128, 256, 1024, 2048, 4096, 16384, 32767 & ~(16 | 32 | 512)]:
        for t in (0.0, 0.37):
            p = other_params(flags)
            a = ref_lib.forces(x, y, vx, vy, q, m, p, t=t)
            b = oracle_lib.forces(x, y, vx, vy, q, m, p, t=t)
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), (flags, t)
    c = W.calm_cloud(64, 3e-3, 31)
    p = oracle.make_params(flags=1 | 4 | 64 | 256 | 1024 | 128 | 2048, shielding=c.shielding,
                           confine=c.confine, **OTHER_FORCES)
    a = ref_lib.rk4_fixed(c.x, c.y, c.vx, c.vy, c.q, c.m, p, 1e-4, 12, t0=0.2)
    b = oracle_lib.rk4_fixed(c.x, c.y, c.vx, c.vy, c.q, c.m, p, 1e-4, 12, t0=0.2)
    assert all(np.array_equal(u, v) for u, v in zip(a, b))


def test_rk2_matches_reference_golden(oracle_lib):
    """Runge_Kutta2::moveParticles, adaptive dt, from t0 = 0.1 with a
    time-dependent force (the reference's own run)."""
    g = load("rk2_move_adaptive_disk512")
    p = oracle.make_params(flags=int(g["flags"]), shielding=2e4, confine=1e8, gamma=3.0, **OTHER_FORCES)
    x, y, vx, vy, steps, t1 = oracle_lib.rk2_move_particles(g["x"], g["y"], g["vx"], g["vy"], g["q"], g["m"], p,
                                                            float(g["dt"]), float(g["t0"]), float(g["end"]))
    assert steps == int(g["steps"]) and t1 == float(g["t1"])
    for a, k in zip((x, y, vx, vy), ("x1", "y1", "vx1", "vy1")):
        assert rel(a, g[k]) < 1e-13, k


def test_rk2_bit_exact_against_compiled_reference(oracle_lib, ref_lib):
    c = W.calm_cloud(64, 3e-3, 32)
    p = oracle.make_params(flags=1 | 2 | 4 | 64 | 256, shielding=c.shielding, confine=c.confine, **OTHER_FORCES)
    a = ref_lib.rk2_move_particles(c.x, c.y, c.vx, c.vy, c.q, c.m, p, 1e-4, 0.2, 0.2 + 11.5e-4)
    b = oracle_lib.rk2_move_particles(c.x, c.y, c.vx, c.vy, c.q, c.m, p, 1e-4, 0.2, 0.2 + 11.5e-4)
    assert a[4] == b[4] == 12 and a[5] == b[5]
    assert all(np.array_equal(u, v) for u, v in zip(a[:4], b[:4]))
    # a calm cloud keeps dt: the fixed-dt restatement takes the same steps
    f = oracle_lib.rk2_fixed(c.x, c.y, c.vx, c.vy, c.q, c.m, p, 1e-4, 12, t0=0.2)
    assert all(np.array_equal(u, v) for u, v in zip(a[:4], f))


def _kick_stats(fx, fy, scale):
    u = np.hypot(fx, fy) / scale
    return u, np.arctan2(fy, fx)


@pytest.mark.parametrize("kind", ["thermal", "localized", "tv"])
def test_thermal_kicks_match_reference_distribution(oracle_lib, kind):
    """ThermalForce (heatVal*U*(cos t, sin t), ThermalForce.cpp:118-122),
    ThermalForceLocalized and TimeVaryingThermalForce: the reference's kicks
    (clock-seeded) and the oracle's counter-based kicks have the same scale
    per region / time and the same magnitude and angle distributions."""
    from scipy import stats

    g = load("thermal_other_ref")
    n = len(g["x"])
    flags = {"thermal": 16, "localized": 32, "tv": 512}[kind]
    t = float(g[kind + "_t"])
    heat = float(g["thermal_heat"])
    p = oracle.make_params(flags=flags, heat=heat, thermal_mode=0, seed=11, **OTHER_FORCES)
    zeros = np.zeros(n)
    fx, fy = oracle_lib.forces(g["x"], g["y"], zeros, zeros, np.full(n, W.Q_DUST), np.full(n, W.M_DUST),
                               p, step=3, stage=2, t=t)
    if kind == "thermal":
        scale = np.full(n, heat)
    elif kind == "localized":
        inside = np.hypot(g["x"], g["y"]) < OTHER_FORCES["heat_radius"]
        scale = np.where(inside, OTHER_FORCES["heat_in"], OTHER_FORCES["heat_out"])
    else:
        scale = np.full(n, OTHER_FORCES["heat_scale"] * t + OTHER_FORCES["heat_offset"])
    ur, ar = _kick_stats(g[kind + "_fx"], g[kind + "_fy"], scale)
    uo, ao = _kick_stats(fx, fy, scale)
    for u in (ur, uo):
        assert u.max() <= 1.0 + 1e-12 and abs(u.mean() - 0.5) < 0.03
    assert stats.ks_2samp(ur, uo).pvalue > 1e-3
    assert stats.ks_2samp(ar, ao).pvalue > 1e-3


def test_golden_files_present():
    assert len(glob.glob(os.path.join(GOLDEN, "*.npz"))) >= 12
