"""CUDA path vs the oracle and the reference's golden fixtures (needs a GB300).

Tolerances (force error e_F = ||F_gpu - F_ref||_2 / ||F_ref||_2 over the 2N
vector, as the parity target states them): FP64 <= 1e-12, FP32C <= 1e-6.
The cutoff decision itself must agree exactly, which the per-particle check
(|dF_i| / sum_j |F_ij|) would expose: a flipped pair changes one particle's
force by a finite fraction.
"""
import os

import numpy as np
import pytest

import oracle
from demon_simulation_code_gb300 import DeviceCloud, workloads as W

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL = {"fp64": 1e-12, "fp32c": 1e-6}


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def e_F(fx, fy, rx, ry):
    return np.sqrt(np.sum((fx - rx) ** 2 + (fy - ry) ** 2) / np.sum(rx**2 + ry**2))


def abs_pair_sum(x, y, q, kappa, C):
    """sum_j |F_ij| per particle (normaliser robust to cancellation)."""
    dx = x[:, None] - x[None, :]
    dy = y[:, None] - y[None, :]
    r = np.sqrt(dx * dx + dy * dy)
    np.fill_diagonal(r, np.inf)
    a = r * kappa
    f = np.where(a < 10.0, np.abs(C * q[:, None] * q[None, :]) * (1 + a) * np.exp(-a) / r**2, 0.0)
    return f.sum(axis=1)


def coulomb_cloud(ctx, x, y, q, kappa):
    n = len(x)
    return DeviceCloud(ctx, x, y, np.zeros(n), np.zeros(n), q, np.full(n, W.M_DUST),
                       dict(flags=W.SHIELDED_COULOMB, shielding=kappa))


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
@pytest.mark.parametrize("name", ["pair_n2", "pair_n4", "pair_n64_dense", "pair_n256_k1e2",
                                  "pair_disk512"])
def test_pair_force_vs_reference_golden(gpu_ctx, oracle_lib, name, prec):
    g = golden(name)
    kappa = float(g["kappa"])
    c = coulomb_cloud(gpu_ctx, g["x"], g["y"], g["q"], kappa)
    fx, fy = c.eval_forces(prec)
    err = e_F(fx, fy, g["fx"], g["fy"])
    assert err <= TOL[prec], err
    s = abs_pair_sum(g["x"], g["y"], g["q"], kappa, oracle_lib.coulomb())
    worst = np.max(np.hypot(fx - g["fx"], fy - g["fy"]) / np.maximum(s, 1e-300))
    assert worst <= 10 * TOL[prec], worst


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
@pytest.mark.parametrize("n", [1, 2, 3, 5, 63, 64, 65, 511, 513, 1000, 2049])
def test_pair_force_ragged_sizes(gpu_ctx, oracle_lib, n, prec):
    rng = np.random.default_rng(n)
    R = 3e-4 * np.sqrt(max(n, 1))
    x, y = W.uniform_disk(rng, n, R)
    q = rng.normal(W.Q_DUST, 5e-17, n)
    c = coulomb_cloud(gpu_ctx, x, y, q, 2e4)
    fx, fy = c.eval_forces(prec)
    rx, ry = oracle_lib.shielded_coulomb(x, y, q, 2e4)
    if n == 1:
        assert fx[0] == 0.0 and fy[0] == 0.0
        return
    assert e_F(fx, fy, rx, ry) <= TOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_pair_force_disk16k(gpu_ctx, oracle_lib, prec):
    c0 = W.disk16k(thermal=False).clouds[0]
    c = coulomb_cloud(gpu_ctx, c0.x, c0.y, c0.q, 2e4)
    fx, fy = c.eval_forces(prec)
    rx, ry = oracle_lib.shielded_coulomb(c0.x, c0.y, c0.q, 2e4, nthreads=8)
    err = e_F(fx, fy, rx, ry)
    print(f"disk16k {prec} e_F = {err:.3e}")
    assert err <= TOL[prec]


def test_cutoff_borderline_pairs_decided_like_reference(gpu_ctx, oracle_lib):
    """Pairs placed within a few ulp of kappa*r = 10 on both sides."""
    kappa = 2e4
    rc = 10.0 / kappa
    n = 64
    x = np.zeros(n)
    y = np.zeros(n)
    for k in range(n // 2):
        d = rc * (1.0 + (k - n // 4) * 2.0**-50)
        x[2 * k] = 0.01 * k
        x[2 * k + 1] = 0.01 * k + d
        y[2 * k] = y[2 * k + 1] = 1e-3 * k
    q = np.full(n, W.Q_DUST)
    rx, ry = oracle_lib.shielded_coulomb(x, y, q, kappa)
    assert 0 < np.count_nonzero(rx) < n
    for prec in ("fp64", "fp32c"):
        c = coulomb_cloud(gpu_ctx, x, y, q, kappa)
        fx, fy = c.eval_forces(prec)
        assert np.array_equal(fx != 0.0, rx != 0.0), prec
        assert e_F(fx, fy, rx, ry) <= TOL[prec]


@pytest.mark.parametrize("name", ["forces_conf_drag_coul", "forces_rect_drag_coul"])
@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_all_forces_vs_reference_golden(gpu_ctx, name, prec):
    g = golden(name)
    c = DeviceCloud(gpu_ctx, g["x"], g["y"], g["vx"], g["vy"], g["q"], g["m"],
                    dict(flags=int(g["flags"]), shielding=2e4, confine=1e8, confine_x=1e8,
                         confine_y=2e8, gamma=3.0))
    fx, fy = c.eval_forces(prec)
    assert rel(fx, g["fx"]) <= TOL[prec] and rel(fy, g["fy"]) <= TOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_rk4_fixed_vs_reference_golden(gpu_ctx, prec):
    g = golden("rk4_fixed_n64")
    c = DeviceCloud(gpu_ctx, g["x"], g["y"], g["vx"], g["vy"], g["q"], g["m"],
                    dict(flags=1 | 2 | 4, shielding=float(g["kappa"]), confine=float(g["confine"]),
                         gamma=3.0))
    t = c.step(int(g["steps"]), float(g["dt"]), prec, t=0.0)
    x, y, vx, vy = c.download()
    tol = 1e-12 if prec == "fp64" else 1e-7
    for a, k in zip((x, y, vx, vy), ("x1", "y1", "vx1", "vy1")):
        assert rel(a, g[k]) <= tol, (k, rel(a, g[k]))
    assert t == pytest.approx(25e-4)


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_rk4_trajectory_100_steps_vs_oracle(gpu_ctx, oracle_lib, prec):
    """Gated short-horizon trajectory on a well-conditioned cloud (minimum
    separation 4e-4 m).  Uniform-random disks contain pairs ~1e-6 m apart
    for which RK4 at dt = 1e-4 s is unstable, so last-bit force differences
    grow without bound there; those are reported, not gated."""
    c0 = W.calm_cloud(512, 1e-2, 1)
    p = oracle.make_params(**c0.params())
    ref = oracle_lib.rk4_fixed(c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, p, 1e-4, 100)
    c = DeviceCloud.from_cloud(gpu_ctx, c0)
    c.step(100, 1e-4, prec)  # 100 steps: CUDA-graph replays + remainder
    out = c.download()
    R = 1e-2
    errx = np.max(np.hypot(out[0] - ref[0], out[1] - ref[1])) / R
    errv = rel(out[2], ref[2])
    assert errx <= (1e-12 if prec == "fp64" else 1e-7), errx
    assert errv <= (1e-10 if prec == "fp64" else 1e-5), errv


def test_graph_and_direct_steps_identical(gpu_ctx):
    c0 = W.disk512().clouds[0]
    a = DeviceCloud.from_cloud(gpu_ctx, c0)
    b = DeviceCloud.from_cloud(gpu_ctx, c0)
    a.step(40, 1e-4, "fp32c")
    for _ in range(40):
        b.step(1, 1e-4, "fp32c")
    assert all(np.array_equal(u, v) for u, v in zip(a.download(), b.download()))


@pytest.mark.parametrize("mode", [0, 1])
def test_thermal_force_vs_oracle(gpu_ctx, oracle_lib, mode):
    n = 3000
    rng = np.random.default_rng(9)
    x, y = W.uniform_disk(rng, n, 1e-2)
    params = dict(flags=W.THERMAL, heat=1e-14, thermal_mode=mode, seed=77)
    c = DeviceCloud(gpu_ctx, x, y, np.zeros(n), np.zeros(n), np.full(n, W.Q_DUST),
                    np.full(n, W.M_DUST), params)
    c.set_step_counter(123)
    fx, fy = c.eval_forces("fp64")
    tx, ty = oracle_lib.thermal(oracle.make_params(**params), n, 123, 1)
    assert rel(fx, tx) < 1e-14 and rel(fy, ty) < 1e-14


def test_thermal_rk4_fp64_vs_oracle(gpu_ctx, oracle_lib):
    c0 = W.calm_cloud(512, 1e-2, 2)
    params = dict(flags=1 | 2 | 4 | 16, shielding=5e3, confine=1e4, gamma=3.0, heat=1e-14,
                  thermal_mode=1, seed=1)
    ref = oracle_lib.rk4_fixed(c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m,
                               oracle.make_params(**params), 1e-4, 20, step0=5)
    c = DeviceCloud(gpu_ctx, c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, params)
    c.set_step_counter(5)
    c.step(20, 1e-4, "fp64")
    assert c.get_step_counter() == 25
    out = c.download()
    for a, b in zip(out, ref):
        assert rel(a, b) < 1e-12


def test_adaptive_dt_vs_reference_golden(gpu_ctx):
    g = golden("move_adaptive_disk512")
    c = DeviceCloud(gpu_ctx, g["x"], g["y"], g["vx"], g["vy"], g["q"], g["m"],
                    dict(flags=1 | 2 | 4, shielding=2e4, confine=1e8, gamma=3.0))
    t, steps = c.move_particles(float(g["end"]), float(g["dt"]), 0.0, "fp64", adaptive=True)
    assert steps == int(g["steps"]) and t == float(g["t1"])
    out = c.download()
    for a, k in zip(out, ("x1", "y1", "vx1", "vy1")):
        assert rel(a, g[k]) <= 1e-12, k


def test_modify_timestep_vs_oracle(gpu_ctx, oracle_lib):
    for seed in range(4):
        c0 = W.disk_cloud(1024, 5e-3 * (seed + 1), seed)
        c = DeviceCloud.from_cloud(gpu_ctx, c0)
        dmin, dt = c.modify_timestep(1e-4)
        assert dmin == np.float32(oracle_lib.checked_min_dist(c0.x, c0.y))
        assert dt == oracle_lib.modify_timestep(c0.x, c0.y, 1e-4)


def test_diagnostics_vs_oracle(gpu_ctx, oracle_lib):
    c0 = W.disk_cloud(2000, 2e-3, 5)
    rng = np.random.default_rng(1)
    c0.vx = rng.normal(0, 1e-3, c0.n)
    c0.vy = rng.normal(0, 1e-3, c0.n)
    c = DeviceCloud.from_cloud(gpu_ctx, c0)
    d = c.diagnostics()
    r = oracle_lib.diagnostics(c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m,
                               oracle.make_params(**c0.params()))
    np.testing.assert_allclose(d, r, rtol=1e-11)


def test_nonfinite_position_is_reported(gpu_ctx):
    from demon_simulation_code_gb300 import DemonError

    c0 = W.disk512().clouds[0]
    c0.x[3] = np.nan
    c = DeviceCloud.from_cloud(gpu_ctx, c0)
    c.step(1, 1e-4, "fp32c")
    with pytest.raises(DemonError):
        c.download()
    # the context stays usable
    ok = DeviceCloud.from_cloud(gpu_ctx, W.disk512().clouds[0])
    ok.step(1, 1e-4, "fp32c")
    assert np.all(np.isfinite(ok.download()[0]))


def test_bad_arguments_rejected(gpu_ctx):
    from demon_simulation_code_gb300 import DemonError

    c = DeviceCloud.from_cloud(gpu_ctx, W.disk512().clouds[0])
    with pytest.raises(DemonError):
        c.set_forces(dict(flags=4, shielding=-1.0))
    with pytest.raises(DemonError):
        c.set_forces(dict(flags=1 << 20))
    with pytest.raises(DemonError):
        c.step(-1, 1e-4)
    odd = DeviceCloud(gpu_ctx, np.zeros(6), np.arange(6.0), np.zeros(6), np.zeros(6),
                      np.full(6, W.Q_DUST), np.full(6, W.M_DUST))
    with pytest.raises(DemonError):
        odd.modify_timestep(1e-4)


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_forces_after_morton_reorder_are_in_caller_order(gpu_ctx, oracle_lib, prec):
    """After steps the device holds the cloud in Morton order; every array
    crossing the ABI must still be in the caller's order."""
    c0 = W.calm_cloud(700, 1e-2, 3)
    c = DeviceCloud.from_cloud(gpu_ctx, c0)
    c.set_reorder_interval(1)
    c.step(3, 1e-4, "fp64")
    x, y, vx, vy = c.download()
    fx, fy = c.eval_forces(prec)
    p = oracle.make_params(**c0.params())
    rx, ry = oracle_lib.forces(x, y, vx, vy, c0.q, c0.m, p)
    assert e_F(fx, fy, rx, ry) <= TOL[prec]
    # upload resets the order; charges and masses must survive it
    c.upload(x, y, vx, vy)
    fx2, fy2 = c.eval_forces(prec)
    assert e_F(fx2, fy2, rx, ry) <= TOL[prec]


def test_reorder_interval_does_not_change_fp64_results_beyond_rounding(gpu_ctx):
    c0 = W.calm_cloud(512, 1e-2, 4)
    outs = []
    for interval in (0, 1, 4, 16):
        c = DeviceCloud.from_cloud(gpu_ctx, c0)
        c.set_reorder_interval(interval)
        c.step(40, 1e-4, "fp64")
        outs.append(c.download())
    for o in outs[1:]:
        for a, b in zip(o, outs[0]):
            assert rel(a, b) < 1e-13


# kernel families by precision: FP32C has the shared-memory (fp32c) and the
# streamed (fp32s) sweeps
FAMILIES = {"fp64": ("fp64<",), "fp32c": ("fp32c<",)}


def _variants(prec):
    from demon_simulation_code_gb300 import _lib

    return [v for v in _lib.kernel_variants() if v.startswith(FAMILIES[prec])]


@pytest.mark.parametrize("n", [65, 3000])
@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_every_kernel_variant_and_split_is_correct(gpu_ctx, oracle_lib, prec, n):
    """The autotuner may pick any variant/split: every one must pass parity."""
    c0 = W.disk_cloud(n, 2.5e-3 * np.sqrt(n / 3000), 21)
    rx, ry = oracle_lib.forces(c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m,
                               oracle.make_params(**c0.params()))
    names = _variants(prec)
    assert names
    for name in names:
        for split in (1, 2, 3, 5, 8, 16, 0):
            c = DeviceCloud.from_cloud(gpu_ctx, c0)
            try:
                c.set_kernel(name, split)
            except Exception:  # e.g. a cluster size the device cannot schedule
                continue
            fx, fy = c.eval_forces(prec)
            assert e_F(fx, fy, rx, ry) <= TOL[prec], (name, split)
            c.step(2, 1e-4, prec)  # stage path through the same variant
            assert np.all(np.isfinite(c.download()[0]))


@pytest.mark.parametrize("name", ["fp32c<8,4,256,false,cull>", "fp32c<4,2,128,false,cull>",
                                  "fp32c<8,4,256,true,cull>"])
def test_culled_variants_on_a_collapsed_cloud(gpu_ctx, oracle_lib, name):
    """A cloud a few cutoffs across: many j groups lie entirely inside the
    cutoff of an i tile (the path without filter or queue), the rest near it."""
    c0 = W.disk_cloud(2048, 1.2e-3, 23)
    rx, ry = oracle_lib.forces(c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, oracle.make_params(**c0.params()))
    for split in (1, 4, 16):
        c = DeviceCloud.from_cloud(gpu_ctx, c0)
        try:
            c.set_kernel(name, split)
        except Exception:  # a cluster size the device cannot schedule
            c.close()
            continue
        fx, fy = c.eval_forces("fp32c")
        assert e_F(fx, fy, rx, ry) <= TOL["fp32c"], (name, split)
        c.close()


def test_autotuner_reports_a_variant(gpu_ctx):
    c = DeviceCloud.from_cloud(gpu_ctx, W.disk_cloud(4096, 4e-3, 2))
    name, split = c.autotune("fp32c")
    assert name.startswith("fp32c<") and split >= 1
    name64, split64 = c.autotune("fp64")
    assert name64.startswith("fp64<") and split64 >= 1


@pytest.fixture(scope="module")
def square256k_forces(gpu_ctx):
    """FP64 and FP32C shielded-Coulomb forces of the N=262144 cloud (0.1 m
    square, charges normal(-1.6e-15, 5%), kappa = 5e4), in caller order.  The
    pair force alone: the 1e8 V/m^2 walls are ~1e4 times stronger and would
    hide it in a total-force comparison."""
    c0 = W.square256k().clouds[0]
    out = {}
    for prec in ("fp64", "fp32c"):
        c = coulomb_cloud(gpu_ctx, c0.x, c0.y, c0.q, c0.shielding)
        out[prec] = c.eval_forces(prec)
        c.close()
    return c0, out


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_square256k_rows_vs_oracle(square256k_forces, oracle_lib, prec):
    """Full size: 1024 seeded rows against the oracle's row-wise restatement
    (same pair values as the reference; only the summation order differs)."""
    c0, out = square256k_forces
    rows = np.sort(np.random.default_rng(11).choice(c0.n, 1024, replace=False))
    p = oracle.make_params(flags=W.SHIELDED_COULOMB, shielding=c0.shielding)
    rx, ry = oracle_lib.forces_rows(c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, p, rows, nthreads=os.cpu_count())
    fx, fy = out[prec]
    err = e_F(fx[rows], fy[rows], rx, ry)
    print(f"square256k {prec} e_F(1024 rows) = {err:.3e}")
    assert err <= TOL[prec]


def test_square256k_fp32c_vs_fp64_all_rows(square256k_forces):
    """Full size, every row: the FP32C forces against the FP64 kernel's."""
    _, out = square256k_forces
    (fx, fy), (rx, ry) = out["fp32c"], out["fp64"]
    err = e_F(fx, fy, rx, ry)
    print(f"square256k fp32c vs fp64 e_F = {err:.3e}")
    assert err <= TOL["fp32c"]


def test_square256k_step_fp32c_tracks_fp64(gpu_ctx):
    """Two RK4 steps of dt = 5e-5 s at full size: FP32C displacements and
    velocities within 1e-5 of the FP64 ones (relative to their largest
    value).  The uniform random square holds pairs ~1e-7 m apart that are
    kicked by decimetres in a step, so errors are relative to the motion,
    not to the box."""
    c0 = W.square256k().clouds[0]
    res = {}
    for prec in ("fp64", "fp32c"):
        c = DeviceCloud.from_cloud(gpu_ctx, c0)
        c.step(2, 5e-5, prec)
        res[prec] = c.download()
        c.close()
    (x, y, vx, vy), (x64, y64, vx64, vy64) = res["fp32c"], res["fp64"]
    assert np.all(np.isfinite(x)) and np.all(np.isfinite(vx))
    disp = max(np.abs(x64 - c0.x).max(), np.abs(y64 - c0.y).max())
    err = max(np.abs(x - x64).max(), np.abs(y - y64).max())
    print(f"square256k 2 steps: max displacement {disp:.3e} m, fp32c-fp64 {err:.3e} m")
    assert err <= 1e-5 * disp
    vmax = max(np.abs(vx64).max(), np.abs(vy64).max())
    assert max(np.abs(vx - vx64).max(), np.abs(vy - vy64).max()) <= 1e-5 * vmax


@pytest.mark.parametrize("name", ["fp32c<8,4,256,false,cull>", "fp32c<8,4,256,true,cull>"])
def test_culled_variants_keep_every_pair_and_skip_far_groups(gpu_ctx, oracle_lib, name):
    """Box culling skips whole 32-particle j groups out of reach of an i
    tile; every pair inside the cutoff must still be counted (forces match
    the oracle) while most of a sparse cloud's pairs are never swept."""
    c0 = W.disk16k(thermal=False).clouds[0]
    c = coulomb_cloud(gpu_ctx, c0.x, c0.y, c0.q, 2e4)
    c.set_kernel(name, 0)
    e0 = c.evaluated_pairs()
    fx, fy = c.eval_forces("fp32c")
    swept = c.evaluated_pairs() - e0
    rx, ry = oracle_lib.shielded_coulomb(c0.x, c0.y, c0.q, 2e4, nthreads=8)
    err = e_F(fx, fy, rx, ry)
    print(f"{name}: e_F = {err:.3e}, swept {swept / c0.n**2:.4f} of all pairs")
    assert err <= TOL["fp32c"]
    assert 0 < swept < 0.1 * c0.n * c0.n


def test_culled_square256k_vs_fp64_all_rows(gpu_ctx, square256k_forces):
    c0, out = square256k_forces
    c = coulomb_cloud(gpu_ctx, c0.x, c0.y, c0.q, c0.shielding)
    c.set_kernel("fp32c<8,4,256,false,cull>", 0)
    fx, fy = c.eval_forces("fp32c")
    swept = c.evaluated_pairs()
    c.close()
    rx, ry = out["fp64"]
    err = e_F(fx, fy, rx, ry)
    print(f"square256k culled: e_F vs fp64 = {err:.3e}, swept {swept / c0.n**2:.2e} of all pairs")
    assert err <= TOL["fp32c"]
    assert swept < 0.01 * c0.n * c0.n
