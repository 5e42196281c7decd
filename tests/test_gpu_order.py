"""The device keeps every cloud in Morton order and re-sorts it (one
cluster launch for clouds of up to 16384 particles, a multi-kernel radix
sort above that, one block per cloud in a batch).  A re-sort must be a pure
permutation: with no forces enabled the RK4 update touches x and v only
through v itself, so the trajectory must equal the oracle's bit for bit
whatever order the device used, and uploads must round-trip exactly."""
import numpy as np
import pytest

import oracle
from demon_simulation_code_gb300 import DeviceBatch, DeviceCloud, workloads as W

pytestmark = pytest.mark.gpu

DT = 1e-4


def free_cloud(n, seed, radius=5e-3):
    """Random positions and velocities, no force enabled."""
    rng = np.random.default_rng(seed)
    x, y = W.uniform_disk(rng, n, radius)
    c = W.Cloud(x=x, y=y, vx=rng.normal(0.0, 1e-3, n), vy=rng.normal(0.0, 1e-3, n),
                q=np.full(n, W.Q_DUST), m=np.full(n, W.M_DUST), flags=0)
    return c


# sizes on both sides of the one-launch sort's limit and of its block slices
@pytest.mark.parametrize("n", [1, 2, 31, 33, 700, 2047, 2049, 16383, 16384, 16385])
def test_resort_every_step_is_a_permutation(gpu_ctx, oracle_lib, n):
    c0 = free_cloud(n, 100 + n)
    c = DeviceCloud.from_cloud(gpu_ctx, c0)
    c.set_reorder_interval(1)
    c.step(3, DT, "fp64")
    got = c.download()
    p = oracle.make_params(**c0.params())
    ref = oracle_lib.rk4_fixed(c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, p, DT, 3)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    c.close()


def test_upload_download_round_trip_keeps_the_internal_order(gpu_ctx):
    c0 = W.disk_cloud(5000, 2e-2, 7)
    c = DeviceCloud.from_cloud(gpu_ctx, c0)
    c.step(2, DT, "fp32c")  # now in Morton order
    rng = np.random.default_rng(8)
    new = [rng.normal(size=5000) for _ in range(4)]
    c.upload(*new)
    got = c.download()
    for a, b in zip(got, new):
        assert np.array_equal(a, b)
    out = [np.empty(5000) for _ in range(4)]
    back = c.download(out=out)
    assert all(a is b for a, b in zip(back, out))
    for a, b in zip(out, new):
        assert np.array_equal(a, b)
    with pytest.raises(ValueError):
        c.download(out=[np.empty(4999)] * 4)
    c.close()


def test_batch_per_cloud_sort_is_a_permutation(gpu_ctx, oracle_lib):
    ns = [1, 33, 64, 1000, 4095, 4096, 257]
    clouds = [free_cloud(n, 300 + n) for n in ns]
    b = DeviceBatch(gpu_ctx, clouds)
    b.step(3, DT)
    parts = [b.split(a) for a in b.download()]  # [component][cloud]
    for k, c0 in enumerate(clouds):
        g = [parts[comp][k] for comp in range(4)]
        p = oracle.make_params(**c0.params())
        ref = oracle_lib.rk4_fixed(c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, p, DT, 3)
        for a, r in zip(g, ref):
            assert np.array_equal(a, r)
    b.close()


@pytest.mark.parametrize("n", [1, 2049, 16384])
def test_eight_block_cluster_sort_is_a_permutation(monkeypatch, oracle_lib, n):
    """The portable 8-block cluster sort (DM_SORT_CLUSTER_CTAS=8, read by a
    context at its first re-sort) keeps the trajectory exact too."""
    from demon_simulation_code_gb300 import Context

    monkeypatch.setenv("DM_SORT_CLUSTER_CTAS", "8")
    ctx = Context(0)
    c0 = free_cloud(n, 500 + n)
    c = DeviceCloud.from_cloud(ctx, c0)
    c.step(3, DT, "fp64")
    got = c.download()
    p = oracle.make_params(**c0.params())
    ref = oracle_lib.rk4_fixed(c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, p, DT, 3)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    c.close()


def test_two_axis_finish_gives_the_per_particle_finish_bits(gpu_ctx):
    """Clouds with only the axis-separable forces complete each stage with
    one thread per particle and axis; adding a zero gravitational force
    routes the same arithmetic through the one-thread-per-particle finish.
    The two must agree bit for bit."""
    base = W.disk16k().clouds[0]
    runs = []
    for extra_flags in (0, W.GRAVITATIONAL):
        c0 = base.copy()
        c0.flags = base.flags | extra_flags
        c0.extra = dict(base.extra, gravity=0.0)
        c = DeviceCloud.from_cloud(gpu_ctx, c0)
        c.set_kernel("fp32c<4,2,128,false,cull>", 16)
        c.step(3, 1e-4, "fp32c")
        runs.append(c.download())
        c.close()
    for a, b in zip(*runs):
        assert np.array_equal(a, b)


def test_page_locked_buffers_are_copied_by_the_device_with_the_same_bits(gpu_ctx):
    """Page-locked caller buffers are read and written by a copy kernel (one
    launch per direction, no DMA copies); the state and trajectory must be
    the same bits as through pageable buffers."""
    torch = pytest.importorskip("torch")
    n = 5000
    c0 = W.disk_cloud(n, 2e-2, 7)
    rng = np.random.default_rng(9)
    new = [rng.normal(0.0, 1e-2 if k < 2 else 1e-3, size=n) for k in range(4)]
    pinned = [torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for _ in range(4)]
    out = [torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for _ in range(4)]
    for p, v in zip(pinned, new):
        p[:] = v
    a = DeviceCloud.from_cloud(gpu_ctx, c0)
    b = DeviceCloud.from_cloud(gpu_ctx, c0)
    a.step(2, DT, "fp32c")
    b.step(2, DT, "fp32c")
    l0 = gpu_ctx.launch_count()
    a.upload(*pinned)
    assert gpu_ctx.launch_count() - l0 == 2  # the copy kernel and the reorder into internal order
    b.upload(*new)
    back = a.download(out=out)
    for x, y in zip(back, new):
        assert np.array_equal(x, y)
    a.step(3, DT, "fp32c")
    b.step(3, DT, "fp32c")
    l0 = gpu_ctx.launch_count()
    ga = a.download(out=out)
    assert gpu_ctx.launch_count() - l0 == 2  # the scatter to caller order and the copy kernel
    gb = b.download()
    for x, y in zip(ga, gb):
        assert np.array_equal(x, y)
    a.close()
    b.close()
