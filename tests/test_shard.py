"""Cloud sharding over ranks (CPU, gloo, world size 2): the assignment is
balanced and deterministic, and per-cloud results computed on each rank's
shard -- here the oracle's FP64 diagnostics of every cloud -- gather to
exactly the single-process result."""
import os
import socket

import numpy as np
import pytest

from demon_simulation_code_gb300 import workloads as W
from demon_simulation_code_gb300.shard import assign_clouds, imbalance

torch = pytest.importorskip("torch")


def test_assignment_covers_every_cloud_once_and_balances():
    ns = W.batch256().clouds
    ns = [c.n for c in ns]
    for world in (1, 2, 3, 4, 8):
        parts = assign_clouds(ns, world)
        flat = sorted(c for p in parts for c in p)
        assert flat == list(range(len(ns)))
        assert imbalance(ns, parts) < 1.01
        assert parts == assign_clouds(ns, world)  # deterministic


def test_assignment_edge_cases():
    assert assign_clouds([], 2) == [[], []]
    assert assign_clouds([5], 3) == [[0], [], []]
    assert assign_clouds([10, 10, 1], 2) == [[0, 2], [1]]
    with pytest.raises(ValueError):
        assign_clouds([1], 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir, nclouds=12):
    import torch.distributed as dist

    import oracle
    from demon_simulation_code_gb300.shard import gather_per_cloud, sum_scalar

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        clouds = W.batch256(nclouds=nclouds, nmin=16, nmax=128).clouds
        ids = assign_clouds([c.n for c in clouds], world)[rank]
        o = oracle.Oracle()
        vals = []
        for c in ids:
            cl = clouds[c]
            d = o.diagnostics(cl.x, cl.y, cl.vx, cl.vy, cl.q, cl.m, oracle.make_params(**cl.params()))
            vals.append(d)
        full = gather_per_cloud(np.array(vals).reshape(len(ids), 5), ids, len(clouds), width=5)
        total = sum_scalar(float(sum(v[1] for v in vals)))
        np.save(os.path.join(out_dir, f"r{rank}.npy"), np.concatenate([full.ravel(), [total]]))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_gather_per_cloud_results(tmp_path):
    import torch.multiprocessing as mp

    import oracle

    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    r0, r1 = np.load(tmp_path / "r0.npy"), np.load(tmp_path / "r1.npy")
    assert np.array_equal(r0, r1)
    clouds = W.batch256(nclouds=12, nmin=16, nmax=128).clouds
    o = oracle.Oracle()
    ref = np.array([o.diagnostics(c.x, c.y, c.vx, c.vy, c.q, c.m, oracle.make_params(**c.params()))
                    for c in clouds])
    assert np.array_equal(r0[:-1].reshape(12, 5), ref)
    assert abs(r0[-1] - ref[:, 1].sum()) <= 1e-12 * abs(ref[:, 1].sum())


def test_gloo_more_ranks_than_clouds(tmp_path):
    """Three ranks, two clouds: the rank that owns no cloud reduces a buffer
    of the same shape as the others, and all three get the full result."""
    import torch.multiprocessing as mp

    import oracle

    mp.spawn(_worker, args=(3, _free_port(), str(tmp_path), 2), nprocs=3, join=True)
    outs = [np.load(tmp_path / f"r{r}.npy") for r in range(3)]
    assert all(np.array_equal(outs[0], o) for o in outs[1:])
    clouds = W.batch256(nclouds=2, nmin=16, nmax=128).clouds
    assert [len(p) for p in assign_clouds([c.n for c in clouds], 3)].count(0) == 1
    o = oracle.Oracle()
    ref = np.array([o.diagnostics(c.x, c.y, c.vx, c.vy, c.q, c.m, oracle.make_params(**c.params()))
                    for c in clouds])
    assert np.array_equal(outs[0][:-1].reshape(2, 5), ref)


class _CpuFit:
    """A CPU stand-in for the device part of a shard's trajectory fit (same
    interface as fit.TrajectoryFit.loss_and_grad): deterministic per-cloud
    values computed from the clouds, so the sharded result can be checked
    exactly against one process."""

    def __init__(self, workload, ids, norm):
        self.clouds = [workload.clouds[i] for i in ids]
        self.ids = list(ids)
        self.norm = norm

    def loss_and_grad(self):
        L = sum(float(np.sum(c.x ** 2 + c.y ** 2)) for c in self.clouds) / self.norm
        g = {"kappa": np.array([float(np.sum(c.x)) * c.shielding for c in self.clouds]),
             "q": np.array([float(c.n) + i for c, i in zip(self.clouds, self.ids)]),
             "kc": np.array([c.confine for c in self.clouds]),
             "x0": np.concatenate([2.0 * c.x / self.norm for c in self.clouds])}
        return L, g


def _fit_worker(rank, world, port, out_dir, nclouds):
    import torch.distributed as dist

    from demon_simulation_code_gb300.fit import ShardedTrajectoryFit

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = W.batch256(nclouds=nclouds, nmin=16, nmax=128)
        fit = ShardedTrajectoryFit(w, make_local=lambda ids, norm: _CpuFit(w, ids, norm))
        L, g = fit.loss_and_grad()
        np.save(os.path.join(out_dir, f"fit{rank}.npy"),
                np.concatenate([[L], g["kappa"], g["q"], g["kc"], g["x0"]]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,nclouds", [(2, 12), (3, 2)])
def test_gloo_sharded_trajectory_fit_equals_one_process(tmp_path, world, nclouds):
    """The trajectory fit's sharding logic end to end on CPU ranks (gloo):
    clouds dealt by assign_clouds, the shard fits built with the whole
    workload's particle count, the loss summed and the per-cloud and
    per-particle gradients gathered -- equal to one process over all clouds,
    also with a rank that owns no cloud."""
    import torch.multiprocessing as mp

    mp.spawn(_fit_worker, args=(world, _free_port(), str(tmp_path), nclouds), nprocs=world, join=True)
    outs = [np.load(tmp_path / f"fit{r}.npy") for r in range(world)]
    assert all(np.array_equal(outs[0], o) for o in outs[1:])
    w = W.batch256(nclouds=nclouds, nmin=16, nmax=128)
    norm = sum(c.n for c in w.clouds)
    L, g = _CpuFit(w, range(nclouds), norm).loss_and_grad()
    ref = np.concatenate([[L], g["kappa"], g["q"], g["kc"], g["x0"]])
    assert abs(outs[0][0] - ref[0]) <= 1e-14 * abs(ref[0])
    assert np.array_equal(outs[0][1:], ref[1:])
