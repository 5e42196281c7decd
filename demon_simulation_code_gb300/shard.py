"""Many clouds over several GPUs: one process per GPU, whole clouds per rank.

Clouds never interact, so the batched and trajectory-fit workloads shard
with no data-path exchange: each rank steps (or differentiates) its own
clouds and only small per-cloud results meet at the end.  Work per cloud is
~N^2 pair interactions, so clouds are dealt by longest-processing-time:
largest N^2 first, each to the rank with the least work so far (ties to the
lower rank) -- deterministic, so every rank computes the same assignment
without talking.

A single cloud does not shard here (this path runs one GPU per cloud:
replicas).  The reference has no multi-process mode.
"""
from __future__ import annotations

import numpy as np


def assign_clouds(ns, world: int) -> list[list[int]]:
    """Cloud indices per rank (each list ascending), balanced by sum N_c^2."""
    if world < 1:
        raise ValueError("world must be >= 1")
    load = [0] * world
    out = [[] for _ in range(world)]
    order = sorted(range(len(ns)), key=lambda c: (-int(ns[c]) ** 2, c))
    for c in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(c)
        load[r] += int(ns[c]) ** 2
    return [sorted(v) for v in out]


def imbalance(ns, parts) -> float:
    """max rank work / mean rank work (1.0 = perfect)."""
    w = [sum(int(ns[c]) ** 2 for c in p) for p in parts]
    return max(w) / (sum(w) / len(w)) if sum(w) else 1.0


def gather_per_cloud(values, ids, nclouds: int, width: int | None = None, group=None):
    """Per-cloud values computed on each rank (values[k] for cloud ids[k])
    -> the full array on every rank: [nclouds] when width is None, else
    [nclouds, width].  Every rank builds the same zero-filled shape from
    (nclouds, width), not from its own values, so a rank that owns no cloud
    (more ranks than clouds) still reduces a buffer of the same size; the
    buffers are summed with one all_reduce (each cloud belongs to exactly one
    rank)."""
    import torch
    import torch.distributed as dist

    shape = (nclouds,) if width is None else (nclouds, int(width))
    ids = np.asarray(ids, dtype=np.int64)
    values = np.asarray(values, dtype=np.float64).reshape((len(ids),) + shape[1:])
    full = np.zeros(shape, dtype=np.float64)
    full[ids] = values
    t = torch.from_numpy(full)
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()


def gather_segments(values, ids, ns, group=None):
    """Per-particle values of each rank's clouds (the concatenation of cloud
    ids[0]'s ns[ids[0]] values, then ids[1]'s, ...) -> the [sum(ns)] array of
    every cloud in cloud order, on every rank (one all_reduce of a buffer of
    that size; each cloud belongs to exactly one rank)."""
    import torch
    import torch.distributed as dist

    offs = np.concatenate([[0], np.cumsum(np.asarray(ns, dtype=np.int64))])
    full = np.zeros(int(offs[-1]), dtype=np.float64)
    values = np.asarray(values, dtype=np.float64).ravel()
    k = 0
    for c in ids:
        m = int(ns[c])
        full[offs[c]:offs[c] + m] = values[k:k + m]
        k += m
    if k != len(values):
        raise ValueError("values do not match the clouds' sizes")
    t = torch.from_numpy(full)
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()


def sum_scalar(value: float, group=None) -> float:
    """Sum of one float over the ranks (e.g. the trajectory-fit loss)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64)
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return float(t.item())
