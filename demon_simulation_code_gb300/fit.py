"""Trajectory fit over many clouds: the differentiable-rollout workload.

Each cloud c has its own shielding kappa_c, grain charge q_c and confinement
constant k_c.  Targets are FP64 rollouts from the true parameters; the fit
starts from parameters perturbed by a seeded uniform factor and the loss is
the mean squared final-position error over all particles,

    L = (1 / N_total) sum_c sum_{i in c} |x_i(T) - x*_i(T)|^2 = sum_c L_c.

Gradients with respect to (kappa, q, k_c) per cloud and to the initial
positions come from the adjoint rollout (adjoint.py).  Because the clouds do
not interact, L_c depends only on cloud c's parameters, so one pair of
perturbed rollouts gives a central finite difference for every cloud at once
(``finite_difference``).
"""
from __future__ import annotations

import numpy as np
import torch

from .adjoint import AdjointKernels, rollout


def start_factors(nclouds: int, perturb: float, seed: int) -> np.ndarray:
    """[nclouds, 3] seeded factors of (kappa, q, k_c) for the fit's start:
    row c is cloud c's, so the first k clouds of a workload start where they
    would in a k-cloud workload, and a shard of clouds starts where those
    clouds do in the whole workload."""
    rng = np.random.default_rng(seed)
    return 1.0 + rng.uniform(-perturb, perturb, (nclouds, 3))


class TrajectoryFit:
    """The fit over `workload`'s clouds, or over the clouds `cloud_ids` of it
    (a shard: start factors as in the whole workload, losses divided by
    `norm` particles, by default this fit's own particle count)."""

    def __init__(self, workload, perturb: float | None = None, seed: int = 4, device=None,
                 precision: str = "fp64", cloud_ids=None, norm: int | None = None, keep_stages="auto"):
        ids = list(range(len(workload.clouds))) if cloud_ids is None else [int(i) for i in cloud_ids]
        clouds = [workload.clouds[i] for i in ids]
        self.cloud_ids = ids
        self.ns = [c.n for c in clouds]
        self.norm = sum(self.ns) if norm is None else int(norm)
        self.dt = float(workload.dt)
        self.steps = int(workload.steps)
        self.every = int(workload.extra.get("checkpoint_every", 20))
        self.keep_stages = keep_stages
        perturb = float(workload.extra.get("perturb", 0.2) if perturb is None else perturb)
        dev = torch.device("cuda", torch.cuda.current_device() if device is None else int(device))

        def cat(attr):
            return torch.tensor(np.concatenate([getattr(c, attr) for c in clouds]), dtype=torch.float64,
                                device=dev)

        self.x0, self.y0, self.vx0, self.vy0, self.m = (cat(a) for a in ("x", "y", "vx", "vy", "m"))
        self.true = {
            "kappa": torch.tensor([c.shielding for c in clouds], dtype=torch.float64, device=dev),
            "q": torch.tensor([float(c.q[0]) for c in clouds], dtype=torch.float64, device=dev),
            "kc": torch.tensor([c.confine for c in clouds], dtype=torch.float64, device=dev),
        }
        gammas = {c.gamma for c in clouds}
        assert len(gammas) == 1, "one drag constant for all clouds"
        flags, gamma = clouds[0].flags, gammas.pop()
        # targets are FP64 rollouts whatever the precision of the fit
        K64 = AdjointKernels(self.ns, flags=flags, gamma=gamma, device=dev.index)
        self.K = K64 if precision == "fp64" else AdjointKernels(self.ns, flags=flags, gamma=gamma,
                                                                device=dev.index, precision=precision)
        with torch.no_grad():
            xT, yT, _, _ = self._rollout(self.x0, self.true["kappa"], self.true["q"], self.true["kc"], K64)
        self.xt, self.yt = xT, yT
        self.K64 = K64
        # row c = cloud c's factors for (kappa, q, k_c): the first k clouds of
        # a workload start where they would in a k-cloud workload
        f = torch.tensor(start_factors(len(workload.clouds), perturb, seed)[ids], dtype=torch.float64,
                         device=dev)
        self.start = {k: self.true[k] * f[:, col] for col, k in enumerate(("kappa", "q", "kc"))}

    @property
    def total(self) -> int:
        return sum(self.ns)

    @property
    def pairs_per_eval(self) -> int:
        return sum(n * (n - 1) for n in self.ns)

    def _rollout(self, x0, kappa, q, kc, K=None):
        return rollout(self.K if K is None else K, x0, self.y0, self.vx0, self.vy0, kappa, q, kc, self.m,
                       self.dt, self.steps, self.every, self.keep_stages)

    def per_cloud_loss(self, kappa, q, kc, x0=None, K=None):
        """[nclouds] tensor of L_c (their sum is the loss)."""
        xT, yT, _, _ = self._rollout(self.x0 if x0 is None else x0, kappa, q, kc, K)
        e = (xT - self.xt) ** 2 + (yT - self.yt) ** 2
        return self.K.per_cloud(e) / self.norm

    def loss(self, kappa, q, kc, x0=None):
        return self.per_cloud_loss(kappa, q, kc, x0).sum()

    def loss_and_grad(self, params=None):
        """Loss at ``params`` (default: the perturbed start) and its adjoint
        gradients {"kappa", "q", "kc", "x0"}."""
        p = self.start if params is None else params
        leaves = {k: p[k].detach().clone().requires_grad_(True) for k in ("kappa", "q", "kc")}
        x0 = self.x0.detach().clone().requires_grad_(True)
        L = self.loss(leaves["kappa"], leaves["q"], leaves["kc"], x0)
        L.backward()
        grads = {k: v.grad for k, v in leaves.items()}
        grads["x0"] = x0.grad
        return L.detach(), grads

    @torch.no_grad()
    def finite_difference(self, name, params=None, rel_step=1e-6, particles=None):
        """Central differences of L with a relative step: for a parameter name,
        one value per cloud; for "x0", one per cloud at the given within-cloud
        particle indices (one per cloud), all from two rollouts.  The
        rollouts are FP64 whatever the fit's precision (FP32 rounding noise
        would swamp a 1e-6 step)."""
        K = self.K64
        p = dict(self.start if params is None else params)
        if name == "x0":
            offs = np.cumsum([0] + self.ns[:-1])
            idx = torch.tensor(offs + np.asarray(particles), device=self.x0.device)
            h = rel_step * torch.clamp(self.x0[idx].abs(), min=1e-12)
            up = self.x0.clone()
            dn = self.x0.clone()
            up[idx] += h
            dn[idx] -= h
            Lu = self.per_cloud_loss(p["kappa"], p["q"], p["kc"], up, K)
            Ld = self.per_cloud_loss(p["kappa"], p["q"], p["kc"], dn, K)
            return (Lu - Ld) / (2 * h), idx
        base = p[name]
        h = rel_step * base.abs()
        Lu = self.per_cloud_loss(**{**p, name: base + h}, K=K)
        Ld = self.per_cloud_loss(**{**p, name: base - h}, K=K)
        return (Lu - Ld) / (2 * h)


class ShardedTrajectoryFit:
    """The trajectory fit over the ranks of a torch.distributed group: whole
    clouds per rank (shard.assign_clouds, balanced by N^2), each rank
    differentiates its own clouds, and the results meet in one all-reduce
    each -- the loss (a sum over clouds), the per-cloud (kappa, q, k_c)
    gradients and the initial-position gradient (a segment per cloud).  No
    data-path exchange: clouds never interact.  Every rank returns the full
    results.

    make_local(ids, norm) builds the fit of a shard (default: TrajectoryFit
    on this rank's GPU); a rank that owns no cloud builds none."""

    def __init__(self, workload, group=None, make_local=None, **kw):
        import torch.distributed as dist

        from .shard import assign_clouds

        self.group = group
        self.world = dist.get_world_size(group)
        self.rank = dist.get_rank(group)
        self.ns_all = [c.n for c in workload.clouds]
        self.ids = assign_clouds(self.ns_all, self.world)[self.rank]
        norm = sum(self.ns_all)
        if make_local is None:
            def make_local(ids, norm):
                return TrajectoryFit(workload, cloud_ids=ids, norm=norm, **kw)
        self.local = make_local(self.ids, norm) if self.ids else None

    def loss_and_grad(self):
        """(loss, {"kappa", "q", "kc": [nclouds], "x0": [N_total]}) as numpy,
        identical on every rank."""
        from .shard import gather_per_cloud, gather_segments, sum_scalar

        if self.local is not None:
            L, g = self.local.loss_and_grad()
            L = float(L)
            g = {k: np.asarray(v.detach().cpu().numpy() if hasattr(v, "detach") else v, dtype=np.float64)
                 for k, v in g.items()}
        else:
            L, g = 0.0, {k: np.zeros(0) for k in ("kappa", "q", "kc", "x0")}
        n = len(self.ns_all)
        out = {k: gather_per_cloud(g[k], self.ids, n, group=self.group) for k in ("kappa", "q", "kc")}
        out["x0"] = gather_segments(g["x0"], self.ids, self.ns_all, group=self.group)
        return sum_scalar(L, group=self.group), out
