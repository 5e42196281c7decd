"""Differentiable RK4 rollout: a hand-written discrete adjoint behind
``torch.autograd.Function``.

All O(N^2) work and the RK4 bookkeeping run in the CUDA kernels of
libdemon_gb300.so on the tensors' device memory: one fused launch per RK4
stage forward (pair force, per-particle forces and stage algebra,
``dm_adjoint_rk4_step``) and one per stage backward (force VJP and the
adjoint recurrences, ``dm_adjoint_rk4_step_vjp``), FP64 or FP32 pair terms
with Kahan sums.  When gradients are wanted, the forward pass keeps the four
stage inputs of every step (16 doubles per particle and step: 3.4 GB for
64 x 2048 particles over 200 steps) as long as they fit the memory budget
(``keep_stages``), and the backward pass walks the steps in reverse from
them: four force sweeps per step forward, four VJP sweeps back.  Otherwise
the forward pass keeps the state every ``checkpoint_every`` steps and the
backward pass recomputes each segment from its checkpoint, keeping the
segment's stage inputs -- four more force sweeps per step.  Both give the
same bits (the forward step is deterministic).

RK4 step (the reference's Runge_Kutta4.cpp:23-137, written for s = (x, y,
vx, vy) and f(s) = (vx, vy, Fx/m, Fy/m)):
    k1 = dt f(s), k2 = dt f(s + k1/2), k3 = dt f(s + k2/2), k4 = dt f(s + k3)
    s' = s + (k1 + 2 (k2 + k3) + k4) / 6
Adjoint of one step, given lam = dL/ds':
    dk4 = lam/6,                 mu4 = J(s4)^T dt dk4
    dk3 = lam/3 + mu4,           mu3 = J(s3)^T dt dk3
    dk2 = lam/3 + mu3/2,         mu2 = J(s2)^T dt dk2
    dk1 = lam/6 + mu2/2,         mu1 = J(s1)^T dt dk1
    dL/ds = lam + mu1 + mu2 + mu3 + mu4,  dL/dtheta += sum_i (df/dtheta)(s_i)^T dt dk_i
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import check
from .workloads import CONFINEMENT, DRAG, SHIELDED_COULOMB


def _p(t: torch.Tensor) -> int:
    assert t.dtype == torch.float64 and t.is_cuda and t.is_contiguous()
    return t.data_ptr()


class AdjointKernels:
    """dm_adjoint for a fixed list of cloud sizes (concatenated clouds), in
    "fp64" or "fp32c" pair arithmetic.

    Owns a context whose work is queued on torch's current CUDA stream at
    each call, so the kernels and the surrounding tensor arithmetic are
    ordered on one stream."""

    def __init__(self, ns, flags=CONFINEMENT | DRAG | SHIELDED_COULOMB, gamma=3.0, device=None,
                 precision="fp64"):
        from .cloud import Context

        self.precision = {"fp64": 0, "fp32c": 1}[precision]

        ctx = Context(torch.cuda.current_device() if device is None else int(device))
        self.ctx = ctx
        self.lib = ctx.lib
        self.ns = [int(v) for v in ns]
        self.nclouds = len(self.ns)
        self.total = sum(self.ns)
        self.flags = int(flags)
        self.gamma = float(gamma)
        self._params = (_lib.ForceParams * self.nclouds)()
        nn = (ctypes.c_int * self.nclouds)(*self.ns)
        self._fill(np.full(self.nclouds, 2e4), np.full(self.nclouds, 1e8))
        h = ctypes.c_void_p()
        check(self.lib.dm_adjoint_create(ctx.h, self.nclouds, nn, self._params, ctypes.byref(h)), ctx.h)
        self.h = h
        self.seg = torch.repeat_interleave(torch.arange(self.nclouds, device="cuda"),
                                           torch.tensor(self.ns, device="cuda"))

    def _fill(self, kappa, kc):
        for c in range(self.nclouds):
            self._params[c] = _lib.force_params(self.flags, shielding=float(kappa[c]),
                                                confine=float(kc[c]), gamma=self.gamma)

    def set_params(self, kappa, kc):
        self._bind_stream()
        self._fill(np.asarray(kappa, dtype=np.float64), np.asarray(kc, dtype=np.float64))
        check(self.lib.dm_adjoint_set_params(self.h, self._params), self.ctx.h)

    def close(self):
        if self.h:
            self.lib.dm_adjoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _bind_stream(self):
        self.ctx.set_stream(torch.cuda.current_stream().cuda_stream)

    def forces(self, x, y, vx, vy, q, m, pair=False):
        self._bind_stream()
        fx = torch.empty_like(x)
        fy = torch.empty_like(x)
        fpx = torch.empty_like(x) if pair else None
        fpy = torch.empty_like(x) if pair else None
        check(self.lib.dm_adjoint_forces(self.h, self.precision, _p(x), _p(y), _p(vx), _p(vy), _p(q), _p(m),
                                         _p(fx), _p(fy), _p(fpx) if pair else None,
                                         _p(fpy) if pair else None), self.ctx.h)
        return (fx, fy, fpx, fpy) if pair else (fx, fy)

    def vjp(self, x, y, vx, vy, q, m, ax, ay):
        self._bind_stream()
        out = [torch.empty_like(x) for _ in range(7)]
        check(self.lib.dm_adjoint_vjp(self.h, self.precision, _p(x), _p(y), _p(vx), _p(vy), _p(q), _p(m), _p(ax), _p(ay),
                                      *(_p(o) for o in out)), self.ctx.h)
        return out  # gx, gy, gvx, gvy, gq_i, gkappa_i, gkc_i

    def per_cloud(self, v):
        """Per-cloud sums of a per-particle tensor, in a fixed order (an
        atomic scatter-add would round differently from call to call)."""
        if len(set(self.ns)) == 1:
            return v.view(self.nclouds, self.ns[0]).sum(dim=1)
        return torch.stack([seg.sum() for seg in torch.split(v, self.ns)])

    def rk4_step(self, s, q, m, dt, stages=None):
        """One fused RK4 step of the state s = (x, y, vx, vy), in place;
        stages: None or a [16, total] FP64 tensor that receives the four
        stage inputs."""
        self._bind_stream()
        check(self.lib.dm_adjoint_rk4_step(self.h, self.precision, float(dt), *(_p(t) for t in s), _p(q), _p(m),
                                           _p(stages) if stages is not None else None), self.ctx.h)

    def rk4_step_vjp(self, stages, q, m, dt, lam, gq, gk, gc):
        """The adjoint of one step from its stage inputs: lam (4 tensors)
        from dL/d(output) to dL/d(input) in place; the parameter gradients
        per particle added to gq, gk (kappa), gc (k_c)."""
        self._bind_stream()
        check(self.lib.dm_adjoint_rk4_step_vjp(self.h, self.precision, float(dt), _p(stages), _p(q), _p(m),
                                               *(_p(t) for t in lam), _p(gq), _p(gk), _p(gc)), self.ctx.h)


class Rollout(torch.autograd.Function):
    """(x0, y0, vx0, vy0, kappa[c], q[c], k_c[c]) -> (x_T, y_T, vx_T, vy_T).

    kappa, q and k_c are per-cloud tensors; every particle of cloud c has
    charge q[c].  Masses, drag, dt, the step count and the checkpoint
    spacing are fixed (``meta``)."""

    @staticmethod
    def forward(ctx, x0, y0, vx0, vy0, kappa, qc, kc, meta):
        K, m, dt, nsteps, every = meta["kernels"], meta["m"], meta["dt"], meta["steps"], meta["every"]
        K.set_params(kappa.detach().cpu().numpy(), kc.detach().cpu().numpy())
        q = qc.detach()[K.seg].contiguous()
        s = tuple(t.detach().clone().contiguous() for t in (x0, y0, vx0, vy0))
        ckpts, store = [], None
        if any(ctx.needs_input_grad) and _keep_all_stages(meta["keep"], nsteps, s[0]):
            store = torch.empty((nsteps, 16, s[0].numel()), dtype=torch.float64, device=s[0].device)
            ckpts.append(tuple(v.clone() for v in s))
            for t in range(nsteps):
                K.rk4_step(s, q, m, dt, stages=store[t])
        else:
            for t in range(nsteps):
                if t % every == 0:
                    ckpts.append(tuple(v.clone() for v in s))
                K.rk4_step(s, q, m, dt)
        K.kept_stages = store is not None  # how the last differentiable rollout ran
        ctx.meta = meta
        ctx.ckpts = ckpts
        ctx.store = store
        ctx.save_for_backward(kappa, qc, kc)
        return s

    @staticmethod
    def backward(ctx, gx, gy, gvx, gvy):
        kappa, qc, kc = ctx.saved_tensors
        meta = ctx.meta
        K, m, dt, nsteps, every = meta["kernels"], meta["m"], meta["dt"], meta["steps"], meta["every"]
        K.set_params(kappa.detach().cpu().numpy(), kc.detach().cpu().numpy())
        q = qc.detach()[K.seg].contiguous()
        ref = ctx.ckpts[0][0]
        lam = tuple(g.clone().contiguous() if g is not None else torch.zeros_like(ref) for g in (gx, gy, gvx, gvy))
        gq = torch.zeros_like(q)
        gk = torch.zeros_like(q)
        gc = torch.zeros_like(q)
        if ctx.store is not None:  # every step's stage inputs kept by the forward pass
            for t in range(nsteps - 1, -1, -1):
                K.rk4_step_vjp(ctx.store[t], q, m, dt, lam, gq, gk, gc)
            ctx.store = None
            return (lam[0], lam[1], lam[2], lam[3], K.per_cloud(gk), K.per_cloud(gq), K.per_cloud(gc), None)
        store = torch.empty((min(every, nsteps), 16, ref.numel()), dtype=torch.float64, device=ref.device)
        for ci in range(len(ctx.ckpts) - 1, -1, -1):
            t0 = ci * every
            t1 = min(nsteps, t0 + every)
            s = tuple(v.clone() for v in ctx.ckpts[ci])
            for t in range(t0, t1):  # recompute the segment, keeping every stage input
                K.rk4_step(s, q, m, dt, stages=store[t - t0])
            for t in range(t1 - 1, t0 - 1, -1):
                K.rk4_step_vjp(store[t - t0], q, m, dt, lam, gq, gk, gc)
        return (lam[0], lam[1], lam[2], lam[3], K.per_cloud(gk), K.per_cloud(gq), K.per_cloud(gc), None)


# Default memory budget for kept stage inputs: this many bytes, and at most a
# quarter of the device memory free at the time.
STAGE_BUDGET_BYTES = 16 << 30


def stage_bytes(nsteps: int, total: int) -> int:
    """Bytes of every step's four stage inputs (x, y, vx, vy each)."""
    return int(nsteps) * 16 * int(total) * 8


def _keep_all_stages(keep, nsteps, like) -> bool:
    if keep is True or keep is False:
        return keep
    if keep != "auto":
        raise ValueError("keep_stages must be True, False or 'auto'")
    need = stage_bytes(nsteps, like.numel())
    free, _ = torch.cuda.mem_get_info(like.device)
    return need <= min(STAGE_BUDGET_BYTES, free // 4)


def rollout(K, x0, y0, vx0, vy0, kappa, qc, kc, m, dt, steps, checkpoint_every=20, keep_stages="auto"):
    """(x_T, y_T, vx_T, vy_T) after `steps` RK4 steps, differentiable with
    respect to the start state and the per-cloud (kappa, q, k_c).
    keep_stages: True keeps every step's stage inputs for the backward pass,
    False recomputes them from checkpoints every `checkpoint_every` steps,
    "auto" keeps them when they fit the memory budget.  Same gradients."""
    meta = {"kernels": K, "m": m, "dt": float(dt), "steps": int(steps), "every": int(checkpoint_every),
            "keep": keep_stages}
    return Rollout.apply(x0, y0, vx0, vy0, kappa, qc, kc, meta)
