"""Differentiable RK4 rollout: a hand-written discrete adjoint behind
``torch.autograd.Function``.

The O(N^2) work -- forces and their vector-Jacobian product -- runs in the
CUDA kernels of libdemon_gb300.so (FP64, or FP32 pair terms with Kahan sums) (``dm_adjoint_forces`` /
``dm_adjoint_vjp`` on the tensors' device memory); the O(N) RK4 stage
bookkeeping is FP64 tensor arithmetic on the same stream.  The forward pass
keeps the state every ``checkpoint_every`` steps; the backward pass
recomputes each segment from its checkpoint and walks it in reverse.

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
        return torch.zeros(self.nclouds, dtype=v.dtype, device=v.device).index_add_(0, self.seg, v)


def _f(K, s, q, m):
    x, y, vx, vy = s
    fx, fy = K.forces(x, y, vx, vy, q, m)
    return (vx, vy, fx / m, fy / m)


def _axpy(s, k, a):
    return tuple(si + a * ki for si, ki in zip(s, k))


def rk4_step(K, s, q, m, dt, stages=False):
    k1 = tuple(dt * v for v in _f(K, s, q, m))
    s2 = _axpy(s, k1, 0.5)
    k2 = tuple(dt * v for v in _f(K, s2, q, m))
    s3 = _axpy(s, k2, 0.5)
    k3 = tuple(dt * v for v in _f(K, s3, q, m))
    s4 = _axpy(s, k3, 1.0)
    k4 = tuple(dt * v for v in _f(K, s4, q, m))
    out = tuple(si + (a + ((b + c) * 2.0 + d)) / 6.0 for si, a, b, c, d in zip(s, k1, k2, k3, k4))
    return (out, (s, s2, s3, s4)) if stages else out


def _vjp_f(K, s, q, m, w):
    """J(s)^T w and the parameter gradients for f(s) = (vx, vy, F/m)."""
    x, y, vx, vy = s
    ax, ay = w[2] / m, w[3] / m
    gx, gy, gvx, gvy, gq, gk, gc = K.vjp(x, y, vx, vy, q, m, ax.contiguous(), ay.contiguous())
    return (gx, gy, w[0] + gvx, w[1] + gvy), gq, gk, gc


def rk4_step_vjp(K, s, q, m, dt, lam):
    _, (s1, s2, s3, s4) = rk4_step(K, s, q, m, dt, stages=True)
    gq = torch.zeros_like(q)
    gk = torch.zeros_like(q)
    gc = torch.zeros_like(q)
    sixth = [v / 6.0 for v in lam]
    third = [v / 3.0 for v in lam]

    def stage(si, dk):
        mu, a, b, c = _vjp_f(K, si, q, m, [dt * v for v in dk])
        return mu, a, b, c

    mu4, a, b, c = stage(s4, sixth)
    gq += a; gk += b; gc += c
    dk3 = [t + u for t, u in zip(third, mu4)]
    mu3, a, b, c = stage(s3, dk3)
    gq += a; gk += b; gc += c
    dk2 = [t + 0.5 * u for t, u in zip(third, mu3)]
    mu2, a, b, c = stage(s2, dk2)
    gq += a; gk += b; gc += c
    dk1 = [t + 0.5 * u for t, u in zip(sixth, mu2)]
    mu1, a, b, c = stage(s1, dk1)
    gq += a; gk += b; gc += c
    lam_prev = tuple(l + u1 + u2 + u3 + u4 for l, u1, u2, u3, u4 in zip(lam, mu1, mu2, mu3, mu4))
    return lam_prev, gq, gk, gc


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
        s = tuple(t.detach().contiguous() for t in (x0, y0, vx0, vy0))
        ckpts = []
        for t in range(nsteps):
            if t % every == 0:
                ckpts.append(s)
            s = rk4_step(K, s, q, m, dt)
        ctx.meta = meta
        ctx.ckpts = ckpts
        ctx.save_for_backward(kappa, qc, kc)
        return tuple(v.clone() for v in s)

    @staticmethod
    def backward(ctx, gx, gy, gvx, gvy):
        kappa, qc, kc = ctx.saved_tensors
        meta = ctx.meta
        K, m, dt, nsteps, every = meta["kernels"], meta["m"], meta["dt"], meta["steps"], meta["every"]
        K.set_params(kappa.detach().cpu().numpy(), kc.detach().cpu().numpy())
        q = qc.detach()[K.seg].contiguous()
        ref = ctx.ckpts[0][0]
        lam = tuple(g.contiguous() if g is not None else torch.zeros_like(ref) for g in (gx, gy, gvx, gvy))
        gq = torch.zeros_like(q)
        gk = torch.zeros_like(q)
        gc = torch.zeros_like(q)
        for ci in range(len(ctx.ckpts) - 1, -1, -1):
            t0 = ci * every
            t1 = min(nsteps, t0 + every)
            states = [ctx.ckpts[ci]]
            for _ in range(t0, t1 - 1):  # recompute the segment
                states.append(rk4_step(K, states[-1], q, m, dt))
            for s in reversed(states):
                lam, a, b, c = rk4_step_vjp(K, s, q, m, dt, lam)
                gq += a
                gk += b
                gc += c
        return (lam[0], lam[1], lam[2], lam[3], K.per_cloud(gk), K.per_cloud(gq), K.per_cloud(gc), None)


def rollout(K, x0, y0, vx0, vy0, kappa, qc, kc, m, dt, steps, checkpoint_every=20):
    meta = {"kernels": K, "m": m, "dt": float(dt), "steps": int(steps), "every": int(checkpoint_every)}
    return Rollout.apply(x0, y0, vx0, vy0, kappa, qc, kc, meta)
