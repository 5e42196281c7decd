"""Object API over the C ABI: a GPU context and a device-resident cloud.

Method names follow the reference's classes where one exists:
``eval_forces`` is the sum of ``Force::force1`` over the ForceArray
(Runge_Kutta2.cpp:90-93); ``move_particles`` is
``Runge_Kutta4::moveParticles`` (Runge_Kutta4.cpp:23-137); ``step`` is the
same for an explicit step count with a fixed dt.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import DM_FP32C, DM_FP64, addr, check, ptr

PRECISIONS = {"fp64": DM_FP64, "fp32c": DM_FP32C, DM_FP64: DM_FP64, DM_FP32C: DM_FP32C}


def _prec(p) -> int:
    try:
        return PRECISIONS[p]
    except KeyError:
        raise ValueError(f"unknown precision {p!r}") from None


class Context:
    """One GPU + one CUDA stream (dm_ctx)."""

    def __init__(self, device: int = 0):
        lib = _lib.load()
        h = ctypes.c_void_p()
        check(lib.dm_ctx_create(device, ctypes.byref(h)), None)
        self.lib = lib
        self.h = h

    def close(self):
        if self.h:
            self.lib.dm_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int | None):
        """Queue all later work on this cudaStream_t handle (0 = the default stream)."""
        check(self.lib.dm_ctx_set_stream(self.h, ctypes.c_void_p(stream_handle or 0)), self.h)

    def reset_stream(self):
        check(self.lib.dm_ctx_reset_stream(self.h), self.h)

    def synchronize(self):
        check(self.lib.dm_ctx_synchronize(self.h), self.h)

    def launch_count(self) -> int:
        v = ctypes.c_longlong()
        check(self.lib.dm_ctx_launch_count(self.h, ctypes.byref(v)), self.h)
        return v.value

    def profile(self, enable: bool):
        check(self.lib.dm_ctx_profile_enable(self.h, int(enable)), self.h)

    def profile_read(self):
        ms = ctypes.c_double()
        n = ctypes.c_longlong()
        pairs = ctypes.c_double()
        check(self.lib.dm_ctx_profile_read(self.h, ctypes.byref(ms), ctypes.byref(n),
                                           ctypes.byref(pairs)), self.h)
        return ms.value, n.value, pairs.value

    def set_autotune(self, enable: bool):
        check(self.lib.dm_ctx_set_autotune(self.h, int(enable)), self.h)

    def probe_peak(self, kind: str = "fp32") -> float:
        v = ctypes.c_double()
        check(self.lib.dm_probe_peak(self.h, 0 if kind == "fp32" else 1, ctypes.byref(v)), self.h)
        return v.value


class DeviceCloud:
    """A device-resident cloud (dm_cloud)."""

    def __init__(self, ctx: Context, x, y, vx, vy, q, m, params=None):
        self.ctx = ctx
        self.lib = ctx.lib
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, vx, vy, q, m)]
        n = len(arrs[0])
        if any(len(a) != n for a in arrs):
            raise ValueError("arrays differ in length")
        h = ctypes.c_void_p()
        check(self.lib.dm_cloud_create(ctx.h, n, *(ptr(a) for a in arrs), ctypes.byref(h)), ctx.h)
        self.h = h
        self.n = n
        if params is not None:
            self.set_forces(params)

    @classmethod
    def from_cloud(cls, ctx: Context, c) -> "DeviceCloud":
        """From a workloads.Cloud."""
        return cls(ctx, c.x, c.y, c.vx, c.vy, c.q, c.m, _lib.force_params(**c.params()))

    def close(self):
        if self.h:
            self.lib.dm_cloud_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        check(rc, self.ctx.h)

    def set_forces(self, params):
        if isinstance(params, dict):
            params = _lib.force_params(**params)
        self._chk(self.lib.dm_cloud_set_forces(self.h, ctypes.byref(params)))

    def upload(self, x, y, vx, vy):
        a = [np.ascontiguousarray(v, dtype=np.float64) for v in (x, y, vx, vy)]
        self._chk(self.lib.dm_cloud_upload(self.h, *(addr(v) for v in a)))

    def download(self, out=None):
        """x, y, vx, vy in the caller's order; `out`: four contiguous float64
        arrays of length n to fill (e.g. pinned host buffers) instead of new
        ones."""
        if out is None:
            out = [np.empty(self.n) for _ in range(4)]
        else:
            out = list(out)
            if len(out) != 4 or any(not (isinstance(v, np.ndarray) and v.dtype == np.float64 and
                                         v.flags.c_contiguous and v.size == self.n) for v in out):
                raise ValueError("download(out=...): four contiguous float64 arrays of length n")
        self._chk(self.lib.dm_cloud_download(self.h, *(addr(v) for v in out)))
        return tuple(out)

    def set_charge_mass(self, q=None, m=None):
        qa = None if q is None else np.ascontiguousarray(q, dtype=np.float64)
        ma = None if m is None else np.ascontiguousarray(m, dtype=np.float64)
        self._chk(self.lib.dm_cloud_set_charge_mass(self.h, None if qa is None else ptr(qa),
                                                    None if ma is None else ptr(ma)))

    def eval_forces(self, precision="fp64"):
        fx = np.empty(self.n)
        fy = np.empty(self.n)
        self._chk(self.lib.dm_cloud_eval_forces(self.h, _prec(precision), ptr(fx), ptr(fy)))
        return fx, fy

    def step(self, nsteps: int, dt: float, precision="fp32c", t: float | None = None):
        """nsteps fixed-dt RK4 steps.  With t, the force time starts at t and
        the time after the steps is returned; without, the steps continue
        from the cloud's force time and None is returned."""
        if t is None:
            self._chk(self.lib.dm_cloud_step(self.h, int(nsteps), float(dt), _prec(precision), None))
            return None
        tt = ctypes.c_double(t)
        self._chk(self.lib.dm_cloud_step(self.h, int(nsteps), float(dt), _prec(precision),
                                         ctypes.byref(tt)))
        return tt.value

    def move_particles(self, end_time: float, dt: float, t: float, precision="fp64",
                       adaptive: bool = False):
        tt = ctypes.c_double(t)
        steps = ctypes.c_int()
        self._chk(self.lib.dm_cloud_move_particles(self.h, float(end_time), float(dt),
                                                   _prec(precision), int(adaptive),
                                                   ctypes.byref(tt), ctypes.byref(steps)))
        return tt.value, steps.value

    def modify_timestep(self, init_dt: float):
        dmin = ctypes.c_float()
        dt = ctypes.c_double()
        self._chk(self.lib.dm_cloud_modify_timestep(self.h, float(init_dt), ctypes.byref(dmin),
                                                    ctypes.byref(dt)))
        return dmin.value, dt.value

    def diagnostics(self):
        out = np.zeros(5)
        self._chk(self.lib.dm_cloud_diagnostics(self.h, ptr(out)))
        return out

    def autotune(self, precision="fp32c"):
        buf = ctypes.create_string_buffer(128)
        split = ctypes.c_int()
        self._chk(self.lib.dm_cloud_autotune(self.h, _prec(precision), buf, len(buf), ctypes.byref(split)))
        return buf.value.decode(), split.value

    def set_kernel(self, variant: str, split: int = 0):
        self._chk(self.lib.dm_cloud_set_kernel(self.h, variant.encode(), int(split)))

    def set_reorder_interval(self, steps: int):
        self._chk(self.lib.dm_cloud_set_reorder_interval(self.h, int(steps)))

    def evaluated_pairs(self) -> int:
        """Ordered pairs the culling kernels swept so far (cumulative)."""
        v = ctypes.c_ulonglong()
        self._chk(self.lib.dm_cloud_evaluated_pairs(self.h, ctypes.byref(v)))
        return int(v.value)

    def set_step_counter(self, step: int):
        self._chk(self.lib.dm_cloud_set_step_counter(self.h, int(step)))

    def get_step_counter(self) -> int:
        v = ctypes.c_uint64()
        self._chk(self.lib.dm_cloud_get_step_counter(self.h, ctypes.byref(v)))
        return v.value

    def set_integrator(self, order: int):
        """4: Runge_Kutta4 (default); 2: Runge_Kutta2, the midpoint method."""
        self._chk(self.lib.dm_cloud_set_integrator(self.h, int(order)))

    def set_time(self, t: float):
        """Force time of the next step (Integrator::currentTime)."""
        self._chk(self.lib.dm_cloud_set_time(self.h, float(t)))

    def get_time(self) -> float:
        v = ctypes.c_double()
        self._chk(self.lib.dm_cloud_get_time(self.h, ctypes.byref(v)))
        return v.value


class DeviceBatch:
    """Many independent clouds advanced together (dm_batch)."""

    def __init__(self, ctx: Context, clouds):
        self.ctx = ctx
        self.lib = ctx.lib
        self.ns = [int(c.n) for c in clouds]
        cat = [np.ascontiguousarray(np.concatenate([getattr(c, k) for c in clouds]), dtype=np.float64)
               for k in ("x", "y", "vx", "vy", "q", "m")]
        params = (_lib.ForceParams * len(clouds))(*[_lib.force_params(**c.params()) for c in clouds])
        nn = (ctypes.c_int * len(clouds))(*self.ns)
        h = ctypes.c_void_p()
        check(self.lib.dm_batch_create(ctx.h, len(clouds), nn, *(ptr(a) for a in cat), params,
                                       ctypes.byref(h)), ctx.h)
        self.h = h
        self.total = sum(self.ns)

    def close(self):
        if self.h:
            self.lib.dm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, nsteps: int, dt: float, precision="fp32c"):
        check(self.lib.dm_batch_step(self.h, int(nsteps), float(dt), _prec(precision)), self.ctx.h)

    def eval_forces(self, precision="fp32c"):
        fx = np.empty(self.total)
        fy = np.empty(self.total)
        check(self.lib.dm_batch_eval_forces(self.h, _prec(precision), ptr(fx), ptr(fy)), self.ctx.h)
        return fx, fy

    def download(self):
        out = [np.empty(self.total) for _ in range(4)]
        check(self.lib.dm_batch_download(self.h, *(ptr(v) for v in out)), self.ctx.h)
        return tuple(out)

    def split(self, arr):
        """Splits a concatenated array into per-cloud arrays."""
        return np.split(arr, np.cumsum(self.ns)[:-1])

    def set_kernel(self, variant: str):
        """Pins a batch kernel variant (names: _lib.batch_variants())."""
        check(self.lib.dm_batch_set_kernel(self.h, variant.encode()), self.ctx.h)

    def evaluated_pairs(self) -> int:
        """Ordered pairs the culling kernels swept so far (cumulative)."""
        v = ctypes.c_ulonglong()
        check(self.lib.dm_batch_evaluated_pairs(self.h, ctypes.byref(v)), self.ctx.h)
        return int(v.value)

    def info(self):
        buf = ctypes.create_string_buffer(128)
        ni = ctypes.c_int()
        g = ctypes.c_int()
        check(self.lib.dm_batch_info(self.h, buf, len(buf), ctypes.byref(ni), ctypes.byref(g)), self.ctx.h)
        return buf.value.decode(), ni.value, g.value

    def set_step_counter(self, step: int):
        check(self.lib.dm_batch_set_step_counter(self.h, int(step)), self.ctx.h)

    def set_integrator(self, order: int):
        check(self.lib.dm_batch_set_integrator(self.h, int(order)), self.ctx.h)

    def set_time(self, t: float):
        check(self.lib.dm_batch_set_time(self.h, float(t)), self.ctx.h)

    def get_time(self) -> float:
        v = ctypes.c_double()
        check(self.lib.dm_batch_get_time(self.h, ctypes.byref(v)), self.ctx.h)
        return v.value
