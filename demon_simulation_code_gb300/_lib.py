"""ctypes binding of libdemon_gb300.so (the C ABI in include/demon_gb300.h).

There is no CPU fallback: if the library is missing or the GPU is not an
sm_103a device, every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import LIB

DM_OK = 0
DM_ERR_ARG = 1
DM_FP64 = 0
DM_FP32C = 1

_dp = ctypes.POINTER(ctypes.c_double)
_lib = None


class DemonError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[dm status {code}] {message}")
        self.code = code


class ForceParams(ctypes.Structure):
    """dm_force_params."""

    _fields_ = [
        ("flags", ctypes.c_longlong),
        ("shielding", ctypes.c_double),
        ("confine", ctypes.c_double),
        ("confine_x", ctypes.c_double),
        ("confine_y", ctypes.c_double),
        ("gamma", ctypes.c_double),
        ("heat", ctypes.c_double),
        ("thermal_mode", ctypes.c_int),
        ("reserved", ctypes.c_int),
        ("seed", ctypes.c_uint64),
        ("void_decay", ctypes.c_double),
        ("drive_const", ctypes.c_double),
        ("drive_amplitude", ctypes.c_double),
        ("drive_shift", ctypes.c_double),
        ("magnetic", ctypes.c_double),
        ("rot_rmin", ctypes.c_double),
        ("rot_rmax", ctypes.c_double),
        ("rot_const", ctypes.c_double),
        ("heat_in", ctypes.c_double),
        ("heat_out", ctypes.c_double),
        ("heat_radius", ctypes.c_double),
        ("drag_scale", ctypes.c_double),
        ("drag_offset", ctypes.c_double),
        ("heat_scale", ctypes.c_double),
        ("heat_offset", ctypes.c_double),
        ("electric", ctypes.c_double),
        ("electric_radius", ctypes.c_double),
        ("gravity", ctypes.c_double),
        ("vert_electric", ctypes.c_double),
        ("vert_decay", ctypes.c_double),
    ]


# dm_force_params fields after seed, in order
EXTRA_FIELDS = [
    "void_decay", "drive_const", "drive_amplitude", "drive_shift", "magnetic",
    "rot_rmin", "rot_rmax", "rot_const", "heat_in", "heat_out", "heat_radius",
    "drag_scale", "drag_offset", "heat_scale", "heat_offset", "electric",
    "electric_radius", "gravity", "vert_electric", "vert_decay",
]


def force_params(flags, shielding=2e4, confine=0.0, confine_x=0.0, confine_y=0.0, gamma=0.0,
                 heat=0.0, thermal_mode=1, seed=0, **extra) -> ForceParams:
    """extra: the other forces' fields of dm_force_params by name (0 if not given)."""
    p = ForceParams(int(flags), shielding, confine, confine_x, confine_y, gamma, heat, int(thermal_mode), 0,
                    int(seed))
    for k, v in extra.items():
        if k not in EXTRA_FIELDS:
            raise TypeError(f"unknown force parameter {k!r}")
        setattr(p, k, float(v))
    return p


# (name, restype, argtypes) of every exported symbol
SIGNATURES = {
    "dm_version": (ctypes.c_int, []),
    "dm_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "dm_ctx_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dm_ctx_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "dm_ctx_reset_stream": (ctypes.c_int, [ctypes.c_void_p]),
    "dm_ctx_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "dm_last_error": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]),
    "dm_ctx_profile_enable": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "dm_ctx_launch_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "dm_ctx_profile_read": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.POINTER(ctypes.c_longlong), _dp]),
    "dm_probe_peak": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp]),
    "dm_ctx_set_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "dm_kernel_variants": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "dm_cloud_set_kernel": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]),
    "dm_cloud_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t,
                                         ctypes.POINTER(ctypes.c_int)]),
    "dm_cloud_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp,
                                       ctypes.POINTER(ctypes.c_void_p)]),
    "dm_cloud_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dm_cloud_size": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    # the per-step state transfers take plain addresses (addr): building a
    # typed pointer per array costs more than the rest of the call's host work
    "dm_cloud_upload": (ctypes.c_int, [ctypes.c_void_p] * 5),
    "dm_cloud_download": (ctypes.c_int, [ctypes.c_void_p] * 5),
    "dm_cloud_set_charge_mass": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp]),
    "dm_cloud_set_forces": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ForceParams)]),
    "dm_cloud_eval_forces": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp]),
    "dm_cloud_eval_forces_stage": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp]),
    "dm_cloud_evaluated_pairs": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_ulonglong)]),
    "dm_batch_evaluated_pairs": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_ulonglong)]),
    "dm_batch_variants": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "dm_batch_set_kernel": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "dm_cloud_eval_forces_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                   ctypes.c_void_p]),
    "dm_cloud_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp]),
    "dm_cloud_move_particles": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_int, ctypes.c_int, _dp,
                                               ctypes.POINTER(ctypes.c_int)]),
    "dm_cloud_modify_timestep": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double,
                                                ctypes.POINTER(ctypes.c_float), _dp]),
    "dm_cloud_diagnostics": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "dm_cloud_set_reorder_interval": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "dm_cloud_set_step_counter": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "dm_cloud_get_step_counter": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
    "dm_cloud_set_integrator": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "dm_cloud_set_time": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "dm_cloud_get_time": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "dm_batch_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _dp, _dp,
                                       _dp, _dp, _dp, _dp, ctypes.POINTER(ForceParams),
                                       ctypes.POINTER(ctypes.c_void_p)]),
    "dm_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dm_batch_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int]),
    "dm_batch_eval_forces": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp]),
    "dm_batch_download": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp, _dp]),
    "dm_batch_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t,
                                     ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "dm_batch_set_step_counter": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "dm_batch_set_integrator": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "dm_batch_set_time": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "dm_batch_get_time": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "dm_adjoint_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(ForceParams), ctypes.POINTER(ctypes.c_void_p)]),
    "dm_adjoint_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "dm_adjoint_set_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ForceParams)]),
    "dm_adjoint_forces": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 10),
    "dm_adjoint_vjp": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 15),
    "dm_adjoint_rk4_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double] + [ctypes.c_void_p] * 7),
    "dm_adjoint_rk4_step_vjp": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]
                                + [ctypes.c_void_p] * 10),
    "dm_diagnostics_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.POINTER(ForceParams),
                                              ctypes.c_void_p, ctypes.c_void_p]),
}


def load(path: str = LIB) -> ctypes.CDLL:
    """Loads the library (no build, no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error(ctx) -> str:
    buf = ctypes.create_string_buffer(1024)
    load().dm_last_error(ctx, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, ctx=None) -> None:
    if rc != DM_OK:
        raise DemonError(rc, last_error(ctx))


def batch_variants() -> list[str]:
    buf = ctypes.create_string_buffer(4096)
    check(load().dm_batch_variants(buf, len(buf)))
    return buf.value.decode().split(";")


def kernel_variants() -> list[str]:
    buf = ctypes.create_string_buffer(4096)
    check(load().dm_kernel_variants(buf, len(buf)))
    return buf.value.decode().split(";")


def ptr(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float64 array")
    return a.ctypes.data_as(_dp)


def addr(a: np.ndarray) -> int:
    """The address of a C-contiguous float64 array (for c_void_p arguments)."""
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float64 array")
    return a.ctypes.data
