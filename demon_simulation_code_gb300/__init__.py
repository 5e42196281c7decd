"""GB300 (sm_103a) implementation of DEMON's RK4 dusty-plasma hot path.

The compute path is libdemon_gb300.so (hand-written CUDA behind a C ABI,
include/demon_gb300.h).  This package holds its ctypes binding
(``_lib``), a thin object API over it (``cloud``), the seeded synthetic
workloads (``workloads``) and the build script (``build``).
"""
from ._lib import DM_FP32C, DM_FP64, DemonError, force_params, load  # noqa: F401
from .cloud import Context, DeviceBatch, DeviceCloud  # noqa: F401
