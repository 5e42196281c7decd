"""ctypes bindings of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this package, and only as the checker (or the timed CPU baseline).
The product library never links or calls it.

Two libraries are exposed:

* ``liboracle.so``: the plain-C restatement (demon_oracle.c), built on any
  architecture by ``make`` in this directory.
* ``_ref/libdemon_ref.so`` (serial) and ``_ref/libdemon_ref_omp.so``: the
  reference's own sources compiled with a stub fitsio.h (``make ref``, x86-64
  only, needs the reference checkout).  Used to pin the restatement.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libdemon_ref.so")
REF_OMP_SO = os.path.join(HERE, "_ref", "libdemon_ref_omp.so")

_dp = ctypes.POINTER(ctypes.c_double)

# ForceFlag bits (Force.h:75-91)
CONFINEMENT = 1
DRAG = 2
SHIELDED_COULOMB = 4
GRAVITATIONAL = 8
THERMAL = 16
THERMAL_LOCALIZED = 32
DRIVING = 64
ROTATIONAL = 128
TIME_VARYING_DRAG = 256
TIME_VARYING_THERMAL = 512
MAGNETIC = 1024
CONFINEMENT_VOID = 2048
ELECTRIC = 4096
RECT_CONFINEMENT = 8192
VERT_ELECTRIC = 16384

# or_params fields after seed, in order
EXTRA_FIELDS = [
    "void_decay", "drive_const", "drive_amplitude", "drive_shift", "magnetic",
    "rot_rmin", "rot_rmax", "rot_const", "heat_in", "heat_out", "heat_radius",
    "drag_scale", "drag_offset", "heat_scale", "heat_offset", "electric",
    "electric_radius", "gravity", "vert_electric", "vert_decay",
]


class Params(ctypes.Structure):
    """Same layout as ``or_params`` / ``dm_force_params``."""

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


def make_params(flags=CONFINEMENT | DRAG | SHIELDED_COULOMB, shielding=2e4, confine=1e8,
                confine_x=0.0, confine_y=0.0, gamma=3.0, heat=0.0, thermal_mode=1, seed=0, **extra):
    """extra: the other forces' fields of or_params by name (0 if not given)."""
    p = Params(flags, shielding, confine, confine_x, confine_y, gamma, heat, thermal_mode, 0, seed)
    for k, v in extra.items():
        if k not in EXTRA_FIELDS:
            raise TypeError(f"unknown force parameter {k!r}")
        setattr(p, k, float(v))
    return p


def _ptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def ref_dir() -> str | None:
    """The reference checkout named by the environment variable
    DEMON_REF_DIR (None when unset or not a directory)."""
    d = os.environ.get("DEMON_REF_DIR", "")
    return d if d and os.path.isdir(d) else None


def build(ref: bool = False) -> None:
    """Compile the restatement (and, if asked, the reference from the
    checkout named by DEMON_REF_DIR)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def ref_available() -> bool:
    return os.path.exists(REF_SO)


class Oracle:
    """The plain-C restatement."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        self.lib = lib
        lib.or_coulomb.restype = ctypes.c_double
        lib.or_shielded_coulomb.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, _dp, _dp]
        lib.or_shielded_coulomb_omp.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_double,
                                                _dp, _dp, ctypes.c_int]
        lib.or_forces.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp,
                                  ctypes.POINTER(Params), ctypes.c_uint64, ctypes.c_int,
                                  ctypes.c_double, _dp, _dp, ctypes.c_int]
        lib.or_forces_rows.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp,
                                       ctypes.POINTER(Params), ctypes.c_uint64, ctypes.c_int,
                                       ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                       _dp, _dp, ctypes.c_int]
        lib.or_rk4_fixed.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp,
                                     ctypes.POINTER(Params), ctypes.c_double, ctypes.c_double,
                                     ctypes.c_int, ctypes.c_uint64, ctypes.c_int]
        lib.or_modify_timestep.restype = ctypes.c_double
        lib.or_modify_timestep.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_float, ctypes.c_double]
        lib.or_checked_min_dist.restype = ctypes.c_float
        lib.or_checked_min_dist.argtypes = [ctypes.c_int, _dp, _dp]
        lib.or_rk4_move_particles.restype = ctypes.c_int
        lib.or_rk4_move_particles.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp,
                                              ctypes.POINTER(Params), ctypes.c_double, _dp,
                                              ctypes.c_double, ctypes.c_uint64, ctypes.c_int]
        lib.or_rk2_fixed.argtypes = lib.or_rk4_fixed.argtypes
        lib.or_rk2_move_particles.restype = ctypes.c_int
        lib.or_rk2_move_particles.argtypes = lib.or_rk4_move_particles.argtypes
        lib.or_diagnostics.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp,
                                       ctypes.POINTER(Params), _dp]
        lib.or_thermal_one.argtypes = [ctypes.POINTER(Params), ctypes.c_uint32, ctypes.c_uint64,
                                       ctypes.c_int, _dp, _dp]
        lib.or_philox4x32_10.argtypes = [ctypes.POINTER(ctypes.c_uint32),
                                         ctypes.POINTER(ctypes.c_uint32),
                                         ctypes.POINTER(ctypes.c_uint32)]

    def coulomb(self) -> float:
        return self.lib.or_coulomb()

    def shielded_coulomb(self, x, y, q, kappa, nthreads=1):
        n = len(x)
        fx = np.zeros(n)
        fy = np.zeros(n)
        if nthreads == 1:
            self.lib.or_shielded_coulomb(n, _ptr(x), _ptr(y), _ptr(q), kappa, _ptr(fx), _ptr(fy))
        else:
            self.lib.or_shielded_coulomb_omp(n, _ptr(x), _ptr(y), _ptr(q), kappa, _ptr(fx),
                                             _ptr(fy), nthreads)
        return fx, fy

    def forces(self, x, y, vx, vy, q, m, params, step=0, stage=1, nthreads=1, t=0.0):
        n = len(x)
        fx = np.zeros(n)
        fy = np.zeros(n)
        self.lib.or_forces(n, _ptr(x), _ptr(y), _ptr(vx), _ptr(vy), _ptr(q), _ptr(m),
                           ctypes.byref(params), step, stage, t, _ptr(fx), _ptr(fy), nthreads)
        return fx, fy

    def forces_rows(self, x, y, vx, vy, q, m, params, rows, step=0, stage=1, nthreads=1, t=0.0):
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        fx = np.zeros(len(rows))
        fy = np.zeros(len(rows))
        self.lib.or_forces_rows(len(x), _ptr(x), _ptr(y), _ptr(vx), _ptr(vy), _ptr(q), _ptr(m),
                                ctypes.byref(params), step, stage, t, len(rows),
                                rows.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _ptr(fx), _ptr(fy),
                                nthreads)
        return fx, fy

    def rk4_fixed(self, x, y, vx, vy, q, m, params, dt, nsteps, step0=0, nthreads=1, t0=0.0):
        x, y, vx, vy = (np.array(a, dtype=np.float64, copy=True) for a in (x, y, vx, vy))
        self.lib.or_rk4_fixed(len(x), _ptr(x), _ptr(y), _ptr(vx), _ptr(vy), _ptr(q), _ptr(m),
                              ctypes.byref(params), t0, dt, nsteps, step0, nthreads)
        return x, y, vx, vy

    def rk2_fixed(self, x, y, vx, vy, q, m, params, dt, nsteps, step0=0, nthreads=1, t0=0.0):
        x, y, vx, vy = (np.array(a, dtype=np.float64, copy=True) for a in (x, y, vx, vy))
        self.lib.or_rk2_fixed(len(x), _ptr(x), _ptr(y), _ptr(vx), _ptr(vy), _ptr(q), _ptr(m),
                              ctypes.byref(params), t0, dt, nsteps, step0, nthreads)
        return x, y, vx, vy

    def rk2_move_particles(self, x, y, vx, vy, q, m, params, init_dt, t0, end_time, step0=0, nthreads=1):
        x, y, vx, vy = (np.array(a, dtype=np.float64, copy=True) for a in (x, y, vx, vy))
        t = ctypes.c_double(t0)
        steps = self.lib.or_rk2_move_particles(len(x), _ptr(x), _ptr(y), _ptr(vx), _ptr(vy),
                                               _ptr(q), _ptr(m), ctypes.byref(params), init_dt,
                                               ctypes.byref(t), end_time, step0, nthreads)
        return x, y, vx, vy, steps, t.value

    def modify_timestep(self, x, y, dt, dist=1.0e-4):
        return self.lib.or_modify_timestep(len(x), _ptr(x), _ptr(y), dist, dt)

    def checked_min_dist(self, x, y):
        return self.lib.or_checked_min_dist(len(x), _ptr(x), _ptr(y))

    def rk4_move_particles(self, x, y, vx, vy, q, m, params, init_dt, t0, end_time,
                           step0=0, nthreads=1):
        x, y, vx, vy = (np.array(a, dtype=np.float64, copy=True) for a in (x, y, vx, vy))
        t = ctypes.c_double(t0)
        steps = self.lib.or_rk4_move_particles(len(x), _ptr(x), _ptr(y), _ptr(vx), _ptr(vy),
                                               _ptr(q), _ptr(m), ctypes.byref(params), init_dt,
                                               ctypes.byref(t), end_time, step0, nthreads)
        return x, y, vx, vy, steps, t.value

    def diagnostics(self, x, y, vx, vy, q, m, params):
        out = np.zeros(5)
        self.lib.or_diagnostics(len(x), _ptr(x), _ptr(y), _ptr(vx), _ptr(vy), _ptr(q), _ptr(m),
                                ctypes.byref(params), _ptr(out))
        return out

    def thermal(self, params, n, step, stage):
        tx = np.zeros(n)
        ty = np.zeros(n)
        a = ctypes.c_double()
        b = ctypes.c_double()
        for i in range(n):
            self.lib.or_thermal_one(ctypes.byref(params), i, step, stage, ctypes.byref(a),
                                    ctypes.byref(b))
            tx[i] = a.value
            ty[i] = b.value
        return tx, ty

    def philox(self, ctr, key):
        c = (ctypes.c_uint32 * 4)(*ctr)
        k = (ctypes.c_uint32 * 2)(*key)
        o = (ctypes.c_uint32 * 4)()
        self.lib.or_philox4x32_10(c, k, o)
        return list(o)


class Reference:
    """The reference's own sources compiled against a stub fitsio.h."""

    def __init__(self, path: str = REF_SO):
        lib = ctypes.CDLL(path)
        self.lib = lib
        lib.ref_shielded_coulomb.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, _dp, _dp]
        lib.ref_forces_at.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp,
                                      ctypes.c_void_p, ctypes.c_double, ctypes.c_int, _dp, _dp]
        lib.ref_rk4_move_particles.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp,
                                               ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_double, _dp]
        lib.ref_rk2_move_particles.argtypes = lib.ref_rk4_move_particles.argtypes
        lib.ref_rk4_fixed.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp,
                                      ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int]

    def shielded_coulomb(self, x, y, q, kappa):
        n = len(x)
        fx = np.zeros(n)
        fy = np.zeros(n)
        rc = self.lib.ref_shielded_coulomb(n, _ptr(x), _ptr(y), _ptr(q), kappa, _ptr(fx), _ptr(fy))
        if rc:
            raise ValueError("reference needs even n")
        return fx, fy

    def forces(self, x, y, vx, vy, q, m, params, t=0.0, thermal=False):
        """Every flagged force's force1(t) in driver order.  thermal=False
        leaves out the three thermal forces (the reference seeds them from
        the clock, RandomNumbers.cpp:18-20)."""
        n = len(x)
        fx = np.zeros(n)
        fy = np.zeros(n)
        rc = self.lib.ref_forces_at(n, _ptr(x), _ptr(y), _ptr(vx), _ptr(vy), _ptr(q), _ptr(m),
                                    ctypes.byref(params), t, int(thermal), _ptr(fx), _ptr(fy))
        if rc:
            raise ValueError("reference needs even n")
        return fx, fy

    def rk4_fixed(self, x, y, vx, vy, q, m, params, dt, nsteps, t0=0.0):
        x, y, vx, vy = (np.array(a, dtype=np.float64, copy=True) for a in (x, y, vx, vy))
        rc = self.lib.ref_rk4_fixed(len(x), _ptr(x), _ptr(y), _ptr(vx), _ptr(vy), _ptr(q), _ptr(m),
                                    ctypes.byref(params), t0, dt, nsteps)
        if rc < 0:
            raise ValueError("reference needs even n")
        return x, y, vx, vy

    def rk4_move_particles(self, x, y, vx, vy, q, m, params, dt, t0, end_time):
        x, y, vx, vy = (np.array(a, dtype=np.float64, copy=True) for a in (x, y, vx, vy))
        t = ctypes.c_double()
        steps = self.lib.ref_rk4_move_particles(len(x), _ptr(x), _ptr(y), _ptr(vx), _ptr(vy),
                                                _ptr(q), _ptr(m), ctypes.byref(params), dt, t0,
                                                end_time, ctypes.byref(t))
        if steps < 0:
            raise ValueError("reference needs n % 4 == 0")
        return x, y, vx, vy, steps, t.value

    def rk2_move_particles(self, x, y, vx, vy, q, m, params, dt, t0, end_time):
        x, y, vx, vy = (np.array(a, dtype=np.float64, copy=True) for a in (x, y, vx, vy))
        t = ctypes.c_double()
        steps = self.lib.ref_rk2_move_particles(len(x), _ptr(x), _ptr(y), _ptr(vx), _ptr(vy),
                                                _ptr(q), _ptr(m), ctypes.byref(params), dt, t0,
                                                end_time, ctypes.byref(t))
        if steps < 0:
            raise ValueError("reference needs n % 4 == 0")
        return x, y, vx, vy, steps, t.value
