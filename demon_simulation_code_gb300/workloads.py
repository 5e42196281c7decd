"""Seeded synthetic inputs for the DEMON hot-path workloads.

The reference publishes no dataset; every workload is generated here from a
seed so the CUDA path, the oracle and the CPU baseline see identical inputs.
Constants follow the reference's units: positions [m], velocities [m/s],
charge [C], mass [kg] (m = 4/3 pi rho r^3 with rho = 2200 kg/m^3 and
r = 1.45e-6 m, Cloud.cpp:74-81 gives 2.81e-14 kg).

Workloads (name: sizes):
  disk512     N=512 in a disk of radius 5e-3 m, kappa=2e4, k_c=1e8, drag 3,
              thermal off, dt=1e-4, 1000 steps
  disk16k     N=16384 in a disk of radius 2e-2 m, same constants, Gaussian
              thermal kicks sigma=1e-14 N (counter RNG seed 1), dt=1e-4,
              10000 steps
  square256k  N=262144 in a 0.1 m x 0.1 m square, RectConfinementForce 1e8/1e8,
              charges normal(-1.6e-15, 5%), kappa=5e4, drag 3, dt=5e-5, 100 steps
  batch256    256 clouds, N ~ U{64..4096}, per-cloud kappa ~ U[1e4,5e4],
              q ~ U[-2e-15,-1e-15], k_c ~ U[5e7,2e8], disk radius 2e-4*sqrt(N),
              drag 3, thermal off, dt=1e-4, 2000 steps
  adjoint64   64 clouds of N=2048 in a disk of radius 9e-3 m, true
              (kappa, q, k_c) = (2e4, -1.6e-15, 1e8), 200 steps of dt=1e-4
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

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

# Parameters of the reference's other forces for the parity cases: the
# driver's defaults (driver.cpp:73-105) where they act on a 2 cm cloud, and
# field strengths large enough to matter next to the confinement force.
OTHER_FORCES = dict(void_decay=0.4, drive_const=1e-5, drive_amplitude=1e-13, drive_shift=0.007,
                    magnetic=1.0, rot_rmin=0.005, rot_rmax=0.012, rot_const=1e-15, heat_in=1e-14,
                    heat_out=3e-14, heat_radius=0.01, drag_scale=-1.0, drag_offset=3.0,
                    heat_scale=1e-14, heat_offset=2e-14, electric=1e5, electric_radius=0.01,
                    gravity=-9.8, vert_electric=1e5, vert_decay=0.02)

Q_DUST = -1.6e-15
M_DUST = 2.81e-14


@dataclass
class Cloud:
    """One cloud: state arrays plus force parameters (dm_force_params fields)."""

    x: np.ndarray
    y: np.ndarray
    vx: np.ndarray
    vy: np.ndarray
    q: np.ndarray
    m: np.ndarray
    flags: int = CONFINEMENT | DRAG | SHIELDED_COULOMB
    shielding: float = 2e4
    confine: float = 1e8
    confine_x: float = 0.0
    confine_y: float = 0.0
    gamma: float = 3.0
    heat: float = 0.0
    thermal_mode: int = 1
    seed: int = 0
    extra: dict = field(default_factory=dict)  # the other forces' dm_force_params fields

    @property
    def n(self) -> int:
        return len(self.x)

    def params(self) -> dict:
        return dict(flags=self.flags, shielding=self.shielding, confine=self.confine,
                    confine_x=self.confine_x, confine_y=self.confine_y, gamma=self.gamma,
                    heat=self.heat, thermal_mode=self.thermal_mode, seed=self.seed, **self.extra)

    def copy(self) -> "Cloud":
        c = Cloud(**{k: (v.copy() if isinstance(v, (np.ndarray, dict)) else v)
                     for k, v in self.__dict__.items()})
        return c


def uniform_disk(rng: np.random.Generator, n: int, radius: float):
    """r = R*sqrt(u), theta = 2*pi*u'."""
    r = radius * np.sqrt(rng.random(n))
    th = 2.0 * np.pi * rng.random(n)
    return r * np.cos(th), r * np.sin(th)


def uniform_disk_minsep(rng: np.random.Generator, n: int, radius: float, min_sep: float):
    """Uniform in a disk with every pair at least `min_sep` apart (random
    sequential addition).  Keeps RK4 at dt ~ 1e-4 s well conditioned: the
    reference itself shrinks dt whenever a pair is closer than 1e-4 m
    (Integrator.cpp:68-134)."""
    xs = np.empty(n)
    ys = np.empty(n)
    k = 0
    tries = 0
    while k < n:
        tries += 1
        if tries > 200 * n:
            raise ValueError("min_sep too large for this disk")
        r = radius * np.sqrt(rng.random())
        th = 2.0 * np.pi * rng.random()
        x, y = r * np.cos(th), r * np.sin(th)
        if k and np.min((xs[:k] - x) ** 2 + (ys[:k] - y) ** 2) < min_sep * min_sep:
            continue
        xs[k] = x
        ys[k] = y
        k += 1
    return xs, ys


def calm_cloud(n: int = 512, radius: float = 1e-2, seed: int = 0, min_sep: float = 4e-4,
               vscale: float = 1e-4) -> Cloud:
    """A well-conditioned cloud for gated trajectory comparisons: minimum pair
    separation 4e-4 m, kappa = 5e3 (Coulomb is ~25-70% of the force),
    k_c = 1e4 (no collapse within a few hundred steps of 1e-4 s), small random
    velocities.  A 1e-15 relative perturbation stays ~1e-15 over 300 steps,
    so FP64 trajectories can be gated at 1e-12."""
    rng = np.random.default_rng(seed)
    x, y = uniform_disk_minsep(rng, n, radius, min_sep)
    return Cloud(x=x, y=y, vx=rng.normal(0, vscale, n), vy=rng.normal(0, vscale, n),
                 q=np.full(n, Q_DUST), m=np.full(n, M_DUST),
                 flags=CONFINEMENT | DRAG | SHIELDED_COULOMB, shielding=5e3, confine=1e4,
                 gamma=3.0)


def disk_cloud(n: int, radius: float, seed: int, *, shielding=2e4, confine=1e8, gamma=3.0,
               q=Q_DUST, m=M_DUST, heat=0.0, thermal_seed=0) -> Cloud:
    rng = np.random.default_rng(seed)
    x, y = uniform_disk(rng, n, radius)
    flags = CONFINEMENT | DRAG | SHIELDED_COULOMB | (THERMAL if heat > 0 else 0)
    return Cloud(x=x, y=y, vx=np.zeros(n), vy=np.zeros(n), q=np.full(n, q), m=np.full(n, m),
                 flags=flags, shielding=shielding, confine=confine, gamma=gamma, heat=heat,
                 thermal_mode=1, seed=thermal_seed)


@dataclass
class Workload:
    name: str
    clouds: list
    dt: float
    steps: int
    description: str = ""
    extra: dict = field(default_factory=dict)

    @property
    def pairs_per_eval(self) -> int:
        """Ordered pairs (i, j), i != j, in one force evaluation."""
        return int(sum(c.n * (c.n - 1) for c in self.clouds))


def disk512(seed: int = 0) -> Workload:
    c = disk_cloud(512, 5e-3, seed)
    return Workload("disk512", [c], 1e-4, 1000,
                    "N=512 disk R=5e-3 m, kappa=2e4, k_c=1e8, drag 3, thermal off, dt=1e-4")


def disk16k(seed: int = 1, thermal: bool = True) -> Workload:
    c = disk_cloud(16384, 2e-2, seed, heat=1e-14 if thermal else 0.0, thermal_seed=1)
    return Workload("disk16k", [c], 1e-4, 10000,
                    "N=16384 disk R=2e-2 m, kappa=2e4, k_c=1e8, drag 3, "
                    f"thermal {'Gaussian sigma=1e-14 N' if thermal else 'off'}, dt=1e-4")


def disk16k_dense(seed: int = 1) -> Workload:
    """disk16k's particles in a 7e-4 m disk: ~35% of all pairs inside the
    cutoff, the density disk16k reaches when it collapses under its
    confinement (for profiling the precise path; the state explodes within a
    few steps)."""
    c = disk_cloud(16384, 7e-4, seed, heat=1e-14, thermal_seed=1)
    return Workload("disk16k_dense", [c], 1e-4, 10,
                    "N=16384 disk R=7e-4 m (35% of pairs within kappa*r < 10), kappa=2e4, k_c=1e8")


def square256k(seed: int = 2, n: int = 262144) -> Workload:
    rng = np.random.default_rng(seed)
    x = (rng.random(n) - 0.5) * 0.1
    y = (rng.random(n) - 0.5) * 0.1
    q = rng.normal(Q_DUST, abs(Q_DUST) * 0.05, n)
    c = Cloud(x=x, y=y, vx=np.zeros(n), vy=np.zeros(n), q=q, m=np.full(n, M_DUST),
              flags=RECT_CONFINEMENT | DRAG | SHIELDED_COULOMB, shielding=5e4, confine=0.0,
              confine_x=1e8, confine_y=1e8, gamma=3.0)
    return Workload("square256k", [c], 5e-5, 100,
                    f"N={n} square 0.1 m, Rect 1e8/1e8, q~N(-1.6e-15,5%), kappa=5e4, dt=5e-5")


def batch256(seed: int = 3, nclouds: int = 256, nmin: int = 64, nmax: int = 4096) -> Workload:
    rng = np.random.default_rng(seed)
    ns = rng.integers(nmin, nmax + 1, nclouds)
    clouds = []
    for c in range(nclouds):
        n = int(ns[c])
        kappa = rng.uniform(1e4, 5e4)
        q = rng.uniform(-2e-15, -1e-15)
        kc = rng.uniform(5e7, 2e8)
        x, y = uniform_disk(rng, n, 2e-4 * np.sqrt(n))
        clouds.append(Cloud(x=x, y=y, vx=np.zeros(n), vy=np.zeros(n), q=np.full(n, q),
                            m=np.full(n, M_DUST), shielding=kappa, confine=kc, gamma=3.0))
    return Workload("batch256", clouds, 1e-4, 2000,
                    f"{nclouds} clouds, N~U{{{nmin}..{nmax}}}, per-cloud kappa/q/k_c, dt=1e-4")


def adjoint64(seed: int = 4, nclouds: int = 64, n: int = 2048) -> Workload:
    rng = np.random.default_rng(seed)
    clouds = []
    for _ in range(nclouds):
        x, y = uniform_disk(rng, n, 9e-3)
        clouds.append(Cloud(x=x, y=y, vx=np.zeros(n), vy=np.zeros(n), q=np.full(n, Q_DUST),
                            m=np.full(n, M_DUST), shielding=2e4, confine=1e8, gamma=3.0))
    return Workload("adjoint64", clouds, 1e-4, 200,
                    f"{nclouds} clouds N={n} disk R=9e-3, true (kappa,q,k_c)=(2e4,-1.6e-15,1e8)",
                    extra={"perturb": 0.2, "checkpoint_every": 20})


def adjoint64_smooth(seed: int = 4, nclouds: int = 64, n: int = 2048) -> Workload:
    """adjoint64's shape (64 x 2048 in a 9e-3 m disk, 200 steps of 1e-4 s,
    checkpoints every 20, +/-20% start) with a loss that is smooth in every
    parameter, for gradient checks against finite differences: minimum pair
    separation 1.2e-4 m, kappa = 400 so that the cutoff radius 10/kappa
    (>= 20.8 mm over the +/-20% range) exceeds the cloud's diameter and no pair
    crosses kappa*r = 10 during the rollout, k_c = 4e4.

    adjoint64 itself is chaotic: k_c = 1e8 pulls the random disk through its
    centre every 0.66 ms, where close pairs are kicked by millimetres per
    step.  And wherever pairs cross the cutoff, the reference's force jumps
    there, so a central difference picks up jump terms that no derivative
    has."""
    rng = np.random.default_rng(seed)
    clouds = []
    for _ in range(nclouds):
        x, y = uniform_disk_minsep(rng, n, 9e-3, 1.2e-4)
        clouds.append(Cloud(x=x, y=y, vx=rng.normal(0, 1e-4, n), vy=rng.normal(0, 1e-4, n),
                            q=np.full(n, Q_DUST), m=np.full(n, M_DUST), shielding=400.0, confine=4e4,
                            gamma=3.0))
    return Workload("adjoint64_smooth", clouds, 1e-4, 200,
                    f"{nclouds} clouds N={n} disk R=9e-3, min separation 1.2e-4, "
                    "true (kappa,q,k_c)=(400,-1.6e-15,4e4)",
                    extra={"perturb": 0.2, "checkpoint_every": 20})


WORKLOADS = {"disk512": disk512, "disk16k": disk16k, "disk16k_dense": disk16k_dense, "square256k": square256k,
             "batch256": batch256, "adjoint64": adjoint64, "adjoint64_smooth": adjoint64_smooth}
