#!/usr/bin/env python
"""Benchmark of the DEMON RK4 / shielded-Coulomb hot path on GB300.

One "step" is one RK4 step (four fused pair-force + stage launches) of the
workload's cloud.  Metric: pair-interactions/s = 4 * N(N-1) * steps / time
(ordered pairs i != j, four force evaluations per RK4 step), whole job.

    python bench.py [--steps K] [--warmup W] [--workload disk16k]
                    [--precision fp32c] [--impl gb300|reference]

The window: W warm-up steps from the seeded state, then every figure starts
from the state reached (s0) and covers the same steps: `value` (K steps of
the tuned kernel), the FP64 kernel and the fastest unculled FP32C kernel
(the first K64 <= K of those steps, K64 bounded by --fp64-budget), `e2e`
(the K steps again through the C ABI with host buffers), the force error at
the window's last and densest states, the FP32C-vs-FP64 trajectory
divergence at the window's output steps, and the CPU legs (the oracle
stepping from states of the window, all cores and one core).  The
`--impl reference` arm times the oracle over steps W .. W+K-1 of its own
FP64 trajectory.

Multi-GPU (torchrun, one rank per GPU): every rank integrates its own
replica of the workload (independent clouds, no collective on the data path,
weak scaling); the time is the max over ranks.

Prints ONE JSON line on rank 0.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from demon_simulation_code_gb300 import workloads as W  # noqa: E402

METRIC = "pair-interactions/s/GPU: FP32-compensated vs FP64 at <=1e-6 rel force err"
UNIT = "pair-interactions/s"
# algorithmic FP32 flops per ordered pair: dx, dy 2; r^2 3; rsqrt 1; r 1;
# kappa r 1; exp 2; 1 + kappa r 1; r^-3 2; q_j (1 + kappa r) e 2; x C q_i 1;
# fx, fy 4; cutoff compare/select 2 (2 of them on the SFU: rsqrt, ex2)
FLOPS_PER_PAIR = 23


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10000,
                    help="timed RK4 steps (default: the configuration's full 10000-step run)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="disk16k", choices=sorted(W.WORKLOADS))
    ap.add_argument("--precision", default="fp32c", choices=["fp32c", "fp64"])
    ap.add_argument("--fp64-steps", type=int, default=0,
                    help="most FP64 steps of the window to time (0 = all K, within --fp64-budget)")
    ap.add_argument("--fp64-budget", type=float, default=40.0,
                    help="seconds of FP64 steps; the FP64 figures cover the first K64 steps of the window")
    ap.add_argument("--no-unculled", dest="unculled", action="store_false",
                    help="skip the unculled FP32C kernel on the FP64 steps")
    ap.add_argument("--cpu-states", type=int, default=5,
                    help="states of the window (evenly spaced) the CPU legs step from")
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds for the all-cores CPU leg")
    ap.add_argument("--cpu-budget-1core", type=float, default=30.0, help="seconds for the 1-core CPU leg")
    ap.add_argument("--ref-max-steps", type=int, default=40,
                    help="--impl reference: most steps of the window timed on the CPU")
    ap.add_argument("--batch-steps", type=int, default=32)
    ap.add_argument("--adjoint-grads", type=int, default=2,
                    help="timed loss+gradient evaluations of the 64-cloud trajectory fit (0 = skip)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--kernel", default=None, help="pin a kernel variant (skips the autotuner)")
    ap.add_argument("--split", type=int, default=0, help="j split for --kernel (0 = cost model)")
    return ap.parse_args()


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if args.impl == "gb300" else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def workload(name):
    if name == "disk16k":
        return W.disk16k(thermal=True)
    return W.WORKLOADS[name]()


def config_of(w, args, extra=None):
    c = w.clouds[0]
    cfg = {
        "workload": w.name,
        "description": w.description,
        "clouds": len(w.clouds),
        "n": int(c.n) if len(w.clouds) == 1 else [int(x.n) for x in w.clouds][:4] + ["..."],
        "dt": w.dt,
        "pairs_per_force_eval": w.pairs_per_eval,
        "force_evals_per_step": 4,
        "precision": args.precision,
        "l2": "flushed between timed steps (256 MiB write)",
        "parallelism": f"replicas x{args.gpus}",
    }
    if extra:
        cfg.update(extra)
    return cfg


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.skip = 0

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once the sampler is running (nvidia-smi
            # takes a fraction of a second to print its first line)
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.skip = len(self.lines)  # samples taken before the timed region
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.n_inside = len(self.lines) - self.skip  # samples taken during the timed region
            if self.n_inside == 0:
                # a region shorter than the sampling interval holds no sample:
                # wait for the first one after it, so the region is bracketed
                t0 = time.time()
                while len(self.lines) <= self.skip and time.time() - t0 < 1.0 and self.proc.poll() is None:
                    time.sleep(0.01)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], [], set()
        skip = getattr(self, "skip", 0)
        n_inside = getattr(self, "n_inside", len(self.lines) - skip)
        lines = self.lines[skip:skip + n_inside]
        bracket = False
        if n_inside == 0 and skip > 0:
            # no sample inside the region: the last one before it and the first after
            lines = self.lines[skip - 1:skip + 1]
            bracket = True
        for ln in lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) != len(self.FIELDS):
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(self.NAMES, parts[2:]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
               "reasons": sorted(reasons), "samples": len(sm)}
        if bracket:
            out["bracketing"] = "timed region shorter than the 50 ms sampling interval"
        return out


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def _oracle():
    import oracle

    oracle.build()
    return oracle, oracle.Oracle()


def oracle_pair_params(oracle, c):
    """The shielded-Coulomb force alone (for force-error figures)."""
    return oracle.make_params(**{**c.params(), "flags": W.SHIELDED_COULOMB})


def cpu_sample_rate(w, states, nthreads, budget_s):
    """The oracle (restatement of the reference's algorithm, OpenMP with
    per-block locks like ShieldedCoulombForce.cpp) on sampled states of the
    timed window: one RK4 step from each state (one force evaluation where an
    RK4 step is above 5e9 pair interactions), in order until `budget_s` is
    spent (at least one).  Rate = pair interactions / summed time."""
    oracle, o = _oracle()
    c = w.clouds[0]
    p = oracle.make_params(**c.params())
    n = c.n
    per_step = 4.0 * n * (n - 1)
    by_eval = per_step > 5e9
    done, total = [], 0.0
    for k, st, ctr, t in states:
        x, y, vx, vy = st
        t0 = time.perf_counter()
        if by_eval:
            o.forces(x, y, vx, vy, c.q, c.m, p, ctr, 1, nthreads, t)
        else:
            o.rk4_fixed(x, y, vx, vy, c.q, c.m, p, w.dt, 1, ctr, nthreads, t)
        total += time.perf_counter() - t0
        done.append(int(k))
        if total >= budget_s:
            break
    pairs = (n * (n - 1) if by_eval else per_step) * len(done)
    unit = "force evaluation" if by_eval else "RK4 step"
    return pairs / total, total, done, unit


def traffic_from_profiles(kernel: str, workload: str):
    """dram bytes per launch recorded from an ncu capture in profiles/."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def ref_window(args):
    """Steps [first, first + steps) of the reference arm: the GPU arm's
    warm-up and step count, the count capped so that the CPU run stays within
    a few minutes."""
    return max(args.warmup, 3), max(1, min(args.steps, args.ref_max_steps))


def run_reference(args, world, rank):
    """The reference's CPU algorithm (oracle port: the reference sources need
    x86 SSE4.2 and do not build on the Arm host) on this host's cores, over
    the same window of steps as the GPU arm."""
    if rank != 0:
        return 0
    w = workload(args.workload)
    c = w.clouds[0]
    threads = cpu_threads()
    first, nst = ref_window(args)
    oracle, o = _oracle()
    p = oracle.make_params(**c.params())
    # untimed: the reference's own (FP64) trajectory up to the window
    x, y, vx, vy = o.rk4_fixed(c.x, c.y, c.vx, c.vy, c.q, c.m, p, w.dt, first, 0, threads, 0.0)
    t0 = time.perf_counter()
    o.rk4_fixed(x, y, vx, vy, c.q, c.m, p, w.dt, nst, first, threads, first * w.dt)
    el = time.perf_counter() - t0
    rate = 4.0 * c.n * (c.n - 1) * nst / el
    out = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
        "steps": nst, "warmup": first, "ms_per_step": el / nst * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator, demon_simulation_code_gb300/workloads.py)",
        "config": config_of(w, args, {"precision": "fp64 (CPU)"}),
        "window": {"first_step": first, "steps": nst,
                   "state": f"the oracle's own FP64 trajectory from the seeded initial state "
                            f"(steps 0..{first - 1} untimed)"},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"RK4 steps {first}..{first + nst - 1} of {w.name} "
                                   f"(oracle/demon_oracle.c, OpenMP per-block locks as in "
                                   f"ShieldedCoulombForce.cpp), {threads} threads, {el:.2f} s"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))
    return 0


def rel_err(a, b, ax, ay):
    """||(a - ax, b - ay)||_2 / ||(ax, ay)||_2 and max_i |dF_i| / max_i |F_i|."""
    d2 = (a - ax) ** 2 + (b - ay) ** 2
    r2 = ax ** 2 + ay ** 2
    return float(np.sqrt(d2.sum() / r2.sum())), float(np.sqrt(d2.max() / r2.max()))


def run_gb300(args, world, rank, local):
    import torch

    if not torch.cuda.is_available():
        raise SystemExit("bench.py: no CUDA device")
    torch.cuda.set_device(local)
    from demon_simulation_code_gb300 import Context, DeviceCloud, _lib

    w = workload(args.workload)
    c0 = w.clouds[0]
    n = c0.n
    K = args.steps
    pairs_step = 4.0 * n * (n - 1)
    prec = args.precision
    # a dedicated (non-default) stream shared by torch events and the library
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = Context(local)
    ctx.set_stream(stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    radius = float(np.sqrt(np.max(c0.x ** 2 + c0.y ** 2)))  # scale of the trajectory errors
    pin = (args.kernel, args.split) if args.kernel else None

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    def max_over_ranks(v):
        if world == 1:
            return v
        import torch.distributed as dist

        t = torch.tensor([v], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def new_cloud(state, t, ctr, p=None, variant=None, forces=None):
        """A cloud at `state` (caller order), force time t, RNG step ctr.
        Every cloud of the window is made the same way, so they run the same
        internal order and the same arithmetic from the same state."""
        cl = DeviceCloud.from_cloud(ctx, c0)
        if forces is not None:
            cl.set_forces(forces)
        if variant:
            cl.set_kernel(*variant)
        cl.upload(*state)
        cl.set_time(t)
        cl.set_step_counter(ctr)
        cl.autotune(p or prec)  # the context's cached choice; sizes the split buffers before any timing
        torch.cuda.synchronize()
        return cl

    def timed(cl, p, k, budget_s=None, keep=(), states=None):
        """Up to k steps of cl, each timed alone with CUDA events on the
        launching stream after a 256 MiB L2 flush; with budget_s, stops once
        the steps so far took that long.  States at the step indices in
        `keep` go into `states`.  Returns the per-step ms."""
        ms, evs = [], []
        t_start = time.perf_counter()
        for i in range(k):
            if states is not None and i in keep:
                states[i] = cl.download()
            flush.fill_(1.0)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            cl.step(1, w.dt, p)
            b.record(stream)
            evs.append((a, b))
            if budget_s is not None and i % 8 == 7:
                torch.cuda.synchronize()
                if time.perf_counter() - t_start > budget_s:
                    break
        torch.cuda.synchronize()
        ms = [a.elapsed_time(b) for a, b in evs]
        if states is not None:
            states[len(ms)] = cl.download()
        return ms

    # -- the window: autotuning and W warm-up steps from the seeded state,
    #    then every number below starts from the state reached (s0)
    warm = DeviceCloud.from_cloud(ctx, c0)
    if pin:
        warm.set_kernel(*pin)
    tuned = warm.autotune(prec)  # autotuner: variant x split on this cloud
    W_steps = max(args.warmup, 3)
    warm.step(W_steps, w.dt, prec)
    s0 = warm.download()
    t0 = warm.get_time()
    ctr0 = warm.get_step_counter()
    warm.close()

    # -- value: K steps of the tuned kernel from s0
    A = new_cloud(s0, t0, ctr0, variant=pin)
    barrier()
    torch.cuda.synchronize()
    l0 = ctx.launch_count()
    ev0 = A.evaluated_pairs()
    with ClockSampler(local) as clk:
        ms32 = timed(A, prec, K)
    launches_timed = ctx.launch_count() - l0
    swept = A.evaluated_pairs() - ev0  # 0: no culling variant ran, every pair was swept
    end_state = A.download()
    A.close()
    elapsed = sum(ms32) / 1e3
    t_max = max_over_ranks(elapsed)
    value = pairs_step * K * world / t_max

    # -- the same K steps again, untimed, keeping states: per-step swept pairs,
    #    the densest step's input state, the output states, the CPU sample,
    #    and each pair launch timed alone (CUDA events on the launching stream
    #    around every pair launch: kept out of the timed pass, where they
    #    would break the launches' programmatic overlap)
    out_every = 100 if K >= 200 else max(1, K // 4)
    out_steps = set(range(out_every, K, out_every))
    cpu_idx = sorted({int(round(v)) for v in np.linspace(0, K - 1, min(K, args.cpu_states))})
    B = new_cloud(s0, t0, ctr0, variant=pin)
    keep32, swept_steps = {}, []
    dense_k, dense_state, dense_sw = 0, s0, -1
    prev = B.evaluated_pairs()
    ctx.profile(True)
    for k in range(K):
        st = B.download()
        if k in out_steps or k in cpu_idx:
            keep32[k] = st
        flush.fill_(1.0)
        B.step(1, w.dt, prec)
        e = B.evaluated_pairs()
        swept_steps.append(e - prev)
        if e - prev > dense_sw:
            dense_k, dense_state, dense_sw = k, st, e - prev
        prev = e
    pair_ms, launches, _ = ctx.profile_read()
    ctx.profile(False)
    keep32[K] = B.download()
    replay_identical = all(np.array_equal(a, b) for a, b in zip(keep32[K], end_state))
    B.close()

    # -- FP64 kernel from s0 over the first K64 steps of the window (all K
    #    unless that exceeds the time budget), states at the output steps
    states64 = {}
    C = new_cloud(s0, t0, ctr0, p="fp64")
    ms64 = timed(C, "fp64", min(K, args.fp64_steps or K), budget_s=args.fp64_budget, keep=out_steps,
                 states=states64)
    C.close()
    K64 = len(ms64)
    fp64_value = pairs_step * K64 / (sum(ms64) / 1e3)
    same32 = pairs_step * K64 / (sum(ms32[:K64]) / 1e3)

    # -- the fastest unculled FP32C kernel over the same K64 steps (culling
    #    and precision separated)
    unculled = None
    if prec == "fp32c" and args.unculled:
        cands = [v for v in _lib.kernel_variants() if v.startswith("fp32c<") and "cull" not in v]
        best = None
        for v in cands:
            for sp in (0, 4, 8, 16, 32):
                try:
                    T = new_cloud(s0, t0, ctr0, variant=(v, sp))
                except _lib.DemonError:
                    continue
                ms = sum(timed(T, prec, 2))
                T.close()
                if best is None or ms < best[0]:
                    best = (ms, v, sp)
        U = new_cloud(s0, t0, ctr0, variant=best[1:])
        msu = timed(U, prec, K64)
        U.close()
        uval = pairs_step * K64 / (sum(msu) / 1e3)
        unculled = {"variant": best[1], "split": best[2], "steps": K64, "value": uval,
                    "over_fp64": uval / fp64_value,
                    "culled_over_unculled": same32 / uval}

    # -- end to end through the public API with host buffers: pinned H2D of
    #    the state, one RK4 step, D2H of the state, every step, from s0
    pinned = [torch.empty(n, dtype=torch.float64, pin_memory=True) for _ in range(4)]
    hx = [p.numpy() for p in pinned]
    for dst, src in zip(hx, s0):
        dst[:] = src
    E = new_cloud(s0, t0, ctr0, variant=pin)
    barrier()
    torch.cuda.synchronize()
    t_e = time.perf_counter()
    for _ in range(K):
        E.upload(*hx)
        E.step(1, w.dt, prec)
        E.download(out=hx)  # back into the same pinned buffers
    torch.cuda.synchronize()
    e2e_el = max_over_ranks(time.perf_counter() - t_e)
    E.close()
    e2e_value = pairs_step * K * world / e2e_el
    e2e_same = all(np.array_equal(a, b) for a, b in zip(hx, end_state))

    # -- force error of the timed kernel at the window's last and densest
    #    states (shielded-Coulomb force alone), FP32C vs the FP64 kernel
    coul = {**c0.params(), "flags": W.SHIELDED_COULOMB}
    parity = {"forces": "shielded-Coulomb pair force alone", "R_m": radius}
    force_states = {"end": (K, keep32[K]), "dense": (dense_k, dense_state)}
    gpu_forces = {}
    for tag, (k, st) in force_states.items():
        F = new_cloud(st, t0, ctr0 + k, variant=pin, forces=coul)
        f32 = F.eval_forces(prec)
        f64 = F.eval_forces("fp64")
        F.close()
        gpu_forces[tag] = (st, f32, f64)
        e2, emax = rel_err(*f32, *f64)
        parity[f"e_F_{prec}_vs_fp64_{tag}"] = e2
        parity[f"maxrel_F_{prec}_vs_fp64_{tag}"] = emax
    parity["dense_step"] = dense_k
    parity["dense_swept_fraction"] = dense_sw / pairs_step if dense_sw > 0 else None
    # trajectory divergence FP32C vs FP64 from the same s0 at each output
    traj = []
    for k in sorted(set(states64) & set(keep32)):
        a, b = keep32[k], states64[k]
        d = np.sqrt((a[0] - b[0]) ** 2 + (a[1] - b[1]) ** 2) / radius
        traj.append({"step": k, "rms_over_R": float(np.sqrt(np.mean(d ** 2))), "max_over_R": float(d.max())})
    parity["trajectory_fp32c_vs_fp64"] = traj

    # batched workload (256 clouds of uneven N, one persistent launch per stage)
    batch = None
    if args.batch_steps > 0:
        from demon_simulation_code_gb300 import DeviceBatch

        from demon_simulation_code_gb300.shard import assign_clouds, imbalance

        wb = W.batch256()
        # N > 1: whole clouds per rank, balanced by sum N^2 (no exchange)
        parts = assign_clouds([c.n for c in wb.clouds], world)
        mine = [wb.clouds[c] for c in parts[rank]]
        bt = DeviceBatch(ctx, mine)
        bt.step(4, wb.dt)
        torch.cuda.synchronize()
        # like for like: the batched FP32C kernel and the plain FP64 kernel
        # (one cloud at a time, the model split) over the same 4 steps from
        # the same state (the batch's state after its warm-up steps)
        bstate = [bt.split(a) for a in bt.download()]
        start = []
        for k, cb in enumerate(mine):
            c = cb.copy()
            c.x, c.y, c.vx, c.vy = (bstate[a][k].copy() for a in range(4))
            start.append(c)
        pairs_like = 4.0 * 4 * sum(c.n * (c.n - 1) for c in mine)
        b2 = DeviceBatch(ctx, start)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        b2.step(4, wb.dt)
        b.record(stream)
        torch.cuda.synchronize()
        like32 = pairs_like / (a.elapsed_time(b) / 1e3)
        b2.close()
        ctx.set_autotune(False)
        singles = [DeviceCloud.from_cloud(ctx, c) for c in start]
        torch.cuda.synchronize()
        a.record(stream)
        for cl in singles:
            cl.step(4, wb.dt, "fp64")
        b.record(stream)
        torch.cuda.synchronize()
        like64 = pairs_like / (a.elapsed_time(b) / 1e3)
        for cl in singles:
            cl.close()
        ctx.set_autotune(True)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        bev0 = bt.evaluated_pairs()
        a.record(stream)
        bt.step(args.batch_steps, wb.dt)
        b.record(stream)
        torch.cuda.synchronize()
        el = max_over_ranks(a.elapsed_time(b) / 1e3)
        bswept = bt.evaluated_pairs() - bev0
        name, nitems, grid = bt.info()
        batch = {"workload": wb.name, "value": 4.0 * wb.pairs_per_eval * args.batch_steps / el,
                 "unit": UNIT, "steps": args.batch_steps, "ms_per_step": el / args.batch_steps * 1e3,
                 "variant": name, "work_items": nitems, "persistent_grid": grid,
                 "like_for_like_4_steps": {"fp32c_batched": like32, "fp64_one_cloud_at_a_time": like64,
                                           "fp32c_over_fp64": like32 / like64},
                 "graph_captured": args.batch_steps >= 16,
                 "swept_pair_fraction": (bswept / (4.0 * sum(wb.clouds[c].n * (wb.clouds[c].n - 1)
                                                              for c in parts[rank]) * args.batch_steps)
                                         if bswept > 0 else 1.0),
                 "sharding": {"ranks": world, "clouds_per_rank": [len(p) for p in parts],
                              "imbalance": imbalance([c.n for c in wb.clouds], parts),
                              "scaling": "strong"}}
        bt.close()

    # differentiable rollout: 64 clouds x 2048, 200 RK4 steps forward, checkpointed
    # adjoint backward (FP32C pair arithmetic; FP64 targets built untimed)
    adjoint = None
    if args.adjoint_grads > 0:
        from demon_simulation_code_gb300.fit import ShardedTrajectoryFit, TrajectoryFit

        wa = W.adjoint64_smooth()
        # N > 1: whole clouds per rank, per-cloud gradients met in all-reduces
        fit = (ShardedTrajectoryFit(wa, precision="fp32c") if world > 1
               else TrajectoryFit(wa, precision="fp32c"))
        local = fit.local if world > 1 else fit
        fit.loss_and_grad()  # warm-up
        torch.cuda.synchronize()
        barrier()
        al0 = local.K.ctx.launch_count()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        t_a = time.perf_counter()
        a.record(stream)
        for _ in range(args.adjoint_grads):
            L, _ = fit.loss_and_grad()
        b.record(stream)
        torch.cuda.synchronize()
        wall = max_over_ranks(time.perf_counter() - t_a)
        el = max_over_ranks(a.elapsed_time(b) / 1e3)
        kernels = (local.K.ctx.launch_count() - al0) / args.adjoint_grads
        # pair sweeps per gradient: 4 force sweeps per step forward and 4 VJP
        # sweeps per step backward, plus 4 per recomputed step when the stage
        # inputs are not kept
        kept = bool(getattr(local.K, "kept_stages", False))
        sweeps = (8 if kept else 12) * local.steps
        adjoint = {"workload": wa.name, "clouds": len(wa.clouds), "n": wa.clouds[0].n, "steps": local.steps,
                   "stage_inputs": "kept from the forward pass" if kept else
                                   f"recomputed from checkpoints every {local.every} steps",
                   "checkpoint_every": local.every, "precision": "fp32c",
                   "seconds_per_gradient": el / args.adjoint_grads,
                   "wall_seconds_per_gradient": wall / args.adjoint_grads,
                   "pair_sweeps_per_gradient": sweeps, "kernels_per_gradient": kernels,
                   "value": sweeps * sum(c.n * (c.n - 1) for c in wa.clouds) * args.adjoint_grads / el,
                   "unit": UNIT, "loss": float(L), "ranks": world,
                   "gradients": "kappa, q, k_c per cloud; initial positions"}
        del fit, local

    # CPU legs (rank 0, N = 1 host): the oracle on the window's own states
    cpu = cpu1 = None
    if rank == 0 and not args.no_cpu and args.cpu_states > 0:
        oracle, o = _oracle()
        pp = oracle_pair_params(oracle, c0)
        for tag, (st, f32, f64) in gpu_forces.items():
            rx, ry = o.forces(*st, c0.q, c0.m, pp, 0, 1, cpu_threads(), 0.0)
            parity[f"e_F_{prec}_vs_oracle_{tag}"] = rel_err(*f32, rx, ry)[0]
            parity[f"e_F_fp64_vs_oracle_{tag}"] = rel_err(*f64, rx, ry)[0]
        sample = [(k, keep32[k], ctr0 + k, t0 + k * w.dt) for k in cpu_idx]
        threads = cpu_threads()
        for nth, budget in ((threads, args.cpu_budget), (1, args.cpu_budget_1core)):
            rate, el, done, unit = cpu_sample_rate(w, sample, nth, budget)
            rec = {"value": rate, "unit": UNIT, "cores": nth, "kind": "port",
                   "sample": f"one {unit} from each of the window's states at steps {done} "
                             f"(of {K}, same states as the GPU run; oracle/demon_oracle.c, OpenMP "
                             f"per-block locks as in the reference), {nth} thread(s), {el:.2f} s"}
            if nth == threads:
                cpu = rec
            else:
                cpu1 = rec

    # roofline of the dominant kernel (the pair launch; FP32 pipe bound)
    peak = ctx.probe_peak("fp32")
    avg_launch_s = pair_ms / 1e3 / max(launches, 1)
    achieved = FLOPS_PER_PAIR * n * (n - 1) / avg_launch_s / 1e12
    kname = "pair_stage_fp32c" if prec == "fp32c" else "pair_stage_fp64"
    swept_frac = swept / (pairs_step * K) if swept > 0 else 1.0
    traffic = traffic_from_profiles(kname + ("_cull" if "cull" in tuned[0] else ""), w.name)

    if rank == 0:
        res = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
            "warmup": W_steps, "ms_per_step": t_max / K * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if prec == "fp32c" else "f64",
            "data": "synthetic (seeded generator, demon_simulation_code_gb300/workloads.py)",
            "config": config_of(w, args),
            "window": {"first_step": W_steps, "steps": K,
                       "state": "every figure below starts from the state after the warm-up steps "
                                "(same internal order, force time and RNG counter)",
                       "replay_bit_identical": replay_identical},
            "tuning": {"variant": tuned[0], "split": tuned[1]},
            "fp64_value": fp64_value,
            "fp64_steps": K64,
            "fp32c_value_same_steps": same32,
            "fp32c_over_fp64": same32 / fp64_value,
            "fp32c_unculled": unculled,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 4 * 8 * n,
                    "d2h_bytes_per_step": 4 * 8 * n, "steps": K, "same_trajectory": e2e_same},
            "parity": parity,
            "step_ms_percentiles": {p: float(np.percentile(ms32, q))
                                    for p, q in (("p10", 10), ("p50", 50), ("p90", 90), ("max", 100))},
            "swept_fraction_per_step": {p: float(np.percentile(np.array(swept_steps) / pairs_step, q))
                                        for p, q in (("p10", 10), ("p50", 50), ("p90", 90), ("max", 100))},
            "gpu_launches": launches_timed,
            "roofline": {"bound": "fp32-pipe", "kernel": kname, "achieved": achieved,
                         "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                         "traffic": traffic,
                         "flops_per_pair": FLOPS_PER_PAIR,
                         "avg_launch_us": avg_launch_s * 1e6,
                         "launch_timing": "CUDA events around each pair kernel launch alone (the stage "
                                          "finish launch outside them), on the bit-identical replay of "
                                          "the window (L2 flushed before each step)",
                         # box culling skips pair groups out of reach: the work the
                         # kernel actually swept, and the pipe fraction on that work
                         "swept_pair_fraction": swept_frac,
                         "achieved_on_swept": achieved * swept_frac,
                         "frac_on_swept": achieved * swept_frac / peak,
                         "peak_source": "in-run FP32 FMA probe (dm_probe_peak); "
                                        "MEASURED_PEAKS.json has no FP32 figure"},
            "batch": batch,
            "adjoint": adjoint,
            "cpu_baseline": cpu,
            "cpu_baseline_1core": cpu1,
            "clocks": clk.summary(),
        }
        print(json.dumps(res))
    return 0


def main():
    args = parse()
    world, rank, local = dist_init(args)
    args.gpus = world if world > 1 else args.gpus
    try:
        if args.impl == "reference":
            return run_reference(args, world, rank)
        return run_gb300(args, world, rank, local)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
