#!/usr/bin/env python
"""Benchmark of the DEMON RK4 / shielded-Coulomb hot path on GB300.

One "step" is one RK4 step (four fused pair-force + stage launches) of the
workload's cloud.  Metric: pair-interactions/s = 4 * N(N-1) * steps / time
(ordered pairs i != j, four force evaluations per RK4 step), whole job.

    python bench.py [--steps K] [--warmup W] [--workload disk16k]
                    [--precision fp32c] [--impl gb300|reference]

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
    ap.add_argument("--fp64-steps", type=int, default=10)
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--cpu-steps", type=int, default=2)
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


def cpu_rk4_rate(w, nsteps, nthreads):
    """The oracle (restatement of the reference's algorithm, OpenMP, per-block
    locks like the reference) on `nsteps` RK4 steps of the first cloud."""
    import oracle

    oracle.build()
    o = oracle.Oracle()
    c = w.clouds[0]
    p = oracle.make_params(**c.params())
    t0 = time.perf_counter()
    o.rk4_fixed(c.x, c.y, c.vx, c.vy, c.q, c.m, p, w.dt, nsteps, 0, nthreads)
    el = time.perf_counter() - t0
    pairs = 4.0 * c.n * (c.n - 1) * nsteps
    return pairs / el, el


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


def run_reference(args, world, rank):
    """The reference's CPU algorithm (oracle port: the reference sources need
    x86 SSE4.2 and do not build on the Arm host) on this host's cores."""
    if rank != 0:
        return 0
    w = workload(args.workload)
    threads = cpu_threads()
    nst = max(1, min(args.steps, 10))
    if args.warmup > 0:
        cpu_rk4_rate(w, 1, threads)
    rate, el = cpu_rk4_rate(w, nst, threads)
    out = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
        "steps": nst, "warmup": min(args.warmup, 1), "ms_per_step": el / nst * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator, demon_simulation_code_gb300/workloads.py)",
        "config": config_of(w, args, {"precision": "fp64 (CPU)"}),
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{nst} RK4 steps of {w.name} (oracle/demon_oracle.c, OpenMP "
                                   f"per-block locks as in ShieldedCoulombForce.cpp), "
                                   f"{threads} threads, {el:.2f} s"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))
    return 0


def run_gb300(args, world, rank, local):
    import torch

    if not torch.cuda.is_available():
        raise SystemExit("bench.py: no CUDA device")
    torch.cuda.set_device(local)
    from demon_simulation_code_gb300 import Context, DeviceCloud

    w = workload(args.workload)
    c0 = w.clouds[0]
    n = c0.n
    pairs_step = 4.0 * n * (n - 1)
    # a dedicated (non-default) stream shared by torch events and the library
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = Context(local)
    ctx.set_stream(stream.cuda_stream)
    cloud = DeviceCloud.from_cloud(ctx, c0)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    step_ms = []

    def timed_steps(prec, k):
        evs = []
        for _ in range(k):
            flush.fill_(1.0)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            cloud.step(1, w.dt, prec)
            b.record(stream)
            evs.append((a, b))
        torch.cuda.synchronize()
        ms = [a.elapsed_time(b) for a, b in evs]
        step_ms[:] = ms
        return sum(ms) / 1e3

    if args.kernel:
        cloud.set_kernel(args.kernel, args.split)
    tuned = cloud.autotune(args.precision)  # autotuner: variant x split on this cloud
    # warm-up (untimed)
    cloud.step(max(args.warmup, 3), w.dt, args.precision)
    torch.cuda.synchronize()

    # timed region: K steps, pair kernels bracketed by events inside the library
    ctx.profile(True)
    barrier()
    torch.cuda.synchronize()
    l0 = ctx.launch_count()
    ev0 = cloud.evaluated_pairs()
    with ClockSampler(local) as clk:
        elapsed = timed_steps(args.precision, args.steps)
    launches_timed = ctx.launch_count() - l0
    # ordered pairs the culling kernel swept (0: no culling variant ran, every pair was swept)
    swept = cloud.evaluated_pairs() - ev0
    pair_ms, launches, pairs_prof = ctx.profile_read()
    main_step_ms = list(step_ms)
    ctx.profile(False)
    t_max = elapsed
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([elapsed], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_max = float(t.item())
    value = pairs_step * args.steps * world / t_max

    # FP64 kernel on the same workload (the 5x comparison)
    fp64_value = None
    if args.precision == "fp32c" and args.fp64_steps > 0:
        c64 = DeviceCloud.from_cloud(ctx, c0)
        c64.step(1, w.dt, "fp64")
        torch.cuda.synchronize()
        cloud_saved = cloud
        cloud = c64
        e64 = timed_steps("fp64", args.fp64_steps)
        cloud = cloud_saved
        fp64_value = pairs_step * args.fp64_steps / e64
        c64.close()

    # end to end through the public API with host buffers: pinned H2D of the
    # state, one RK4 step, D2H of the state, every step
    pin = [torch.empty(n, dtype=torch.float64, pin_memory=True) for _ in range(4)]
    hx = [p.numpy() for p in pin]
    st = cloud.download()
    for dst, src in zip(hx, st):
        dst[:] = src
    e2e_cloud = DeviceCloud.from_cloud(ctx, c0)
    e2e_cloud.upload(*hx)
    e2e_cloud.step(1, w.dt, args.precision)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        e2e_cloud.upload(*hx)
        e2e_cloud.step(1, w.dt, args.precision)
        e2e_cloud.download(out=hx)  # back into the same pinned buffers
    torch.cuda.synchronize()
    e2e_el = time.perf_counter() - t0
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([e2e_el], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_el = float(t.item())
    e2e_value = pairs_step * args.e2e_steps * world / e2e_el if args.e2e_steps > 0 else None

    # roofline of the dominant kernel (fused pair + stage, FP32 pipe bound)
    peak = ctx.probe_peak("fp32")
    avg_launch_s = pair_ms / 1e3 / max(launches, 1)
    achieved = FLOPS_PER_PAIR * n * (n - 1) / avg_launch_s / 1e12
    kname = "pair_stage_fp32c" if args.precision == "fp32c" else "pair_stage_fp64"
    swept_frac = swept / (pairs_step * args.steps) if swept > 0 else 1.0
    traffic = traffic_from_profiles(kname + ("_cull" if "cull" in tuned[0] else ""), w.name)

    # batched workload (256 clouds of uneven N, one persistent launch per stage)
    batch = None
    if args.batch_steps > 0:
        from demon_simulation_code_gb300 import DeviceBatch

        from demon_simulation_code_gb300.shard import assign_clouds, imbalance

        wb = W.batch256()
        # N > 1: whole clouds per rank, balanced by sum N^2 (no exchange)
        parts = assign_clouds([c.n for c in wb.clouds], world)
        bt = DeviceBatch(ctx, [wb.clouds[c] for c in parts[rank]])
        bt.step(4, wb.dt)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        ev0 = bt.evaluated_pairs()
        a.record(stream)
        bt.step(args.batch_steps, wb.dt)
        b.record(stream)
        torch.cuda.synchronize()
        el = a.elapsed_time(b) / 1e3
        bswept = bt.evaluated_pairs() - ev0
        if world > 1:
            import torch.distributed as dist

            t = torch.tensor([el], device="cuda", dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            el = float(t.item())
        name, nitems, grid = bt.info()
        batch = {"workload": wb.name, "value": 4.0 * wb.pairs_per_eval * args.batch_steps / el,
                 "unit": UNIT, "steps": args.batch_steps, "ms_per_step": el / args.batch_steps * 1e3,
                 "variant": name, "work_items": nitems, "persistent_grid": grid,
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
        from demon_simulation_code_gb300.fit import TrajectoryFit

        wa = W.adjoint64_smooth()
        fit = TrajectoryFit(wa, precision="fp32c")
        fit.loss_and_grad()  # warm-up
        torch.cuda.synchronize()
        l0 = fit.K.ctx.launch_count()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        a.record(stream)
        for _ in range(args.adjoint_grads):
            L, _ = fit.loss_and_grad()
        b.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        el = a.elapsed_time(b) / 1e3
        sweeps = (fit.K.ctx.launch_count() - l0) / args.adjoint_grads  # force + VJP launches per gradient
        adjoint = {"workload": wa.name, "clouds": len(fit.ns), "n": fit.ns[0], "steps": fit.steps,
                   "checkpoint_every": fit.every, "precision": "fp32c",
                   "seconds_per_gradient": el / args.adjoint_grads,
                   "wall_seconds_per_gradient": wall / args.adjoint_grads,
                   "pair_sweeps_per_gradient": sweeps,
                   "value": sweeps * fit.pairs_per_eval * args.adjoint_grads / el, "unit": UNIT,
                   "loss": float(L.item()), "gradients": "kappa, q, k_c per cloud; initial positions"}
        del fit

    cpu = None
    if rank == 0 and not args.no_cpu and args.cpu_steps > 0:
        threads = cpu_threads()
        rate, el = cpu_rk4_rate(w, args.cpu_steps, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{args.cpu_steps} RK4 steps of {w.name} (oracle/demon_oracle.c, "
                         f"OpenMP per-block locks as in the reference), {threads} threads, "
                         f"{el:.2f} s"}

    if rank == 0:
        res = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": t_max / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.precision == "fp32c" else "f64",
            "data": "synthetic (seeded generator, demon_simulation_code_gb300/workloads.py)",
            "config": config_of(w, args),
            "tuning": {"variant": tuned[0], "split": tuned[1]},
            "fp64_value": fp64_value,
            "fp32c_over_fp64": (value / world / fp64_value) if fp64_value else None,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 4 * 8 * n,
                    "d2h_bytes_per_step": 4 * 8 * n, "steps": args.e2e_steps},
            "step_ms_percentiles": {p: float(np.percentile(main_step_ms, q))
                                    for p, q in (("p10", 10), ("p50", 50), ("p90", 90), ("max", 100))},
            "gpu_launches": launches_timed,
            "roofline": {"bound": "fp32-pipe", "kernel": kname, "achieved": achieved,
                         "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                         "traffic": traffic,
                         "flops_per_pair": FLOPS_PER_PAIR,
                         "avg_launch_us": avg_launch_s * 1e6,
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
