"""Benchmark of the DG scalar-wave evolution hot path (grid-point RHS/s).

Workload (the configuration the metric is quoted on that fits one GPU):
ScalarWave first-order system on the periodic cube [0, 2pi]^3 split into
32^3 elements of 8^3 Legendre-Gauss-Lobatto points (16,777,216 points, 5 FP64
variables), Gaussian pulse psi = exp(-|x-c|^2/0.25), c = (pi, pi, pi),
UpwindPenalty correction, SSP-RK3 with dt = 2e-4.  One bench step = one
SSP-RK3 step over the whole grid = 3 right-hand-side evaluations of every
grid point.  Metric: grid-point RHS evaluations per second (points x 3 x
steps / time).

The state (671 MB per copy) is larger than L2 (129 MB), so no L2 flush is
done between timed steps.

`--impl reference` times the reference algorithm on the host CPU cores
instead: the FP64 C++ restatement in oracle/ (the reference executable
needs Charm++, Blaze, LIBXSMM and HDF5, none of which is in this image).

Multi-GPU: the path is run as independent replicas (one evolution per
rank, no collective); value = total grid-point RHS over all ranks / max time.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid-pt RHS/s FP64 vs batched mixed at <=1e-6 rel L2; adjoint s/grad"
UNIT = "grid-point RHS/s"
ELEMS = 32
N_PTS = 8
DT = 2e-4
# timed steps of the CPU baseline on the workload itself (about 10 s on 16 cores)
CPU_SAMPLE_STEPS = 10
# timed steps of the reference arm at most (the rest of --steps is not run)
REFERENCE_MAX_STEPS = 20
# Compulsory HBM bytes per grid point per stage launch.  Plain FP64: read
# ucur (40 B) + write unext (40 B) + read u0 on stages 2 and 3 (40 B).
BYTES_PER_POINT_LAUNCH = (80.0 + 120.0 + 120.0) / 3.0
# Mixed: stage 1 reads u0 (40 B) and writes d1 in FP32 (20 B); stage 2 reads
# d1 and writes s2 (20 + 20 B); stage 3 reads s2, d1 (FP32) and u0, and
# writes u (20 + 20 + 40 + 40 B).
MIXED_BYTES_PER_POINT_LAUNCH = (60.0 + 40.0 + 120.0) / 3.0
# DRAM traffic (read + write) per grid point per stage launch measured by ncu
# on the 20^3 x 8^3 case (4,096,000 points): 287.7, 470.1 and 452.9 MB for the
# three FP64 stages; 180.5 + 120.3 + 204.1 + 355.4 MB for the three mixed
# stages and the FP64 accumulate, per three stage launches.
# Traffic grows with the points, so the 32^3 figure is this times its points.
FP64_TRAFFIC_PER_POINT_LAUNCH = 1210.7e6 / 3 / 4096000
MIXED_TRAFFIC_PER_POINT_LAUNCH = 860.3e6 / 3 / 4096000
# FP64 pipe instructions per point per stage of the plain kernel at N = 8
# (even/odd contraction 6 per derivative x 6, dt Pi sum 2, RK update 5-11,
# face corrections ~3.75); the ncu capture of the 20^3 case measured
# 42.7 / 47.6 / 47.6 per point for the three stages.
FP64_INST_PER_POINT_STAGE = 46.0
# DFMA / DADD throughput measured on this machine's GB300 (0.505 T inst/s)
FP64_PEAK_TINST = 0.505


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region.

    Every line is stamped when it arrives; with begin() / end() marking the
    timed region, only the lines stamped inside it count (all lines when
    none is)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.device_index = device_index
        self.proc = None
        self.lines = []
        self.thread = None
        self.window = [None, None]

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device_index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def begin(self):
        self.window[0] = time.perf_counter()

    def end(self):
        self.window[1] = time.perf_counter()

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lo, hi = self.window
        lines = [ln for t, ln in self.lines
                 if lo is not None and hi is not None and lo <= t <= hi]
        in_window = bool(lines)
        if not lines:
            lines = [ln for _, ln in self.lines]
        for ln in lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm),
                "window": "timed region" if in_window else "whole sampler run"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, ws):
    """The largest of each rank's x (seconds or ms): the job's time is set by
    the slowest replica.  All-reduce on the process group's own device type
    (CUDA tensors under NCCL, CPU tensors under gloo)."""
    if ws <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(points_per_rank, rhs_per_step, steps, seconds_per_rank, ws):
    """Whole-job grid-point RHS/s of ws independent replicas (weak scaling):
    all ranks' point-RHS over the slowest rank's time."""
    slowest = max_over_ranks(seconds_per_rank, ws)
    return points_per_rank * rhs_per_step * steps * ws / slowest, slowest


def host_link_rates(host, dev):
    """GB/s of whole-state copies between the pinned host buffer and the
    device, measured beside the e2e run: host->device alone, device->host
    alone, and both at once on two streams (half the state each way; each
    the mean of 3 rounds).  The host link is shared with whatever else the
    host runs, so the e2e figure moves with it."""
    import torch
    d = torch.empty(host.numel(), dtype=host.dtype, device=dev)
    nbytes = host.numel() * host.element_size()
    half = host.numel() // 2
    s1, s2 = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    out = {}
    for name in ("h2d", "d2h", "both"):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(3):
            if name == "h2d":
                d.copy_(host, non_blocking=True)
            elif name == "d2h":
                host.copy_(d, non_blocking=True)
            else:  # one half in, the other half out, at once
                with torch.cuda.stream(s1):
                    d[:half].copy_(host[:half], non_blocking=True)
                with torch.cuda.stream(s2):
                    host[half:].copy_(d[half:], non_blocking=True)
        torch.cuda.synchronize(dev)
        out[name] = 3 * nbytes / (time.perf_counter() - t0) / 1e9
    del d
    return out


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


_FAST_OK = None


def cpu_fast_ok():
    """Whether the speed build of the oracle runs on this host: a small
    evolution in a child process (a CPU that lacks an instruction the build
    uses ends that process, not the bench)."""
    global _FAST_OK
    if _FAST_OK is None:
        import subprocess
        code = ("import sys; sys.path.insert(0, %r); from oracle import pyoracle; "
                "from spectre_gb300.dgsw import Brick; b = [Brick((2, 2, 2))]; "
                "u = pyoracle.initial_data(b, 4, 'plane_wave', [1.0, 1.0, 1.0]); "
                "pyoracle.evolve(b, 4, u, 1e-3, 2, fast=True)" % ROOT)
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, timeout=300)
        _FAST_OK = r.returncode == 0
    return _FAST_OK


def cpu_flags():
    from oracle import pyoracle
    if not cpu_fast_ok():
        return "the portable checker flags (the speed build does not run on this host)"
    try:
        return pyoracle.fast_build_flags()
    except Exception:
        return "unknown flags"


def cpu_reference_run(steps, warmup, threads, elems=None):
    """Times the FP64 oracle (C++ restatement of the reference) on host cores.

    The sample is the workload itself (the 32^3-element brick of N = 8 LGL
    points, the same initial data): `warmup` untimed steps, then `steps`
    SSP-RK3 steps timed in one call.
    """
    from oracle import pyoracle
    from spectre_gb300.dgsw import Brick
    elems = elems or ELEMS
    bricks = [Brick((elems, elems, elems))]
    params = pyoracle.gaussian_params(1, amp=1.0, width=0.5)
    u = pyoracle.initial_data(bricks, N_PTS, "gaussian", params)
    points = elems ** 3 * N_PTS ** 3
    if warmup:
        u = pyoracle.evolve(bricks, N_PTS, u, DT, warmup, threads=threads, fast=cpu_fast_ok())
    t0 = time.perf_counter()
    u = pyoracle.evolve(bricks, N_PTS, u, DT, steps, threads=threads, fast=cpu_fast_ok())
    el = time.perf_counter() - t0
    return points * 3 * steps / el, el, points


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    threads = cpu_threads()
    # a bounded sample: one SSP-RK3 step of the workload takes about 1 s on 16
    # host cores, so at most REFERENCE_MAX_STEPS of the requested steps run
    steps = max(1, min(args.steps, REFERENCE_MAX_STEPS))
    value, el, points = cpu_reference_run(steps, min(args.warmup, 1), threads)
    sample = ("FP64 C++ restatement of the reference (oracle/, built with %s) on the "
              "workload itself, 32^3 elements x 8^3 LGL points (%d points), %d SSP-RK3 steps, "
              "%d threads, %.1f s" % (cpu_flags(), points, steps, threads, el))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup,
        "ms_per_step": el / steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(elems=ELEMS):
    return {"workload": "ScalarWave %d^3 elements x 8^3 LGL points periodic [0,2pi]^3, "
                        "Gaussian pulse, UpwindPenalty, SSP-RK3 dt=2e-4" % elems,
            "elements": elems ** 3, "points_per_dim": N_PTS,
            "grid_points": elems ** 3 * N_PTS ** 3, "variables": 5, "dt": DT,
            "precision": "plain FP64", "l2": "inputs larger than L2 (671 MB state), no flush"}


def time_path(args, precision, dev, rank, ws, sample_clocks):
    """Times args.steps SSP-RK3 steps of one precision; returns the numbers
    and the final state (host copy)."""
    import torch
    from spectre_gb300 import Brick, DgEvolution, PRECISION_MIXED
    bricks = [Brick((args.elements, args.elements, args.elements))]
    params = np.array([[1.0, 0.5, math.pi, math.pi, math.pi]])
    ev = DgEvolution(bricks, N_PTS, precision=precision, device=dev)
    ev.set_initial_data("gaussian", params)
    if precision == PRECISION_MIXED and args.mixed_variant >= 0:
        ev.tune(force_variant=args.mixed_variant)
    stream = torch.cuda.ExternalStream(ev.stream_ptr(), device=dev)
    warm = max(args.warmup, 3)
    for _ in range(warm):
        ev.step(1, DT, sync=False)
    ev.synchronize()
    sampler = ClockSampler(dev) if (rank == 0 and sample_clocks) else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if sampler:
        sampler.begin()
    e0.record(stream)
    ev.step(args.steps, DT, sync=False)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    if sampler:
        sampler.end()
    ms = e0.elapsed_time(e1)
    if ws > 1:
        ms = max_over_ranks(ms, ws)
        torch.distributed.barrier()
    clocks = sampler.stop() if sampler else None
    state = ev.get_state()
    return ev, ms, clocks, state, warm


def time_batched(args, dev):
    """The batched case: 256 independent evolutions, per-element LGL extents in
    {4..10}, p-nonconforming mortars, Gaussian pulses; FP64 and mixed, and
    the worst per-instance rel L2 of mixed against FP64 after the same steps."""
    import torch
    from spectre_gb300 import DgEvolution, PRECISION_FP64, PRECISION_MIXED, workloads
    bricks, pts, params = workloads.batched_instances(256, seed=2024)
    dt = 1e-4
    steps = max(1, min(args.steps, 20))
    res = {}
    states = {}
    paths = (("fp64", PRECISION_FP64), ("mixed", PRECISION_MIXED))
    only = getattr(args, "batched_precision", "both")
    if only != "both":
        paths = tuple(p for p in paths if p[0] == only)
    for name, prec in paths:
        ev = DgEvolution(bricks, pts, precision=prec, device=dev)
        ev.set_initial_data("gaussian", params)
        for _ in range(max(1, args.warmup)):
            ev.step(1, dt, sync=False)
        ev.synchronize()
        stream = torch.cuda.ExternalStream(ev.stream_ptr(), device=dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        ev.step(steps, dt, sync=False)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        states[name] = ev.get_state()
        res[name] = {"value": ev.grid_points * 3 * steps / (ms * 1e-3), "unit": UNIT,
                     "ms_per_step": ms / steps}
        points = ev.grid_points
        n_elem = ev.n_elements
        if name == "mixed":
            # launch shape the autotuner chose, re-timed after the timed region
            res[name]["tune"] = ev.tune()
            hbm = load_peaks()[0].get("hbm_gbs")
            gbs = MIXED_BYTES_PER_POINT_LAUNCH * points / (ms / (3 * steps) * 1e-3) / 1e9
            res[name]["roofline"] = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                                     "frac": gbs / hbm if hbm else None,
                                     "bytes_per_point_launch": MIXED_BYTES_PER_POINT_LAUNCH,
                                     "note": "algorithmic bytes per grid point and stage "
                                             "launch ÷ the step's mean time per stage"}
        ev.close()
    out = {"workload": "256 periodic ScalarWave evolutions on [0,2pi]^3, elements per axis "
                       "U{2..8}, LGL points per element U{4..10} (p-nonconforming mortars), "
                       "Gaussian pulses, SSP-RK3 dt=1e-4, seed 2024",
           "grid_points": points, "elements": n_elem, "steps": steps}
    out.update(res)
    if len(states) < 2:
        return out
    # per-instance relative L2 of mixed vs FP64 after warm-up + timed steps
    worst = 0.0
    off = 0
    e = 0
    for b in bricks:
        ne = b.elements[0] * b.elements[1] * b.elements[2]
        size = int(5 * np.sum(np.asarray(pts[e:e + ne], dtype=np.int64) ** 3))
        a = states["fp64"][off:off + size]
        m = states["mixed"][off:off + size]
        worst = max(worst, float(np.linalg.norm(m - a) / np.linalg.norm(a)))
        off += size
        e += ne
    out.update({"mixed_speedup_vs_fp64": res["fp64"]["ms_per_step"] / res["mixed"]["ms_per_step"],
                "max_instance_rel_l2_mixed_vs_fp64": worst,
                "steps_compared": max(1, args.warmup) + steps})
    if not getattr(args, "no_full_length", False):
        out["full_length"] = batched_full_length(bricks, pts, params, dev)
    return out


def instance_rel_l2(bricks, pts, a, b):
    """Per-instance relative L2 of b against a."""
    errs = []
    off = 0
    e = 0
    for br in bricks:
        ne = br.elements[0] * br.elements[1] * br.elements[2]
        size = int(5 * np.sum(np.asarray(pts[e:e + ne], dtype=np.int64) ** 3))
        errs.append(float(np.linalg.norm(b[off:off + size] - a[off:off + size])
                          / np.linalg.norm(a[off:off + size])))
        off += size
        e += ne
    return errs


def batched_full_length(bricks, pts, params, dev, steps=300, dt=1e-4):
    """The 256-instance case over its configured 300 steps from the initial
    data: per-instance relative L2 of the mixed path against the FP64 path."""
    from spectre_gb300 import DgEvolution, PRECISION_FP64, PRECISION_MIXED
    states = {}
    for name, prec in (("fp64", PRECISION_FP64), ("mixed", PRECISION_MIXED)):
        with DgEvolution(bricks, pts, precision=prec, device=dev) as ev:
            ev.set_initial_data("gaussian", params)
            ev.step(steps, dt)
            states[name] = ev.get_state()
    errs = instance_rel_l2(bricks, pts, states["fp64"], states["mixed"])
    return {"steps": steps, "dt": dt, "max_instance_rel_l2_mixed_vs_fp64": max(errs),
            "median_instance_rel_l2_mixed_vs_fp64": float(np.median(errs))}


def config2_full_length(dev, steps=500):
    """The 32^3 x 8^3 Gaussian case over its configured 500 steps: relative L2
    of the mixed path against the FP64 path."""
    from spectre_gb300 import Brick, DgEvolution, PRECISION_FP64, PRECISION_MIXED
    params = np.array([[1.0, 0.5, np.pi, np.pi, np.pi]])
    states = {}
    for name, prec in (("fp64", PRECISION_FP64), ("mixed", PRECISION_MIXED)):
        with DgEvolution([Brick((ELEMS, ELEMS, ELEMS))], N_PTS, precision=prec, device=dev) as ev:
            ev.set_initial_data("gaussian", params)
            ev.step(steps, DT)
            states[name] = ev.get_state()
    a, m = states["fp64"], states["mixed"]
    return {"steps": steps, "dt": DT,
            "rel_l2_mixed_vs_fp64": float(np.linalg.norm(m - a) / np.linalg.norm(a))}


def _time_gradient(p, psi0, reps=3):
    """(J, gradient, s per gradient, s per forward misfit run) of a MisfitProblem."""
    import torch
    p.value_and_gradient(psi0)  # warm-up (tuning, graph capture)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        J, g = p.value_and_gradient(psi0)
    torch.cuda.synchronize()
    s_per_grad = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        p.value(psi0)
    torch.cuda.synchronize()
    return J, g, s_per_grad, (time.perf_counter() - t0) / reps


def time_adjoint(dev, steps=2000):
    """The adjoint case: 8^3 elements x 8^3 points, dt 5e-4, 2000 SSP-RK3 steps, 64
    samples every 10 steps; seconds per gradient (forward misfit run + the
    discrete adjoint sweep) in FP64 and in mixed precision (FP64 states, FP32
    increments), with central-difference checks against the FP64 objective
    and tangent-linear checks along seeded directions, and the mixed
    gradient's error against the FP64 one."""
    import torch
    from spectre_gb300.adjoint import MisfitProblem
    p = MisfitProblem(device=dev, steps=steps)
    pm = MisfitProblem(device=dev, steps=steps, precision="mixed")
    try:
        psi0 = p.initial_psi()
        J, g, s_grad, s_fwd = _time_gradient(p, psi0)
        Jm, gm, s_grad_m, s_fwd_m = _time_gradient(pm, psi0)
        split, split_ms = p.ev.adjoint_autotune()
        stage_variant, stage_ms = p.ev.autotune()
        rng = torch.Generator(device="cuda").manual_seed(11)
        eps = 1e-6
        fd_err = fd_err_m = 0.0
        for _ in range(2):
            v = torch.randn(psi0.shape, dtype=torch.float64, device="cuda", generator=rng)
            fd = (p.value(psi0 + eps * v) - p.value(psi0 - eps * v)) / (2 * eps)
            fd_err = max(fd_err, abs(fd - float(torch.sum(g * v))) / abs(fd))
            fd_err_m = max(fd_err_m, abs(fd - float(torch.sum(gm * v))) / abs(fd))
        v = torch.randn(psi0.shape, dtype=torch.float64, device="cuda", generator=rng)
        tl = p.tangent_linear(psi0, v)
        tl_err = abs(tl - float(torch.sum(g * v))) / abs(tl)
        tl_err_m = abs(tl - float(torch.sum(gm * v))) / abs(tl)
        mixed_max = float((gm - g).abs().max()) / float(g.abs().max())
        mixed_l2 = float(torch.linalg.norm(gm - g)) / float(torch.linalg.norm(g))
        return {"workload": "ScalarWave 8^3 elements x 8^3 LGL points, SSP-RK3 dt=5e-4, "
                            "%d steps, 64 seeded samples of Psi every 10 steps; control Psi(t=0)"
                            % steps,
                "s_per_grad": s_grad_m, "s_per_grad_precision": "mixed",
                "fp64": {"s_per_grad": s_grad, "s_forward": s_fwd,
                         "s_adjoint_sweep": s_grad - s_fwd, "J": J,
                         "fd_max_rel_err_2_dirs": fd_err, "tangent_linear_rel_err": tl_err,
                         "forward_stage_variant": stage_variant,
                         "forward_ms_per_stage_variants": [float(x) for x in stage_ms],
                         "adjoint_split": split,
                         "adjoint_ms_per_launch_splits": [float(x) for x in split_ms]},
                "mixed": {"s_per_grad": s_grad_m, "s_forward": s_fwd_m,
                          "s_adjoint_sweep": s_grad_m - s_fwd_m, "J": Jm,
                          "J_rel_err_vs_fp64": abs(Jm - J) / abs(J),
                          "grad_max_rel_err_vs_fp64": mixed_max,
                          "grad_l2_rel_err_vs_fp64": mixed_l2,
                          "fd_max_rel_err_2_dirs": fd_err_m,
                          "tangent_linear_rel_err": tl_err_m,
                          "speedup_vs_fp64": s_grad / s_grad_m},
                "note": "forward misfit run + hand-written discrete adjoint sweep; the step "
                        "map is linear, so no forward states are stored.  FP64: 3 L^T launches "
                        "per step (reverse SSP-RK3 stages).  Mixed: both sweeps as the step's "
                        "Taylor polynomial, W1 = dt L u, W2 = dt L W1, W3 = dt L W2, "
                        "u += W1 + W2/2 + W3/6 (L^T backwards), FP64 states and double-float "
                        "increments formed in FP32 arithmetic (taylor_df.cu). "
                        "Central differences and the tangent-linear run use the FP64 "
                        "objective."}
    finally:
        p.close()
        pm.close()


def time_curved_adams(shell, n, dt, steps, dev):
    """The shell stepped as the reference's curved executable steps it:
    AdamsBashforth(3), global stepping at dt, and local time stepping with
    the slab 4 dt and the radial layers on levels by element size (the
    logarithmic radial map makes the inner layers smallest: layers 0-1 step
    dt, 2-4 2 dt, 5-7 4 dt).  Both cover the same simulated time."""
    import torch
    from spectre_gb300.dgsw import CurvedDgEvolution, PRECISION_FP64, PRECISION_MIXED
    E = 768
    layer = np.arange(E) % 8  # radial segment: the innermost index of a wedge's elements
    levels = np.where(layer < 2, 2, np.where(layer < 5, 1, 0)).astype(np.int32)
    res, states = {}, {}
    nl = max(1, steps // 4)
    for name, lv, slab, slabs, filt, prec in (
            ("gts", None, dt, steps, False, PRECISION_FP64),
            ("lts", levels, 4 * dt, nl, False, PRECISION_FP64),
            ("lts_filtered", levels, 4 * dt, nl, True, PRECISION_FP64),
            ("gts_mixed", None, dt, steps, False, PRECISION_MIXED),
            ("lts_filtered_mixed", levels, 4 * dt, nl, True, PRECISION_MIXED)):
        ev = CurvedDgEvolution(shell, n, precision=prec, gamma2=1.0, device=dev,
                               time_stepper="adams_bashforth", order=3, step_levels=lv)
        if filt:
            # the executable's step actions end with the filter on every element
            ev.set_exponential_filter(36.0, 8)
        ev.set_gaussian_shell(1.0, 8.0, 1.0)
        u0 = ev.get_state()
        ev.step(2, slab)  # start-up and switch
        ev.set_state(u0)  # time the whole run from t = 0, start-up included
        stream = torch.cuda.ExternalStream(ev.stream_ptr(), device=dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        ev.step(slabs, slab, sync=False)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        info = ev.adams_info()
        states[name] = ev.get_state()
        res[name] = {"value": info["rhs_points_per_slab"] * slabs / (ms * 1e-3), "unit": UNIT,
                     "ms_per_unit_time": ms / (slabs * slab), "slab": slab, "slabs": slabs,
                     "launches_per_slab": 2 * info["launches_per_slab"]}
        ev.close()
    res["lts_filtered"]["filter"] = "Filters::Exponential alpha=36, half_power=8, after every element step"
    res["lts_speedup_vs_gts"] = res["gts"]["ms_per_unit_time"] / res["lts"]["ms_per_unit_time"]
    for m, f in (("gts_mixed", "gts"), ("lts_filtered_mixed", "lts_filtered")):
        res[m]["speedup_vs_fp64"] = res[f]["ms_per_unit_time"] / res[m]["ms_per_unit_time"]
        res[m]["rel_l2_vs_fp64"] = float(np.linalg.norm(states[m] - states[f]) /
                                         np.linalg.norm(states[f]))
    a, b = states["gts"], states["lts"]
    res["max_abs_lts_vs_gts"] = float(np.abs(a - b).max())
    res["note"] = ("AdamsBashforth(3); value counts each element's own steps; the start-up "
                   "(self-start at dt/3 resp. the finest step / 3) is inside the timed run")
    return res


def time_curved(args, dev, with_cpu):
    """The curved case: CurvedScalarWave on Schwarzschild in Kerr-Schild coordinates
    (M = 1, gamma1 = 0, gamma2 = 1), six-wedge shell r in [1.9, 20], 4 x 4
    angular x 8 radial elements per wedge (768), logarithmic radial map, 10^3
    LGL points per element, Gaussian shell Psi = exp(-(r-8)^2), excision
    inside the horizon and the constraint-preserving radiation condition
    outside; SSP-RK3 dt = 1e-3 for 1000 steps, plain FP64 and mixed."""
    import torch
    from oracle import pyoracle
    from spectre_gb300.dgsw import (CurvedDgEvolution, PRECISION_FP64, PRECISION_MIXED,
                                    Shell)
    shell = Shell(1.9, 20.0, 2, 3, "logarithmic", 1.0, 0.0)
    n, dt = 10, 1e-3
    steps = 1000 if not args.curved_steps else args.curved_steps
    res, states = {}, {}
    for name, prec in (("fp64", PRECISION_FP64), ("mixed", PRECISION_MIXED)):
        ev = CurvedDgEvolution(shell, n, precision=prec, gamma2=1.0, device=dev)
        ev.set_gaussian_shell(1.0, 8.0, 1.0)
        if prec == PRECISION_MIXED and args.curved_variant >= 0:
            ev.tune(force_variant=args.curved_variant)
        u0 = ev.get_state()
        # warm-up: graphs captured, then the state reset to t = 0
        ev.step(16, dt)
        ev.step(1, dt)
        ev.set_state(u0)
        stream = torch.cuda.ExternalStream(ev.stream_ptr(), device=dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        ev.step(steps, dt, sync=False)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        states[name] = ev.get_state()
        res[name] = {"value": ev.grid_points * 3 * steps / (ms * 1e-3), "unit": UNIT,
                     "ms_per_step": ms / steps}
        points = ev.grid_points
        if name == "mixed":
            # the launch shape the tuner chose, re-timed after the timed region
            res["mixed"]["tune"] = ev.tune()
        if name == "fp64":
            # FP64 against the oracle over the first steps
            k = 3
            ev.set_state(u0)
            ev.step(k, dt)
            s_orc = pyoracle.shell(1.9, 20.0, 2, 3, n, 1.0, 0.0, 1.0)
            ref, _ = pyoracle.shell_evolve(s_orc, u0.reshape(-1, 5, n ** 3), dt, k,
                                           threads=cpu_threads())
            got = ev.get_state().reshape(ref.shape)
            res["fp64"]["max_rel_err_vs_oracle_%d_steps" % k] = float(
                max(np.abs(got[:, v] - ref[:, v]).max() / np.abs(ref[:, v]).max()
                    for v in range(5)))
        ev.close()
    a, m = states["fp64"], states["mixed"]
    out = {"workload": "CurvedScalarWave, Kerr-Schild M=1 (gamma1=0, gamma2=1), 6-wedge shell "
                       "r in [1.9,20], 4x4x8 elements per wedge (768), log radial map, 10^3 "
                       "LGL points, Gaussian shell Psi=exp(-(r-8)^2), excision + CPSR, "
                       "SSP-RK3 dt=1e-3",
           "grid_points": points, "steps": steps, "fp64": res["fp64"], "mixed": res["mixed"],
           "mixed_speedup_vs_fp64": res["fp64"]["ms_per_step"] / res["mixed"]["ms_per_step"],
           "rel_l2_mixed_vs_fp64_after_steps": float(np.linalg.norm(m - a) / np.linalg.norm(a)),
           "max_abs_mixed_vs_fp64": float(np.abs(m - a).max())}
    out["adams"] = time_curved_adams(shell, n, dt, steps, dev)
    out["filtered"] = time_curved_filtered(shell, n, dt, steps, dev)
    if with_cpu:
        s_orc = pyoracle.shell(1.9, 20.0, 2, 3, n, 1.0, 0.0, 1.0)
        u = pyoracle.shell_initial_data(s_orc, 8.0, 1.0)
        threads = cpu_threads()
        pyoracle.shell_rhs(s_orc, u, threads=threads, fast=cpu_fast_ok())
        t0 = time.perf_counter()
        reps = 2
        for _ in range(reps):
            pyoracle.shell_rhs(s_orc, u, threads=threads, fast=cpu_fast_ok())
        el = (time.perf_counter() - t0) / reps
        out["cpu_baseline"] = {"value": points / el, "unit": UNIT, "cores": threads,
                               "kind": "port",
                               "sample": "oracle curved RHS of the full shell (built with %s), "
                                         "%d evaluations, %.2f s each (includes its geometry "
                                         "set-up)" % (cpu_flags(), reps, el)}
    return out


def time_curved_filtered(shell, n, dt, steps, dev):
    """The curved case with the exponential filter (alpha 36, half power 8)
    after every substep, as the reference's curved executable applies it:
    FP64 and mixed over the same steps, and their rel L2 difference."""
    import torch
    from spectre_gb300.dgsw import CurvedDgEvolution, PRECISION_FP64, PRECISION_MIXED
    res, states = {}, {}
    for name, prec in (("fp64", PRECISION_FP64), ("mixed", PRECISION_MIXED)):
        with CurvedDgEvolution(shell, n, precision=prec, gamma2=1.0, device=dev) as ev:
            ev.set_exponential_filter(36.0, 8)
            ev.set_gaussian_shell(1.0, 8.0, 1.0)
            u0 = ev.get_state()
            ev.step(16, dt)
            ev.step(1, dt)
            ev.set_state(u0)
            stream = torch.cuda.ExternalStream(ev.stream_ptr(), device=dev)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            ev.step(steps, dt, sync=False)
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            states[name] = ev.get_state()
            res[name] = {"value": ev.grid_points * 3 * steps / (ms * 1e-3), "unit": UNIT,
                         "ms_per_step": ms / steps}
    a, m = states["fp64"], states["mixed"]
    res["filter"] = "Filters::Exponential alpha=36, half_power=8, after every substep"
    res["steps"] = steps
    res["mixed_speedup_vs_fp64"] = res["fp64"]["ms_per_step"] / res["mixed"]["ms_per_step"]
    res["rel_l2_mixed_vs_fp64_after_steps"] = float(np.linalg.norm(m - a) / np.linalg.norm(a))
    return res


def ab_bytes_per_point(order, n):
    """Compulsory HBM bytes per grid point of one AdamsBashforth launch of an
    element (update + record, global stepping): read u and `order` recorded
    time derivatives, write u and the new record (5 FP64 vars each); of the
    face records (12 n^2 values per element: both w's of six faces) read
    `order` (each value once: its element reads one w, the neighbour the
    other) and write one."""
    vol = (5 + 5 * order + 5 + 5) * 8.0
    faces = (12 * order + 12) * n * n * 8.0 / n ** 3
    return vol + faces


# FP64 thread instructions per grid point of one AB3 launch at N = 8 (update
# + record): DFMA 156.7M + DADD 76.8M + DMUL 30.0M per launch on the 20^3 x
# 8^3 case (ncu sass op counters, 4,096,000 points)
AB3_FP64_INST_PER_POINT = (156.672e6 + 76.8e6 + 30.048e6) / 4096000
# DRAM read + write per launch of that capture, per point
AB3_TRAFFIC_PER_POINT = (814.1e6 + 415.1e6) / 4096000


def time_next_rows(args, dev):
    """The rows built around the path, each timed once at the 32^3 x 8^3 size
    (or the refined lattice below) with CUDA events on the handle's stream:
    Gauss-point quadrature, an h-refined lattice with 2:1 faces, ObserveNorms,
    the exponential filter on the flat path, and the AMR p-projection of every
    element.  Achieved GB/s are algorithmic bytes / time."""
    import torch
    from spectre_gb300 import Brick, DgEvolution
    from spectre_gb300.dgsw import RefinedBrick, amr_project
    E = args.elements
    params = np.array([[1.0, 0.5, math.pi, math.pi, math.pi]])
    res = {}

    def timed(ev, fn, reps):
        stream = torch.cuda.ExternalStream(ev.stream_ptr(), device=dev)
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    steps = 20
    with DgEvolution([Brick((E, E, E))], N_PTS, device=dev) as ev:
        ev.set_initial_data("gaussian", params)
        ms_gll = timed(ev, lambda: ev.step(steps, DT, sync=False), 1) / steps
        pts = ev.grid_points
        ev.set_exponential_filter(36.0, 8)
        ms_f = timed(ev, lambda: ev.step(steps, DT, sync=False), 1) / steps
        ev.set_exponential_filter(36.0, 8, enable=False)
        # ObserveNorms of the state: one reduction launch pair and the
        # 27-value result copied to the host
        ms_norms = timed(ev, lambda: ev.observe_norms(), 10)
        # AMR p-projection of every element 8 -> 9 (ProjectVariables)
        st = torch.from_numpy(ev.get_state()).to("cuda:%d" % dev)
        ne = ev.n_elements
        src = np.arange(ne, dtype=np.int32)
        se = np.full((ne, 3), N_PTS, np.int32)
        de = np.full((ne, 3), N_PTS + 1, np.int32)
        ch = np.zeros((ne, 3), np.int8)
        ino = np.arange(ne, dtype=np.int64) * 5 * N_PTS ** 3
        ms_amr = timed(ev, lambda: amr_project(ev, 5, st, ino, src, se, de, ch), 3)
        amr_bytes = ne * 5 * (N_PTS ** 3 + (N_PTS + 1) ** 3) * 8
    filt_app = (ms_f - ms_gll) / 3
    res["gll_fp64_ms_per_step"] = ms_gll
    res["exponential_filter"] = {
        "ms_per_application": filt_app,
        "achieved_gbs": 80.0 * pts / (filt_app * 1e-3) / 1e9 if filt_app > 0 else None,
        "note": "Filters::Exponential alpha=36 half_power=8 after every substep on the FP64 "
                "path; cost = (filtered step - plain step) / 3; 80 B per point algorithmic"}
    res["observe_norms"] = {
        "ms_per_call": ms_norms,
        "achieved_gbs": 40.0 * pts / (ms_norms * 1e-3) / 1e9,
        "note": "Max, Min, L2Norm, L2IntegralNorm, VolumeIntegral of the five variables, "
                "result on the host; 40 B per point read"}
    res["amr_p_projection"] = {
        "ms": ms_amr, "achieved_gbs": amr_bytes / (ms_amr * 1e-3) / 1e9,
        "note": "amr::projectors::ProjectVariables p-refinement 8 -> 9 of every element "
                "(read 8^3, write 9^3 values x 5 variables)"}
    with DgEvolution([Brick((E, E, E))], N_PTS, device=dev, quadrature="gauss") as ev:
        ev.set_initial_data("gaussian", params)
        ms_g = timed(ev, lambda: ev.step(steps, DT, sync=False), 1) / steps
        res["gauss_quadrature"] = {
            "value": ev.grid_points * 3 / (ms_g * 1e-3), "unit": UNIT, "ms_per_step": ms_g,
            "vs_gll": ms_gll / ms_g,
            "workload": "%d^3 elements x %d^3 Legendre-Gauss points, FP64, SSP-RK3" % (E, N_PTS)}
    # 4 x 4 x 4 blocks, checkerboard levels 2 / 3 (every face 2:1)
    lv = [2 + ((i + j + k) % 2) for k in range(4) for j in range(4) for i in range(4)]
    with DgEvolution(RefinedBrick((4, 4, 4), lv), N_PTS, device=dev) as ev:
        ev.set_initial_data("gaussian", params)
        ms_r = timed(ev, lambda: ev.step(steps, DT, sync=False), 1) / steps
        res["h_refined"] = {
            "value": ev.grid_points * 3 / (ms_r * 1e-3), "unit": UNIT, "ms_per_step": ms_r,
            "elements": ev.n_elements,
            "workload": "4^3 blocks, levels 2/3 in a checkerboard (2:1 mortars on every block "
                        "face), %d^3 LGL points, FP64, SSP-RK3" % N_PTS}
    return res


def time_adams(args, dev):
    """AdamsBashforth(3) on the 32^3-element mesh (8^3 points,
    Gaussian pulse, slab = step = 2e-4): global stepping, and local time
    stepping with half of the elements (seeded) on level 1 (two steps of
    1e-4 per slab).  The start-up runs in the warm-up; the timed slabs are
    steady-state AB3.  One launch per tick position."""
    import torch
    from spectre_gb300.dgsw import Brick, DgEvolution
    e = args.elements
    bricks = [Brick((e, e, e), (0.0, 0.0, 0.0), (2 * math.pi,) * 3)]
    slabs = max(10, args.steps * 2)
    out = {"workload": "AdamsBashforth(3), %d^3 elements x %d^3 LGL points, Gaussian pulse, "
                       "slab %.0e" % (e, N_PTS, DT), "slabs": slabs}
    rng = np.random.default_rng(7)
    for name, levels in (("gts", None), ("lts_2to1", rng.integers(0, 2, size=e ** 3))):
        ev = DgEvolution(bricks, N_PTS, device=dev, time_stepper="adams_bashforth", order=3,
                         step_levels=levels)
        ev.set_initial_data("gaussian", [1.0, 0.5, math.pi, math.pi, math.pi])
        ev.step(4, DT)  # self-start + switch + steady slabs
        info = ev.adams_info()
        stream = torch.cuda.ExternalStream(ev.stream_ptr(), device=dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        ev.step(slabs, DT, sync=False)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        pts = info["rhs_points_per_slab"]
        launches = info["launches_per_slab"] * slabs
        r = {"value": pts * slabs / (ms * 1e-3), "unit": UNIT, "ms_per_slab": ms / slabs,
             "gpu_launches": launches, "ring_slots": info["ring_slots"],
             "rhs_points_per_slab": pts}
        if name == "gts":
            bpp = ab_bytes_per_point(3, N_PTS)
            gbs = bpp * pts * slabs / (ms * 1e-3) / 1e9
            r["roofline"] = {"bound": "hbm", "achieved": gbs, "unit": "GB/s",
                             "bytes_per_point_launch": bpp, "avg_launch_ms": ms / launches,
                             "traffic": AB3_TRAFFIC_PER_POINT * pts,
                             "traffic_note": "ncu DRAM bytes per launch, 20^3 capture scaled "
                                             "by points"}
            inst = AB3_FP64_INST_PER_POINT * pts * slabs / (ms * 1e-3) / 1e12
            r["fp64_pipe"] = {"achieved_tinst_s": inst, "peak_tinst_s": FP64_PEAK_TINST,
                              "frac": inst / FP64_PEAK_TINST,
                              "inst_per_point_launch": AB3_FP64_INST_PER_POINT,
                              "note": "the FP64 pipe binds this kernel"}
        else:
            r["elements_per_level"] = [int((levels == 0).sum()), int((levels == 1).sum())]
        out[name] = r
        ev.close()
    return out


def run_ours(args):
    import torch
    from spectre_gb300 import PRECISION_FP64, PRECISION_MIXED
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = local if ws > 1 else 0
    torch.cuda.set_device(dev)
    peaks, peak_kind = load_peaks()
    hbm = peaks.get("hbm_gbs")

    ev, ms, clocks, state64, warm = time_path(args, PRECISION_FP64, dev, rank, ws, True)
    points = ev.grid_points
    # the launch configuration the autotuner chose for the timed FP64 stages,
    # re-timed here after the timed region
    tuned_variant, tuned_ms = ev.autotune()
    autotune = {"stage_variant": tuned_variant,
                "ms_per_launch_variants": [float(x) for x in tuned_ms]}
    value = points * 3 * args.steps * ws / (ms * 1e-3)
    launch_ms = ms / (3 * args.steps)
    achieved_gbs = BYTES_PER_POINT_LAUNCH * points / (launch_ms * 1e-3) / 1e9

    # end to end through the C ABI with pinned host buffers: every step reads
    # the state from host memory and writes the new state back
    # (dgsw_step_host: the copies overlap the step chunk by chunk)
    host = torch.empty(ev.state_size, dtype=torch.float64, pin_memory=True)
    hnp = host.numpy()
    ev.get_state(hnp)
    k2 = max(1, min(args.steps, 20))
    # warm-up calls as for the device-timed region (the first also sets up
    # the chunk schedule, streams and graphs)
    for _ in range(max(args.warmup, 3)):
        ev.step_host(hnp, 1, DT)
    torch.cuda.synchronize()
    import gc
    gc.collect()
    gc.disable()  # no collector pauses inside the timed calls
    stream = torch.cuda.ExternalStream(ev.stream_ptr(), device=dev)
    marks = [torch.cuda.Event(enable_timing=True) for _ in range(k2 + 1)]
    walls = []
    t0 = time.perf_counter()
    marks[0].record(stream)
    for i in range(k2):
        a = time.perf_counter()
        ev.step_host(hnp, 1, DT)
        walls.append(time.perf_counter() - a)
        marks[i + 1].record(stream)
    el = time.perf_counter() - t0
    gc.enable()
    torch.cuda.synchronize()
    device_ms = [marks[i].elapsed_time(marks[i + 1]) for i in range(k2)]
    e2e_value, el = replica_throughput(points, 3, k2, el, ws)
    e2e = {"value": e2e_value, "unit": UNIT,
           "h2d_bytes_per_step": ev.state_size * 8, "d2h_bytes_per_step": ev.state_size * 8,
           "steps": k2, "call": "dgsw_step_host(h, pinned host state, 1, dt) per step",
           "ms_per_step": el / k2 * 1e3,
           "ms_per_call_min_median_max": [float(np.min(walls) * 1e3), float(np.median(walls) * 1e3),
                                          float(np.max(walls) * 1e3)],
           "device_ms_per_call_median": float(np.median(device_ms)),
           "device_ms_per_call_max": float(np.max(device_ms)),
           "host_pinned": bool(host.is_pinned()),
           "host_link_gbs": host_link_rates(host, dev)}
    ev.close()

    mixed = None
    if not args.no_mixed:
        evm, msm, _, statem, _ = time_path(args, PRECISION_MIXED, dev, rank, ws, False)
        # the launch shape the autotuner chose, re-timed after the timed region
        mixed_tune = evm.tune()
        evm.close()
        err = float(np.linalg.norm(statem - state64) / np.linalg.norm(state64))
        launch_m = msm / (3 * args.steps)
        gbs_m = MIXED_BYTES_PER_POINT_LAUNCH * points / (launch_m * 1e-3) / 1e9
        mixed = {"value": points * 3 * args.steps * ws / (msm * 1e-3), "unit": UNIT,
                 "ms_per_step": msm / args.steps,
                 "speedup_vs_fp64": ms / msm,
                 "rel_l2_vs_fp64_after_steps": err, "steps_compared": warm + args.steps,
                 "tune": mixed_tune,
                 "dtype": "f32 split-product contractions, f64 state and step accumulation",
                 "roofline": {"bound": "hbm", "achieved": gbs_m, "peak": hbm, "unit": "GB/s",
                              "frac": gbs_m / hbm,
                              "traffic": MIXED_TRAFFIC_PER_POINT_LAUNCH * points,
                              "traffic_note": "ncu DRAM bytes per stage launch, 20^3 capture "
                                              "scaled by points",
                              "bytes_per_point_launch": MIXED_BYTES_PER_POINT_LAUNCH,
                              "avg_launch_ms": launch_m}}

    if mixed is not None and not args.no_full_length and args.elements == ELEMS:
        mixed["full_length"] = config2_full_length(dev)

    # double-float arithmetic on the FP64 state (Taylor form of the step,
    # taylor_df.cu): FP64-level agreement at FP32-pipe rates
    double_float = None
    if not args.no_mixed:
        from spectre_gb300 import PRECISION_DOUBLE_FLOAT
        evd, msd, _, stated, _ = time_path(args, PRECISION_DOUBLE_FLOAT, dev, rank, ws, False)
        # host-resident state through dgsw_step_host, as the FP64 e2e leg
        hostd = torch.empty(evd.state_size, dtype=torch.float64, pin_memory=True)
        hd = hostd.numpy()
        evd.get_state(hd)
        for _ in range(max(args.warmup, 3)):
            evd.step_host(hd, 1, DT)
        torch.cuda.synchronize()
        kd = max(1, min(args.steps, 20))
        t0 = time.perf_counter()
        for _ in range(kd):
            evd.step_host(hd, 1, DT)
        e2e_d_ms = (time.perf_counter() - t0) / kd * 1e3
        evd.close()
        double_float = {
            "value": points * 3 * args.steps * ws / (msd * 1e-3), "unit": UNIT,
            "ms_per_step": msd / args.steps, "speedup_vs_fp64": ms / msd,
            "rel_l2_vs_fp64_after_steps": float(np.linalg.norm(stated - state64) /
                                                np.linalg.norm(state64)),
            "max_abs_vs_fp64_after_steps": float(np.max(np.abs(stated - state64))),
            "e2e": {"value": points * 3 * ws / (e2e_d_ms * 1e-3), "unit": UNIT,
                    "ms_per_step": e2e_d_ms, "steps": kd,
                    "call": "dgsw_step_host(h, pinned host state, 1, dt) per step"},
            "steps_compared": warm + args.steps,
            "dtype": "double-float (hi + lo f32 pairs, compensated products and sums), "
                     "f64 state; step as its Taylor polynomial",
            "launches_per_step": 3}

    batched = None
    if not args.no_batched:
        batched = time_batched(args, dev)
    adjoint = None
    if not args.no_adjoint:
        adjoint = time_adjoint(dev)
    adams = None
    if not args.no_adams:
        adams = time_adams(args, dev)
        peak = hbm or 1.0
        adams["gts"]["roofline"]["peak"] = hbm
        adams["gts"]["roofline"]["frac"] = adams["gts"]["roofline"]["achieved"] / peak
        # per unit of simulated time at the same step: AB3 takes one launch
        # per step where SSP-RK3 takes three
        adams["time_to_solution_speedup_vs_rk3_fp64"] = (ms / args.steps) / adams["gts"]["ms_per_slab"]
    curved = None
    if not args.no_curved:
        curved = time_curved(args, dev, rank == 0 and not args.no_cpu_baseline)
    next_rows = None
    if not args.no_next_rows:
        next_rows = time_next_rows(args, dev)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = cpu_threads()
        v, elc, pts = cpu_reference_run(CPU_SAMPLE_STEPS, 0, threads, args.elements)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "FP64 C++ restatement (oracle/, built with %s) on the workload "
                         "itself, %d^3 elements x 8^3 points, %d SSP-RK3 steps, %.1f s"
                         % (cpu_flags(), args.elements, CPU_SAMPLE_STEPS, elc)}
    if ws > 1:
        torch.distributed.barrier()
    if rank == 0:
        fp64_inst = FP64_INST_PER_POINT_STAGE * points / (launch_ms * 1e-3) / 1e12
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": warm, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(args.elements),
            "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm, "unit": "GB/s",
                         "frac": achieved_gbs / hbm,
                         "traffic": FP64_TRAFFIC_PER_POINT_LAUNCH * points,
                         "traffic_note": "ncu DRAM bytes per launch, 20^3 capture scaled by "
                                         "points",
                         "peak_source": peak_kind,
                         "bytes_per_point_launch": BYTES_PER_POINT_LAUNCH,
                         "avg_launch_ms": launch_ms},
            "fp64_pipe": {"achieved_tinst_s": fp64_inst, "peak_tinst_s": FP64_PEAK_TINST,
                          "frac": fp64_inst / FP64_PEAK_TINST,
                          "inst_per_point_stage": FP64_INST_PER_POINT_STAGE,
                          "note": "FP64 pipe binds the plain path on GB300; peak from a "
                                  "DFMA/DADD throughput probe on this pool's GB300"},
            "autotune": autotune,
            "mixed": mixed, "double_float": double_float, "batched": batched, "adjoint": adjoint,
            "curved": curved,
            "adams": adams, "next_rows": next_rows,
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": 3 * args.steps,
            "gpu_launches_note": "stage kernels of the timed FP64 region (one launch per stage)",
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-curved", action="store_true")
    ap.add_argument("--no-adams", action="store_true")
    ap.add_argument("--no-next-rows", action="store_true",
                    help="skip the Gauss / h-refined / ObserveNorms / filter / AMR timings")
    ap.add_argument("--curved-steps", type=int, default=0,
                    help="SSP-RK3 steps of the curved shell run (default 1000)")
    ap.add_argument("--curved-only", action="store_true",
                    help="run only the curved shell workload and print its numbers (for "
                         "profiling captures)")
    ap.add_argument("--batched-only", action="store_true",
                    help="run only the 256-instance mixed-extent workload and print its "
                         "numbers (for profiling captures)")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="run only the misfit-gradient workload (FP64 and mixed) and print its "
                         "numbers (for profiling captures)")
    ap.add_argument("--adjoint-steps", type=int, default=2000,
                    help="SSP-RK3 steps of the misfit-gradient workload (default 2000; fewer "
                         "only for profiling captures)")
    ap.add_argument("--double-float-only", action="store_true",
                    help="run only the double-float path on the --elements cube and print its "
                         "numbers (for profiling captures)")
    ap.add_argument("--no-full-length", action="store_true",
                    help="skip the accuracy runs over the configured step counts (500 steps "
                         "of the 32^3 case, 300 of the 256-instance case)")
    ap.add_argument("--batched-precision", default="both", choices=["both", "fp64", "mixed"],
                    help="which precision paths the 256-instance workload times (both by "
                         "default; one alone only for profiling captures)")
    ap.add_argument("--mixed-variant", type=int, default=-1,
                    help="impose one launch candidate of the uniform mixed path (dgsw_tune) "
                         "instead of the fastest; for profiling captures")
    ap.add_argument("--curved-variant", type=int, default=-1,
                    help="impose one launch candidate of the mixed curved path (dgsw_tune) "
                         "instead of the fastest; for profiling captures")
    ap.add_argument("--elements", type=int, default=ELEMS,
                    help="elements per axis (default 32: the benchmark workload; smaller "
                         "values only for profiling captures)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.curved_only:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(time_curved(args, 0, not args.no_cpu_baseline)), flush=True)
        return 0
    if args.batched_only:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(time_batched(args, 0)), flush=True)
        return 0
    if args.adjoint_only:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(time_adjoint(0, args.adjoint_steps)), flush=True)
        return 0
    if args.double_float_only:
        import torch
        from spectre_gb300 import PRECISION_DOUBLE_FLOAT
        torch.cuda.set_device(0)
        ev, ms, _, _, _ = time_path(args, PRECISION_DOUBLE_FLOAT, 0, 0, 1, False)
        pts = ev.grid_points
        ev.close()
        print(json.dumps({"precision": "double_float", "elements_per_axis": args.elements,
                          "ms_per_step": ms / args.steps,
                          "value": pts * 3 * args.steps / (ms * 1e-3), "unit": UNIT}),
              flush=True)
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
