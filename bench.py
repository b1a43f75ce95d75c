"""Benchmark of the nonlinear ray-casting hot path.

Headline workload (one "step"): the Cornell room at 1920x1080, one ray per
pixel, three field functions rendered in turn (linear, twist, point lens),
RK4 h = 0.005 for 4000 steps with Kahan-compensated position and time, FP32.
Metric: RK4 ray-steps per second (accepted steps summed over all rays of the
step / device time), plus ms per 1080p frame.  Inputs are resident (scene,
compiled fields); L2 is flushed (256 MB write) between timed steps, outside
the timed events.

Also reported: `e2e` (the same metric through the C-ABI host call
linon_render_host, device->host copies of all output planes inside the timed
region), the batched persistent kernel vs the plain per-view kernel on the
64-view uneven workload, the FP32 roofline of the march kernel against a
measured FFMA peak, and the oracle's CPU throughput on a bounded sample.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "RK4 ray-steps/s (1920x1080, 3 fields x 4000 steps)"
UNIT = "ray-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=10.0)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []  # (host time of arrival, csv line)
        self.first = threading.Event()

    def start(self):
        """Starts sampling every 100 ms and returns once the first sample has
        arrived (at most 3 s), so the sampler is live when the timed region
        begins."""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            self.first.wait(timeout=3.0)
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))
            self.first.set()

    def stop(self, t_begin: float | None = None, t_end: float | None = None):
        """Summary of the samples that arrived between t_begin and t_end
        (host perf_counter; all samples when none fall inside)."""
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        lines = [ln for t, ln in self.lines
                 if (t_begin is None or t >= t_begin) and (t_end is None or t <= t_end)]
        window = "timed region" if lines else "whole sampler run (no sample inside the timed region)"
        if not lines:
            lines = [ln for _, ln in self.lines]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm), "window": window, "interval_ms": 100}


def flops_per_step(pyoracle, w, fid):
    """Algorithmic FP32 operations of one accepted RK4 step: the operations
    the ray's endpoint depends on (oracle TraceFloat liveness), without
    loop-invariant work or products by launch constants, on an empty scene
    (intersection work excluded: the BVH culls it and brute-force-equivalent
    FLOPs are not claimed).  Returns (arithmetic ops, transcendental calls)
    per step; every + - * / sqrt counts 1, so an FMA is 2."""
    pix = np.array([w.width // 2 + (w.height // 2) * w.width, 17 + 11 * w.width], np.int32)
    live = pyoracle.count_live_ops(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32), w.camera,
                                   w.settings, w.params, fid, w.width, w.height, pix)
    return float(live[:, :4].sum(axis=1).mean()), float(live[:, 4].mean())


def kernel_name(field, label):
    """The march kernel a 1080p frame of `field` runs: two rays per thread
    (v30) when the field has a compiled pair form and at least 4 FP32
    operations and at most one transcendental per evaluation (the engine's
    rule; 1080p frames fill the GPU), else one ray per thread (v14)."""
    arith, transc = field.flops()
    pairs = field.pair_state() == 1 and arith >= 4 and transc <= 1
    return (f"linon_march_v{30 if pairs else 14} ({label} field; fixed steps, Kahan, field_weight 1; "
            f"{'two rays' if pairs else 'one ray'} per thread)")


def cpu_baseline(pyoracle, w, budget_s=12.0):
    """The oracle (FP32 restatement) on the host cores over a stratified
    pixel sample of the same frames; returns ray-steps/s and the sample."""
    threads = pyoracle.max_threads()
    rng = np.random.default_rng(0)
    n_total = w.width * w.height
    # calibrate on a sample that keeps every thread busy, then size the
    # measured sample to the time budget
    n_cal = min(n_total, 32 * threads)
    pix = np.sort(rng.choice(n_total, size=n_cal, replace=False)).astype(np.int32)
    t0 = time.perf_counter()
    for fid in w.fields:
        pyoracle.render(w.xyz, w.faces, w.face_rgb, w.camera, w.settings, w.params, fid, w.width, w.height,
                        pixels=pix, threads=threads, want=("steps",))
    dt = time.perf_counter() - t0
    n = int(min(n_total, max(n_cal, n_cal * budget_s / max(dt, 1e-3))))
    pix = np.sort(rng.choice(n_total, size=n, replace=False)).astype(np.int32)
    t0 = time.perf_counter()
    steps = 0
    for fid in w.fields:
        r = pyoracle.render(w.xyz, w.faces, w.face_rgb, w.camera, w.settings, w.params, fid, w.width, w.height,
                            pixels=pix, threads=threads, want=("steps",))
        steps += int(r["steps"].sum())
    dt = time.perf_counter() - t0
    return steps / dt, threads, f"{n} of {n_total} pixels (uniform random, seed 0) x {len(w.fields)} fields, {dt:.1f} s"


def cpu_views_sample(pyoracle, views, w, budget_s=4.0):
    """The oracle on a few rays of the uneven-view batch (each view's own
    camera, step size and field).  Like the reference it tests every face on
    every step (no BVH), which on the 82k-triangle scene limits the sample
    to a few rays per core; returns ray-steps/s, threads and the sample."""
    threads = pyoracle.max_threads()
    rng = np.random.default_rng(1)
    done, steps, rays, t_start = 0, 0, 0, time.perf_counter()
    order = rng.permutation(len(views))
    while time.perf_counter() - t_start < budget_s and done < len(order):
        W, H, camera, params, fidx = views[int(order[done])]
        pix = np.sort(rng.choice(W * H, size=threads, replace=False)).astype(np.int32)
        r = pyoracle.render(w.xyz, w.faces, w.face_rgb, camera, w.settings, params, w.fields[fidx], W, H,
                            pixels=pix, threads=threads, want=("steps",))
        steps += int(r["steps"].sum())
        rays += len(pix)
        done += 1
    dt = time.perf_counter() - t_start
    return steps / dt, threads, f"{rays} rays ({threads} per view) of {done} views, brute-force faces, {dt:.1f} s"


def bench_configs(eng, wl, predefined_source, pyoracle, cpu, keep=None):
    """The other workloads' GPU and CPU numbers: the 512^2 twist frame (h
    0.01 x 1000 steps), and the oracle on bounded samples of it, of the
    1024^2 Lyapunov render and of the 64 uneven views.  keep: receives the
    512^2 frame's planes for the accuracy leg."""
    import torch
    out = {}
    w = wl.plain_small()
    eng.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fld = eng.compile_field(predefined_source(w.fields[0]))
    from linon_gb300 import FramePlanes
    planes = FramePlanes.allocate(w.width, w.height)
    ts = []
    with torch.cuda.stream(eng.stream):
        for i in range(6):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(eng.stream)
            eng.render(fld, w.camera, w.settings, w.params, planes)
            b.record(eng.stream)
            b.synchronize()
            if i:
                ts.append(a.elapsed_time(b))
    steps = int(planes.steps.sum().item())
    ms = statistics.median(ts)
    out["plain_512_twist"] = {"workload": w.name, "frame_ms": ms, "ray_steps_per_s": steps / (ms * 1e-3)}
    if keep is not None:
        keep["plain_512_twist"] = (w, planes)
    if cpu:
        v, th, smp = cpu_baseline(pyoracle, w, budget_s=3.0)
        out["plain_512_twist"]["cpu"] = {"value": v, "unit": UNIT, "cores": th, "kind": "port", "sample": smp}
        w2 = wl.lyapunov_1024()
        v, th, smp = cpu_baseline(pyoracle, w2, budget_s=3.0)
        out["lyapunov_1024_render_cpu"] = {"value": v, "unit": UNIT, "cores": th, "kind": "port", "sample": smp}
        w3 = wl.batch_uneven(64)
        v, th, smp = cpu_views_sample(pyoracle, w3.extra["views"], w3)
        out["batch_uneven_64_cpu"] = {"value": v, "unit": UNIT, "cores": th, "kind": "port", "sample": smp}
    return out


def run_reference(args):
    """--impl reference: the reference path's CPU implementation on the host
    cores.  The reference is WGSL run through wgpu on a graphics API, which
    does not exist on this machine, so its CPU path is the oracle port (the
    FP32 restatement of the shader, OpenMP over all host threads)."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from linon_gb300 import workloads as wl
    from oracle import pyoracle
    w = wl.frames_1080p(args.width, args.height)
    vals = []
    # each timed step is a bounded sample (about a minute of CPU work over
    # all timed steps, 1-6 s each), each warm-up step a 1 s sample
    budget = max(1.0, min(6.0, 60.0 / max(args.steps, 1)))
    for i in range(args.warmup + args.steps):
        v, threads, sample = cpu_baseline(pyoracle, w, budget_s=budget if i >= args.warmup else 1.0)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    # this leg stands alone: the workload builders fill every struct in
    # Python, so the engine library must not have been mapped
    maps = Path("/proc/self/maps").read_text() if Path("/proc/self/maps").exists() else ""
    if "liblinon.so" in maps:
        raise RuntimeError("the CPU reference leg mapped the engine library liblinon.so")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w.name, "width": w.width, "height": w.height, "fields": ["linear", "twist", "lens"],
                       "h": 0.005, "steps_per_ray": 4000, "kahan": True},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    import torch.distributed as dist

    from linon_gb300 import Engine, FramePlanes, workloads as wl
    from linon_gb300.engine import predefined_source
    from oracle import pyoracle

    rank, world, local = dist_info()
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    os.environ.setdefault("LINON_CACHE_DIR", str(ROOT / "_build_cache"))
    Path(os.environ["LINON_CACHE_DIR"]).mkdir(exist_ok=True)

    w = wl.frames_1080p(args.width, args.height)
    eng = Engine(local)
    stream = torch.cuda.Stream(device=dev)
    eng.set_stream(stream)
    eng.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fields = [eng.compile_field(predefined_source(fid)) for fid in w.fields]
    planes = [FramePlanes.allocate(w.width, w.height, dev) for _ in fields]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step():
        for f, p in zip(fields, planes):
            eng.render(f, w.camera, w.settings, w.params, p)

    with torch.cuda.stream(stream):
        for _ in range(max(3, args.warmup)):
            step()
        stream.synchronize()
        eng.synchronize()
        steps_per_frame = [int(p.steps.sum().item()) for p in planes]
    ray_steps = sum(steps_per_frame)

    # ---- timed region: device time of exactly K steps (events on the
    #      engine's stream), L2 flushed between steps outside the events ----
    clocks = ClockSampler(torch.cuda.current_device())
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    fev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in fields]
           for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_wall = time.perf_counter()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()
            evs[k][0].record(stream)
            for i, (f, p) in enumerate(zip(fields, planes)):
                fev[k][i][0].record(stream)
                eng.render(f, w.camera, w.settings, w.params, p)
                fev[k][i][1].record(stream)
            evs[k][1].record(stream)
    torch.cuda.synchronize()
    t_end = time.perf_counter()
    wall = t_end - t_wall
    clk = clocks.stop(t_wall, t_end)
    eng.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = sum(step_ms)
    frame_ms = [[a.elapsed_time(b) for a, b in row] for row in fev]
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = ray_steps * args.steps * world / (total_ms * 1e-3)
    ms_per_step = total_ms / args.steps
    per_field_ms = [statistics.median(col) for col in zip(*frame_ms)]

    # ---- e2e: the reference-facing C-ABI call with host output buffers ----
    n_pix = w.width * w.height
    host = [{"color": torch.empty((w.height, w.width, 4), dtype=torch.uint8).pin_memory().numpy(),
             "mapping": torch.empty((w.height, w.width, 4), dtype=torch.float32).pin_memory().numpy(),
             "hit_id": torch.empty((w.height, w.width), dtype=torch.int32).pin_memory().numpy(),
             "steps": torch.empty((w.height, w.width), dtype=torch.int32).pin_memory().numpy()} for _ in fields]
    # warm the host-path buffers; the ray-steps of one call per field are
    # counted here from the returned step planes (the same inputs give the
    # same counts on every call, so the timed loop only renders and copies)
    steps_per_field = []
    for f, h in zip(fields, host):
        eng.render_host(f, w.camera, w.settings, w.params, w.width, w.height, **h)
        steps_per_field.append(int(h["steps"].sum(dtype=np.int64)))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for f, h in zip(fields, host):
            eng.render_host(f, w.camera, w.settings, w.params, w.width, w.height, **h)
    e2e_dt = time.perf_counter() - t0
    e2e_steps = args.steps * sum(steps_per_field)
    for h, k in zip(host, steps_per_field):  # the last call returned the same planes
        assert int(h["steps"].sum(dtype=np.int64)) == k
    e2e = {"value": e2e_steps / e2e_dt * world, "unit": UNIT,
           "h2d_bytes_per_step": len(fields) * (112 + 24 + 48),
           "d2h_bytes_per_step": len(fields) * n_pix * (4 + 16 + 4 + 4),
           "path": "linon_render_host (C ABI), host planes copied back inside the call"}

    result = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
              "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
              "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene and cameras)",
              "config": {"workload": w.name, "width": w.width, "height": w.height,
                         "fields": ["linear", "twist", "lens"], "h": 0.005, "steps_per_ray": 4000,
                         "kahan": True, "bvh": True, "l2": "flushed between steps (256 MB write, outside events)",
                         "parallelism": f"replicas x{world}"},
              "frame_ms_1080p": {n: round(v, 3) for n, v in zip(["linear", "twist", "lens"], per_field_ms)},
              "wall_s_timed_region": wall, "e2e": e2e, "clocks": clk,
              "gpu_launches": args.steps * len(fields)}

    # ---- roofline: FP32 against a measured FFMA peak ----
    if rank == 0:
        peak = eng.probe_fp32_peak()
        fl = [flops_per_step(pyoracle, w, fid) for fid in w.fields]
        n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
        # dominant kernel: the march launch with the largest median time
        i = int(np.argmax(per_field_ms))
        achieved = fl[i][0] * steps_per_frame[i] / (per_field_ms[i] * 1e-3) / 1e12
        result["roofline"] = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                              "frac": achieved / peak, "traffic": None,
                              "traffic_note": "not measured in this run (ncu cannot run inside it); a separate ncu "
                                              "capture of the same kernels at 1080p (profiles/"
                                              "march_1080p_traffic.md) counts 0.10 MB read + 3.55 MB written "
                                              "per lens launch, 37-39 MB per linear or twist launch: most of "
                                              "the 58 MB of output planes is still L2-resident when the "
                                              "launch ends",
                              "kernel": kernel_name(fields[i], ["linear", "twist", "lens"][i]),
                              "peak_source": "measured FFMA probe in this run (linon_probe_fp32_peak)",
                              "peak_nominal_at_median_clock": (n_sm * 128 * 2 * clk["sm_mhz"] * 1e6 / 1e12
                                                               if clk.get("sm_mhz") else None),
                              "peak_nominal_formula": f"{n_sm} SMs x 128 FP32 lanes x 2 (FMA) x median SM clock",
                              "flops_definition": "live FP32 operations per ray-step (oracle TraceFloat)",
                              "executed_note": "not measured in this run; ncu instruction counters of the same "
                                               "kernels at 1080p (profiles/fp32_executed_ops_batch64_and_1080p_"
                                               "frames.md) count 17.3 / 82.7 / 152.9 executed FP32 operations "
                                               "per linear / twist / lens ray-step: the lens kernel 0.60 and "
                                               "the three frames 0.51 of the FFMA probe",
                              "flops_per_step": {n: round(a, 2) for n, (a, _) in zip(["linear", "twist", "lens"], fl)},
                              "transcendentals_per_step": {n: round(t, 2) for n, (_, t) in
                                                           zip(["linear", "twist", "lens"], fl)},
                              "all_fields_frac": sum(a * s for (a, _), s in zip(fl, steps_per_frame))
                              / (sum(per_field_ms) * 1e-3) / 1e12 / peak}

    # engine planes of the headline frames at the accuracy leg's pixels
    keep = {}
    if rank == 0 and not args.no_accuracy:
        from oracle import accuracy as acc
        pix = acc.sample_pixels(w.width, w.height, 4000, seed=11)
        keep["frames_1080p"] = (w, pix, [p.sample(pix) for p in planes])

    # ---- batched persistent kernel vs plain per-view kernel (64 views) ----
    if rank == 0 and not args.no_batch:
        result["batch_uneven_64"] = bench_batch(eng, stream, wl, torch, dev, predefined_source, keep)

    # ---- Lyapunov pipeline at 1024^2 (scaled Lorenz + v0, h 0.002 x 2000) ----
    if rank == 0 and not args.no_batch:
        result["lyapunov_1024"] = bench_lyapunov(eng, wl, predefined_source, keep)

    # ---- serving: Poisson request stream, continuous batching ----
    if rank == 0 and not args.no_serve:
        result["serving"] = bench_serving(eng, wl, predefined_source, args.serve_seconds)

    # ---- CPU baseline (oracle port on this host's cores, bounded sample) ----
    if rank == 0 and world == 1 and not args.no_cpu:
        v, threads, sample = cpu_baseline(pyoracle, w)
        result["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}
    # ---- the other workloads: 512^2 twist frame; CPU samples of the rest ----
    if rank == 0 and world == 1 and not args.no_batch:
        result["configs"] = bench_configs(eng, wl, predefined_source, pyoracle, cpu=not args.no_cpu, keep=keep)
    # ---- accuracy: every benchmarked workload against the FP64 oracle ----
    if rank == 0 and not args.no_accuracy:
        result["accuracy"] = accuracy_leg(keep)
    if rank == 0:
        print(json.dumps(result))
    eng.close()
    if world > 1:
        dist.destroy_process_group()


def accuracy_leg(keep):
    """The engine's results against the FP64 oracle (and the FP32 oracle's
    own error beside them) on seeded pixel samples of every benchmarked
    workload; oracle/accuracy.py defines each figure.  Runs after every timed
    region, on the host cores."""
    import torch
    from linon_gb300 import _abi
    from oracle import accuracy as acc
    FIELD_NAMES = {_abi.FIELD_IDS[n]: n for n in ("linear", "twist", "lens", "lorenz_scaled")}
    t0 = time.perf_counter()
    out = {"endpoint_err_unit": "scene units (Euclidean distance to the FP64 oracle's endpoint)"}
    if "frames_1080p" in keep:
        w, pix, px = keep["frames_1080p"]
        info = acc.FaceInfo(w.xyz, w.faces)
        out["frames_1080p"] = {FIELD_NAMES[f]: acc.public(acc.frame_pixels_report(w, f, e, pix, info))
                               for f, e in zip(w.fields, px)}
        out["frames_1080p"]["sample"] = f"{len(pix)} pixels per field (seed 11) of the last timed frames"
    if "plain_512_twist" in keep:
        w, planes = keep["plain_512_twist"]
        pix = acc.sample_pixels(w.width, w.height, 4000, seed=5)
        out["plain_512_twist"] = acc.public(acc.frame_pixels_report(w, w.fields[0], planes.sample(pix), pix))
        out["plain_512_twist"]["sample"] = "4000 pixels (seed 5)"
    if "lyapunov_1024" in keep:
        w, r = keep["lyapunov_1024"]
        centres = acc.sample_pixels(w.width, w.height, 4000, seed=23, border=2)
        idx = torch.as_tensor(centres.astype(np.int64), device=r["ftle"].device)
        rep = acc.lyapunov_report(w, w.fields[0], centres, r["ftle"].reshape(-1)[idx].cpu().numpy(),
                                  r["exponents"].reshape(-1)[idx].cpu().numpy(), r["threshold"],
                                  r["outline_pixels"], w.extra["T"], engine_px=r["planes"].sample(centres),
                                  info=acc.FaceInfo(w.xyz, w.faces))
        out["lyapunov_1024"] = acc.public(rep)
        out["lyapunov_1024"]["sample"] = "4000 interior pixels (seed 23), each with its 4 neighbours"
    if "batch_uneven_64" in keep:
        w, planes = keep["batch_uneven_64"]
        views = w.extra["views"]
        pix = [acc.sample_pixels(W, H, 200, seed=100 + i) for i, (W, H, *_r) in enumerate(views)]
        eng = [p.sample(px) for p, px in zip(planes, pix)]
        names = {i: FIELD_NAMES[f] for i, f in enumerate(w.fields)}
        out["batch_uneven_64"] = acc.public(acc.batch_report(w, views, eng, pix, names))
        out["batch_uneven_64"]["sample"] = "200 pixels per view (seeds 100..163), pooled per field"
    out["oracle_s"] = time.perf_counter() - t0
    return out


def bench_lyapunov(eng, wl, predefined_source, keep=None):
    """Render + FP64 overlay + finite-time exponent (T = 4) + p95 threshold +
    outline pixels + 8x100 outline capture, per-stage device ms (median of 3).
    keep: receives the last run's maps for the accuracy leg."""
    import torch
    from linon_gb300 import lyapunov
    w = wl.lyapunov_1024()
    eng.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fld = eng.compile_field(predefined_source(w.fields[0]))
    with torch.cuda.stream(eng.stream):  # events and engine work on one stream
        runs = [lyapunov.run(eng, fld, w, horizon=w.extra["T"], quantile=w.extra["quantile"], timings=True)
                for _ in range(4)][1:]
    ms = {k: statistics.median(r["ms"][k] for r in runs) for k in runs[0]["ms"]}
    steps = int(runs[-1]["planes"].steps.sum().item())
    if keep is not None:
        keep["lyapunov_1024"] = (w, runs[-1])
    return {"workload": w.name, "ms": ms, "total_ms": sum(ms.values()),
            "render_ray_steps_per_s": steps / (ms["render"] * 1e-3), "threshold_p95": runs[-1]["threshold"]}


def bench_serving(eng, wl, predefined_source, seconds):
    """Poisson 200 req/s (seeded) of frames 256^2..1920x1080 (60%), Enhance at
    h/4 (15%), 1024^2 FP64 Lyapunov overlays (10%) and 16x16-ray captures with
    4000-point polylines (15%), field switched every 5 s, over the Cornell room
    + four icospheres behind the BVH; 40 GB budget for request outputs."""
    from linon_gb300 import serving
    w = wl.batch_uneven(1, seed=0)
    eng.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    flds = [eng.compile_field(predefined_source(fid)) for fid in w.fields]
    arrivals = serving.request_stream(duration_s=seconds, rate=200.0, seed=0)
    srv = serving.Server(eng, flds, hbm_budget=40 << 30, slots=3)
    try:
        # warm the batch module and pool outside the measurement
        serving.replay(srv, serving.request_stream(duration_s=0.25, rate=200.0, seed=99))
        records = serving.replay(srv, arrivals)
        stats = srv.stats()
    finally:
        srv.stop()
    s = serving.summarize(records)
    s.update({"rate_req_per_s": 200.0, "duration_s": seconds, "hbm_budget_bytes": 40 << 30, "slots": 3,
              "bytes_peak": stats["bytes_peak"], "latency": "submit -> completion seen by the server (host clock)"})
    return s


def bench_batch(eng, stream, wl, torch, dev, predefined_source, keep=None):
    from linon_gb300 import FramePlanes, _abi
    w = wl.batch_uneven(64, seed=0)
    eng.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    flds = [eng.compile_field(predefined_source(fid)) for fid in w.fields]
    views, planes = [], []
    for (W, H, camera, params, fidx) in w.extra["views"]:
        p = FramePlanes.allocate(W, H, dev)
        v = _abi.View()
        v.camera, v.settings, v.params = camera, wl.settings(), params
        v.width, v.height, v.field_index = W, H, fidx
        v.out = p.abi()
        views.append(v)
        planes.append(p)

    def timed(fn, reps=5):
        ts = []
        with torch.cuda.stream(stream):
            fn()
            stream.synchronize()
            for _ in range(reps):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                b.record(stream)
                b.synchronize()
                ts.append(a.elapsed_time(b))
        return statistics.median(ts)

    plain_ms = timed(lambda: eng.render_views_plain(flds, views))
    steps_plain = sum(int(p.steps.sum().item()) for p in planes)
    # the persistent work-queue forms on their own: resident CTAs take
    # 8x16-pixel tiles from a device counter (schedule 3), or warps take
    # 4x8-pixel tiles of 32 rays (schedule 1, 128-thread CTAs)
    forms = {"cta_tiles": _abi.BatchTuning(0, 0, 0, 0, 0, 0, 3),
             "warp_tiles": _abi.BatchTuning(1024, 128, 0, 4, 8, 0, 1)}
    form_ms = {k: timed(lambda t=t: eng.render_batch(flds, views, t)) for k, t in forms.items()}
    best_form = min(form_ms, key=form_ms.get)
    tuning, tune_ms = eng.autotune_batch(flds, views)
    batch_ms = timed(lambda: eng.render_batch(flds, views, tuning))
    eng.synchronize()
    steps_batch = sum(int(p.steps.sum().item()) for p in planes)
    rays = sum(v.width * v.height for v in views)
    if keep is not None:  # the planes of the last (autotuned batched) render
        keep["batch_uneven_64"] = (w, planes)
    return {"views": len(views), "rays": rays, "ray_steps": steps_batch, "plain_ms": plain_ms,
            "batched_ms": batch_ms, "plain_ray_steps_per_s": steps_plain / (plain_ms * 1e-3),
            "batched_ray_steps_per_s": steps_batch / (batch_ms * 1e-3), "speedup": plain_ms / batch_ms,
            "persistent_queue": {"ms": form_ms[best_form], "speedup": plain_ms / form_ms[best_form],
                                 "form": best_form,
                                 "forms": {k: {"ms": v, "speedup": plain_ms / v} for k, v in form_ms.items()},
                                 "cta_tiles": "schedule 3: 8x16-pixel tiles, 128-thread CTAs",
                                 "warp_tiles": "schedule 1: 4x8-pixel tiles, 128-thread CTAs, refill_below 0"},
            "tuning": {"schedule": {1: "persistent queue of warp tiles" + (" (lane refills)" if tuning.refill_below
                                                                           else ""),
                                    2: "one CTA per tile", 3: "persistent queue of CTA tiles"}.get(tuning.schedule,
                                                                                                  "auto"),
                       "quantum": tuning.quantum, "block_threads": tuning.block_threads,
                       "tile": [tuning.tile_w, tuning.tile_h], "refill_below": tuning.refill_below}}


if __name__ == "__main__":
    main()
