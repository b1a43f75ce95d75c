"""Command line: render one workload with the engine.

    python -m linon_gb300 render --workload frames_1080p --field twist \
        --width 480 --height 270 --repeat 2 [--precise] [--brute-force]
    python -m linon_gb300 batch --views 64 --repeat 2 [--plain]
    python -m linon_gb300 lyapunov --width 1024 --height 1024 --repeat 2
    python -m linon_gb300 validate --field lens        # NVRTC report, no GPU
    python -m linon_gb300 validate --body my_field.wgsl [--helpers my_helpers.wgsl]

Prints one JSON line with the device time per launch (CUDA events).
"""
from __future__ import annotations

import argparse
import json
import statistics

from . import _abi, workloads as wl
from .engine import Engine, FramePlanes, predefined_source, validate_field


def _field_id(name):
    return _abi.FIELD_IDS[name]


def cmd_render(a):
    import torch
    w = getattr(wl, a.workload)(a.width, a.height)
    eng = Engine(0)
    stream = torch.cuda.Stream()
    eng.set_stream(stream)
    eng.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=not a.brute_force)
    fld = eng.compile_field(predefined_source(_field_id(a.field)), precise=a.precise)
    planes = FramePlanes.allocate(w.width, w.height)
    torch.cuda.synchronize()
    ts = []
    for _ in range(a.repeat):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        eng.render(fld, w.camera, w.settings, w.params, planes)
        e.record(stream)
        eng.synchronize()
        e.synchronize()
        ts.append(s.elapsed_time(e))
    steps = int(planes.steps.sum().item())
    hits = float((planes.hit_id >= 0).float().mean().item())
    print(json.dumps({"workload": w.name, "field": a.field, "width": w.width, "height": w.height,
                      "ms": ts, "ray_steps": steps, "ray_steps_per_s": steps / (statistics.median(ts) * 1e-3),
                      "hit_fraction": hits}))
    eng.close()


def cmd_batch(a):
    import torch
    w = wl.batch_uneven(a.views, seed=a.seed)
    eng = Engine(0)
    stream = torch.cuda.Stream()
    eng.set_stream(stream)
    eng.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    flds = [eng.compile_field(predefined_source(fid)) for fid in w.fields]
    views, planes = [], []
    for (W, H, camera, params, fidx) in w.extra["views"]:
        p = FramePlanes.allocate(W, H)
        v = _abi.View()
        v.camera, v.settings, v.params = camera, wl.settings(), params
        v.width, v.height, v.field_index = W, H, fidx
        v.out = p.abi()
        views.append(v)
        planes.append(p)
    torch.cuda.synchronize()
    ts = []
    for _ in range(a.repeat):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        if a.plain:
            eng.render_views_plain(flds, views)
        elif a.schedule == 1:
            eng.render_batch(flds, views, _abi.BatchTuning(a.quantum, a.block_threads, a.ctas_per_sm, a.tile[0], a.tile[1],
                                                           a.refill_below, 1))
        elif a.schedule in (2, 3):
            eng.render_batch(flds, views, _abi.BatchTuning(0, 0, a.ctas_per_sm, 0, 0, 0, a.schedule))
        else:
            eng.render_batch(flds, views)
        e.record(stream)
        eng.synchronize()
        e.synchronize()
        ts.append(s.elapsed_time(e))
    steps = sum(int(p.steps.sum().item()) for p in planes)
    print(json.dumps({"views": len(views), "plain": a.plain, "schedule": a.schedule, "quantum": a.quantum,
                      "refill_below": a.refill_below, "block_threads": a.block_threads, "tile": list(a.tile), "ms": ts, "ray_steps": steps,
                      "ray_steps_per_s": steps / (statistics.median(ts) * 1e-3)}))
    eng.close()


def cmd_lyapunov(a):
    """The Lyapunov pipeline (render, FP64 overlay, finite-time exponent,
    quantile threshold, outline pixels, outline capture) of the 1024^2
    workload at the given size; per-stage device ms."""
    import torch
    from . import lyapunov
    w = wl.lyapunov_1024(a.width, a.height)
    eng = Engine(0)
    stream = torch.cuda.Stream()
    eng.set_stream(stream)
    eng.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fld = eng.compile_field(predefined_source(w.fields[0]))
    runs = []
    with torch.cuda.stream(stream):
        for _ in range(a.repeat):
            runs.append(lyapunov.run(eng, fld, w, horizon=w.extra["T"], quantile=w.extra["quantile"], timings=True))
    print(json.dumps({"workload": w.name, "width": w.width, "height": w.height,
                      "ms": [r["ms"] for r in runs], "threshold": runs[-1]["threshold"]}))
    eng.close()


def cmd_validate(a):
    """Front end + NVRTC on a predefined field or on a user's field body
    (and helper functions) read from files, as the reference's shader reload
    does with an edited file (src/main.rs:206-222, main_view.rs:649-690).
    A rejected field prints the diagnostics and exits with status 1."""
    from pathlib import Path
    body = Path(a.body).read_text() if a.body else predefined_source(_field_id(a.field))
    helpers = Path(a.helpers).read_text() if a.helpers else None
    try:
        print(validate_field(body, helpers, precise=a.precise, batched=a.batched))
    except _abi.LinonCompileError as e:
        print(e.message)
        raise SystemExit(1)


def main():
    ap = argparse.ArgumentParser(prog="python -m linon_gb300")
    sub = ap.add_subparsers(dest="cmd", required=True)
    r = sub.add_parser("render")
    r.add_argument("--workload", default="frames_1080p")
    r.add_argument("--field", default="twist")
    r.add_argument("--width", type=int, default=480)
    r.add_argument("--height", type=int, default=270)
    r.add_argument("--repeat", type=int, default=2)
    r.add_argument("--precise", action="store_true")
    r.add_argument("--brute-force", action="store_true")
    b = sub.add_parser("batch")
    b.add_argument("--views", type=int, default=64)
    b.add_argument("--seed", type=int, default=0)
    b.add_argument("--repeat", type=int, default=2)
    b.add_argument("--plain", action="store_true")
    b.add_argument("--schedule", type=int, default=0, choices=(0, 1, 2, 3),
                   help="0 the default (one CTA per tile), 1 persistent queue of warp tiles, 2 one CTA per tile, "
                        "3 persistent queue of CTA tiles")
    b.add_argument("--quantum", type=int, default=1024, help="RK4 steps per quantum (persistent queue)")
    b.add_argument("--refill-below", type=int, default=0,
                   help="persistent queue: refill a warp's free lanes once fewer than this many are marching")
    b.add_argument("--block-threads", type=int, default=128, help="persistent queue: threads per CTA")
    b.add_argument("--ctas-per-sm", type=int, default=0, help="persistent queue: resident CTAs per SM (0 = most)")
    b.add_argument("--tile", type=int, nargs=2, default=(4, 8), metavar=("W", "H"),
                   help="persistent queue: pixel tile of 32 rays a warp takes")
    ly = sub.add_parser("lyapunov")
    ly.add_argument("--width", type=int, default=1024)
    ly.add_argument("--height", type=int, default=1024)
    ly.add_argument("--repeat", type=int, default=2)
    v = sub.add_parser("validate")
    v.add_argument("--field", default="twist")
    v.add_argument("--body", help="file holding a field_function body (instead of --field)")
    v.add_argument("--helpers", help="file holding WGSL helper functions for the body")
    v.add_argument("--precise", action="store_true")
    v.add_argument("--batched", action="store_true", help="also compile the batched kernels")
    a = ap.parse_args()
    {"render": cmd_render, "batch": cmd_batch, "lyapunov": cmd_lyapunov, "validate": cmd_validate}[a.cmd](a)


if __name__ == "__main__":
    main()
