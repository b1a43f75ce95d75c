"""The Lyapunov-overlay pipeline with outline rays.

Reference: the overlay pass (src/overlay.wgsl:99-135, dispatched by
src/main_view.rs:844-846) and the Outline button (src/main_view.rs:804-829),
which re-renders and traces the 8 rays at the extremal pixels of the
diverging region (src/main_view.wgsl:381-480) for the path mesh of
src/ray_samples.rs:42-49.  Here the region's threshold can be the fixed
exponent of the shader (0.8 on the scaled exponent) or a quantile of the
finite-time exponent ln(max_nb |dx| / |d0|) / T (FP64 on the GPU).
"""
from __future__ import annotations

import time

import numpy as np

from . import _abi, workloads as wl
from .engine import FramePlanes, outline_indices


def run(engine, field, w, horizon: float = 4.0, quantile: float = 0.95, delta: int = 1,
        scaling: float = 50.0, timings: bool = False):
    import torch
    W, H = w.width, w.height
    out = {}
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(7)]
    s = torch.cuda.current_stream()
    ev[0].record(s)
    planes = FramePlanes.allocate(W, H)
    engine.render(field, w.camera, w.settings, w.params, planes)
    ev[1].record(s)
    st = wl.settings(overlay_mode=1, delta=delta, scaling=scaling)
    target = torch.empty((H, W, 4), dtype=torch.uint8, device="cuda")
    expo = torch.zeros((H, W), dtype=torch.float32, device="cuda")
    engine.overlay(st, W, H, planes.color, planes.mapping, target, expo, fp64=True)
    ev[2].record(s)
    ftle = torch.empty((H, W), dtype=torch.float32, device="cuda")
    engine.ftle(w.camera, w.params, W, H, planes.mapping, horizon, ftle)
    ev[3].record(s)
    thr = engine.exponent_quantile(ftle, W, H, quantile, border=1)
    ev[4].record(s)
    pix, pos = engine.outline_select(ftle, W, H, thr)
    ev[5].record(s)
    samples = torch.zeros((800, 8), dtype=torch.float32, device="cuda")
    engine.capture_reference(field, w.camera, w.settings, w.params, W, H, samples, positions=pos)
    ev[6].record(s)
    engine.synchronize()
    torch.cuda.synchronize()
    out.update(planes=planes, overlay=target, exponents=expo, ftle=ftle, threshold=thr, outline_pixels=pix,
               outline_positions=pos, samples=samples, indices=outline_indices())
    if timings:
        names = ["render", "overlay_fp64", "ftle_fp64", "quantile", "outline_select", "outline_capture"]
        out["ms"] = {n: ev[i].elapsed_time(ev[i + 1]) for i, n in enumerate(names)}
    return out
