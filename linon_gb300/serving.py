"""Python side of the serving loop (linon_serve_* in include/linon.h) and the
seeded request stream it is measured on.

The request stream restates what the reference's UI produces
(src/application.rs:275-291,466-489; src/main_view.rs:740-829): frames of
the current view at varying window sizes, Enhance re-renders at a finer step,
Lyapunov overlays, and ray-sample captures around clicked pixels; the field
function is switched periodically (the field combo box).  Arrivals are a
Poisson process (seeded).
"""
from __future__ import annotations

import ctypes as C
import math
import threading
import time
from dataclasses import dataclass

import numpy as np

from . import _abi, camera as cam, workloads as wl
from ._abi import check, load


class Server:
    """A running linon_server (scheduler thread inside the library)."""

    def __init__(self, engine, fields, hbm_budget: int = 0, slots: int = 2, max_wave: int = 256,
                 tuning: _abi.BatchTuning | None = None):
        self.lib = load()
        self.engine = engine
        cfg = _abi.ServeConfig()
        cfg.hbm_budget = hbm_budget
        cfg.slots = slots
        cfg.max_wave = max_wave
        if tuning is not None:
            cfg.tuning = tuning
        fa = (C.c_void_p * len(fields))(*[f.handle.value for f in fields])
        h = C.c_void_p()
        check(self.lib.linon_serve_start(engine.ctx, fa, len(fields), C.byref(cfg), C.byref(h)))
        self.h = h
        self._keep = []

    def submit(self, req: _abi.Request, pos=None) -> int:
        if pos is not None:
            pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 2)
            req.pos_xy = pos.ctypes.data
            req.n_rays = len(pos)
        rid = C.c_uint64()
        check(self.lib.linon_serve_submit(self.h, C.byref(req), C.byref(rid)))
        return rid.value

    def poll(self, rid: int) -> _abi.Result:
        r = _abi.Result()
        check(self.lib.linon_serve_poll(self.h, rid, C.byref(r)))
        return r

    def wait(self, rid: int, timeout_ms: float = 60000.0) -> _abi.Result:
        r = _abi.Result()
        check(self.lib.linon_serve_wait(self.h, rid, float(timeout_ms), C.byref(r)))
        return r

    def copy(self, rid: int, plane: int, out) -> None:
        """plane: 0 color, 1 mapping, 2 hit_id, 3 steps, 4 overlay, 5 exponents, 6 paths."""
        ptr = out.data_ptr() if hasattr(out, "data_ptr") else out.ctypes.data
        nbytes = out.numel() * out.element_size() if hasattr(out, "numel") else out.nbytes
        check(self.lib.linon_serve_copy(self.h, rid, plane, ptr, nbytes))

    def release(self, rid: int) -> None:
        check(self.lib.linon_serve_release(self.h, rid))

    def stats(self) -> dict:
        s = _abi.ServeStats()
        check(self.lib.linon_serve_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    def stop(self) -> None:
        if self.h:
            h, self.h = self.h, C.c_void_p()
            check(self.lib.linon_serve_stop(h))


def frame_request(field_index, camera, settings, params, width, height, kind=_abi.LINON_REQ_FRAME, fp64=True):
    r = _abi.Request()
    r.kind = kind
    r.field_index = field_index
    r.camera = camera
    r.settings = settings
    r.params = params
    r.width, r.height = width, height
    r.fp64_overlay = 1 if fp64 else 0
    return r


def capture_request(field_index, camera, settings, params, width, height, h, n_steps, every):
    r = _abi.Request()
    r.kind = _abi.LINON_REQ_CAPTURE
    r.field_index = field_index
    r.camera = camera
    r.settings = settings
    r.params = params
    r.width, r.height = width, height
    r.h = h
    r.n_steps = n_steps
    r.record_every = every
    return r


# ---- the seeded serving workload ------------------------------------------------
FRAME_SIZES = [(256, 256), (512, 512), (1024, 1024), (1280, 720), (1920, 1080)]


@dataclass
class Arrival:
    t: float          # seconds after the start
    req: _abi.Request
    pos: np.ndarray | None
    label: str


def request_stream(duration_s: float = 10.0, rate: float = 200.0, seed: int = 0, n_fields: int = 3,
                   switch_s: float = 5.0, h: float = 0.02):
    """Poisson arrivals at `rate`/s: 60% frames (256^2..1920x1080) at step h
    for t <= 4, 15% Enhance re-renders at h/4, 10% 1024^2 Lyapunov overlays
    (FP64), 15% captures of 16x16 rays around a clicked pixel with full
    polylines of 4000 points; the field switches every `switch_s` seconds;
    cameras on the radius-3 sphere.  The interactive step h = 0.02 is the
    coarsest step of the batch workload (Enhance then runs 800 steps)."""
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration_s:
            break
        fidx = int(t // switch_s) % n_fields
        d = rng.normal(size=3)
        camera = cam.look_at(3.0 * d / np.linalg.norm(d))
        u = rng.random()
        st = wl.settings()
        if u < 0.60:
            W, H = FRAME_SIZES[int(rng.integers(len(FRAME_SIZES)))]
            p = wl.fixed_steps(h, int(round(4.0 / h)), kahan=True, stop_on_hit=True)
            out.append(Arrival(t, frame_request(fidx, camera, st, p, W, H), None, "frame"))
        elif u < 0.75:
            W, H = FRAME_SIZES[int(rng.integers(len(FRAME_SIZES)))]
            p = wl.fixed_steps(h / 4, int(round(4.0 / (h / 4))), kahan=True, stop_on_hit=True)
            out.append(Arrival(t, frame_request(fidx, camera, st, p, W, H), None, "enhance"))
        elif u < 0.85:
            st = wl.settings(overlay_mode=1, delta=1, scaling=50.0)
            p = wl.fixed_steps(h, int(round(4.0 / h)), kahan=True)
            out.append(Arrival(t, frame_request(fidx, camera, st, p, 1024, 1024, kind=_abi.LINON_REQ_OVERLAY),
                               None, "overlay"))
        else:
            W, H = 1024, 1024
            px, py = rng.integers(8, W - 8), rng.integers(8, H - 8)
            g = (np.arange(16) - 7.5) / (W - 1)
            pos = np.stack(np.meshgrid(px / (W - 1) + g, py / (H - 1) + g), -1).reshape(-1, 2).astype(np.float32)
            p = wl.fixed_steps(h, int(round(4.0 / h)))
            out.append(Arrival(t, capture_request(fidx, camera, st, p, W, H, 0.001, 3999, 1), pos, "capture"))
    return out


def replay(server: Server, arrivals, time_scale: float = 1.0, timeout_s: float = 120.0):
    """Submits the arrivals in real time (a submitter thread) while the caller's
    thread collects completions; returns per-request records."""
    ids = [None] * len(arrivals)
    t0 = time.perf_counter()
    err = []

    def submitter():
        try:
            for i, a in enumerate(arrivals):
                dt = a.t * time_scale - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
                ids[i] = server.submit(a.req, a.pos)
        except Exception as e:  # surfaced to the caller below
            err.append(e)

    th = threading.Thread(target=submitter, daemon=True)
    th.start()
    records = []
    deadline = time.perf_counter() + timeout_s + arrivals[-1].t * time_scale if arrivals else 0
    i = 0
    while i < len(arrivals):
        if err:
            raise err[0]
        if ids[i] is None:
            if time.perf_counter() > deadline:
                raise TimeoutError("submission stalled")
            time.sleep(0.0002)
            continue
        r = server.wait(ids[i], timeout_ms=max(1.0, (deadline - time.perf_counter()) * 1000.0))
        records.append({"label": arrivals[i].label, "status": r.status, "latency_ms": r.t_done_ms - r.t_submit_ms,
                        "queue_ms": r.t_admit_ms - r.t_submit_ms, "t_submit_ms": r.t_submit_ms,
                        "t_done_ms": r.t_done_ms, "ray_steps": r.ray_steps, "wave": r.wave})
        server.release(ids[i])
        i += 1
    th.join()
    return records


def summarize(records):
    ok = [r for r in records if r["status"] == 0]
    lat = np.array([r["latency_ms"] for r in ok]) if ok else np.zeros(1)
    span_ms = (max(r["t_done_ms"] for r in ok) - min(r["t_submit_ms"] for r in ok)) if ok else 1.0
    by = {}
    for lab in sorted({r["label"] for r in ok}):
        v = np.array([r["latency_ms"] for r in ok if r["label"] == lab])
        by[lab] = {"n": int(len(v)), "p50_ms": float(np.percentile(v, 50)), "p99_ms": float(np.percentile(v, 99))}
    waves = {r["wave"] for r in ok}
    return {"requests": len(records), "completed": len(ok), "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat.max()),
            "ray_steps_per_s": float(sum(r["ray_steps"] for r in ok) / (span_ms * 1e-3)),
            "span_s": span_ms * 1e-3, "waves": len(waves), "by_kind": by}
