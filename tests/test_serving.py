"""Serving loop (continuous batching): results alone == results in the mix
== the drop-in calls' results, HBM-budget admission, overlap of waves,
bounded waits."""
import numpy as np
import pytest
import torch

from linon_gb300 import _abi, scene, serving, workloads as wl
from linon_gb300.engine import predefined_source


def test_request_stream_is_seeded_and_mixed():
    a = serving.request_stream(duration_s=20.0, rate=200.0, seed=3)
    b = serving.request_stream(duration_s=20.0, rate=200.0, seed=3)
    assert [x.t for x in a] == [x.t for x in b]
    labels = [x.label for x in a]
    n = len(labels)
    assert 0.9 * 4000 < n < 1.1 * 4000
    frac = {k: labels.count(k) / n for k in ("frame", "enhance", "overlay", "capture")}
    assert abs(frac["frame"] - 0.60) < 0.04 and abs(frac["enhance"] - 0.15) < 0.03
    assert abs(frac["overlay"] - 0.10) < 0.03 and abs(frac["capture"] - 0.15) < 0.03
    # field switched every 5 s
    f = [x.req.field_index for x in a]
    assert set(f[:10]) == {0} and set(x.req.field_index for x in a if 5.0 <= x.t < 10.0) == {1}
    caps = [x for x in a if x.label == "capture"]
    assert caps[0].pos.shape == (256, 2) and caps[0].req.n_steps == 3999


def test_summarize_statistics():
    """Serving summary on synthetic records: failed requests excluded,
    percentiles per kind, throughput over the span of completed requests."""
    recs = []
    for i in range(100):
        recs.append({"status": 0, "latency_ms": float(i + 1), "t_submit_ms": float(i), "t_done_ms": float(i + 10),
                     "label": "frame" if i % 4 else "capture", "ray_steps": 1000, "wave": i // 10})
    recs.append({"status": 4, "latency_ms": 1e9, "t_submit_ms": 0.0, "t_done_ms": 1e9, "label": "frame",
                 "ray_steps": 10 ** 12, "wave": 99})
    sm = serving.summarize(recs)
    assert sm["requests"] == 101 and sm["completed"] == 100
    assert sm["p50_ms"] == np.percentile(np.arange(1, 101), 50) and sm["max_ms"] == 100.0
    assert sm["p99_ms"] == np.percentile(np.arange(1, 101), 99)
    assert sm["waves"] == 10
    assert abs(sm["span_s"] - 0.109) < 1e-12                       # first submit 0 ms, last done 109 ms
    assert abs(sm["ray_steps_per_s"] - 100 * 1000 / 0.109) < 1e-6
    assert sm["by_kind"]["capture"]["n"] == 25 and sm["by_kind"]["frame"]["n"] == 75
    lat_c = [float(i + 1) for i in range(100) if i % 4 == 0]
    assert sm["by_kind"]["capture"]["p50_ms"] == np.percentile(lat_c, 50)


def _setup(engine, precise=False):
    xyz, faces, rgb = scene.cornell_with_spheres(seed=2, subdivisions=3)
    engine.upload_scene(xyz, faces, rgb, bvh=True)
    names = ["linear", "twist", "lens"]
    return [engine.compile_field(predefined_source(_abi.FIELD_IDS[n]), precise=precise) for n in names]


def _requests(seed=5):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(10):
        d = rng.normal(size=3)
        camera = serving.cam.look_at(3.0 * d / np.linalg.norm(d))
        W, H = [(64, 48), (96, 96), (128, 72), (33, 17)][i % 4]
        kind = i % 3
        if kind == 0:
            p = wl.fixed_steps(0.02, 200, kahan=True, stop_on_hit=True)
            out.append((serving.frame_request(i % 3, camera, wl.settings(), p, W, H), None))
        elif kind == 1:
            p = wl.fixed_steps(0.02, 150, kahan=True)
            st = wl.settings(overlay_mode=1, delta=1)
            out.append((serving.frame_request(i % 3, camera, st, p, W, H, kind=_abi.LINON_REQ_OVERLAY), None))
        else:
            pos = rng.uniform(0.2, 0.8, size=(40, 2)).astype(np.float32)
            p = wl.fixed_steps(0.02, 100)
            out.append((serving.capture_request(i % 3, camera, wl.settings(), p, W, H, 0.005, 301, 3), pos))
    return out


def _fetch(server, rid, req):
    r = server.poll(rid)
    assert r.status == 0, r.status
    out = {}
    if req.kind == _abi.LINON_REQ_CAPTURE:
        t = torch.empty((req.n_rays, r.n_points, 4), dtype=torch.float32, device="cuda")
        server.copy(rid, 6, t)
        out["paths"] = t.cpu().numpy()
        return out
    n = req.width * req.height
    for plane, name, dt, k in ((0, "color", torch.uint8, 4), (1, "mapping", torch.float32, 4),
                               (2, "hit_id", torch.int32, 1), (3, "steps", torch.int32, 1)):
        t = torch.empty(n * k, dtype=dt, device="cuda")
        server.copy(rid, plane, t)
        out[name] = t.cpu().numpy()
    if req.kind == _abi.LINON_REQ_OVERLAY:
        for plane, name, dt in ((4, "overlay", torch.uint8), (5, "exponents", torch.float32)):
            t = torch.empty(n * (4 if name == "overlay" else 1), dtype=dt, device="cuda")
            server.copy(rid, plane, t)
            out[name] = t.cpu().numpy()
    out["ray_steps"] = r.ray_steps
    return out


@pytest.mark.gpu
def test_results_alone_equal_results_in_the_mix(engine):
    fields = _setup(engine)
    reqs = _requests()
    alone = []
    srv = serving.Server(engine, fields)
    try:
        for req, pos in reqs:
            rid = srv.submit(req, pos)
            srv.wait(rid)
            alone.append(_fetch(srv, rid, req))
            srv.release(rid)
    finally:
        srv.stop()
    srv = serving.Server(engine, fields, slots=3)
    try:
        ids = [srv.submit(req, pos) for req, pos in reqs]  # all in flight together
        mixed = []
        for rid, (req, _) in zip(ids, reqs):
            srv.wait(rid)
            mixed.append(_fetch(srv, rid, req))
        waves = {srv.poll(rid).wave for rid in ids}
        for rid in ids:
            srv.release(rid)
    finally:
        srv.stop()
    assert len(waves) < len(reqs)  # requests shared waves
    for a, b in zip(alone, mixed):
        for k in a:
            np.testing.assert_array_equal(np.asarray(a[k]), np.asarray(b[k]))
    assert all(x["ray_steps"] > 0 for x in alone if "ray_steps" in x)


@pytest.mark.gpu
def test_served_results_equal_the_plain_calls(engine):
    """Frames, overlays and captures served in shared waves (precise
    modules) equal, bit for bit, what the drop-in calls give for the same
    request: linon_render, linon_overlay (linear output) and
    linon_capture_paths."""
    from linon_gb300 import FramePlanes
    fields = _setup(engine, precise=True)
    reqs = _requests()
    srv = serving.Server(engine, fields, slots=3)
    try:
        ids = [srv.submit(req, pos) for req, pos in reqs]
        served = []
        for rid, (req, _) in zip(ids, reqs):
            srv.wait(rid)
            served.append(_fetch(srv, rid, req))
        for rid in ids:
            srv.release(rid)
    finally:
        srv.stop()
    for (req, pos), s in zip(reqs, served):
        fld = fields[req.field_index]
        W, H = req.width, req.height
        if req.kind == _abi.LINON_REQ_CAPTURE:
            npts = -(-req.n_steps // req.record_every) + 1
            out = torch.empty((req.n_rays, npts, 4), dtype=torch.float32, device="cuda")
            engine.capture_paths(fld, req.camera, req.settings, req.params, W, H, pos, req.h, req.n_steps,
                                 req.record_every, out)
            engine.synchronize()
            np.testing.assert_array_equal(out.cpu().numpy(), s["paths"])
            continue
        planes = FramePlanes.allocate(W, H)
        engine.render(fld, req.camera, req.settings, req.params, planes)
        engine.synchronize()
        for k in ("color", "mapping", "hit_id", "steps"):
            np.testing.assert_array_equal(getattr(planes, k).cpu().numpy().reshape(-1), s[k], err_msg=k)
        if req.kind == _abi.LINON_REQ_OVERLAY:
            target = torch.empty((H, W, 4), dtype=torch.uint8, device="cuda")
            expo = torch.zeros((H, W), dtype=torch.float32, device="cuda")
            engine.overlay(req.settings, W, H, planes.color, planes.mapping, target, expo, srgb=False,
                           fp64=bool(req.fp64_overlay))
            engine.synchronize()
            np.testing.assert_array_equal(target.cpu().numpy().reshape(-1), s["overlay"])
            # the served exponents buffer starts zeroed like this one; border pixels stay 0
            np.testing.assert_array_equal(expo.cpu().numpy().reshape(-1), s["exponents"])


@pytest.mark.gpu
def test_budget_admission_and_errors(engine):
    fields = _setup(engine)
    camera = serving.cam.look_at((0.0, 0.0, 3.0))
    p = wl.fixed_steps(0.02, 200, kahan=True)
    one = 256 * 256 * 28 + 4 * 256
    srv = serving.Server(engine, fields, hbm_budget=2 * one + 1024)
    try:
        ids = [srv.submit(serving.frame_request(0, camera, wl.settings(), p, 256, 256)) for _ in range(6)]
        for rid in ids:
            assert srv.wait(rid).status == 0
            srv.release(rid)
        st = srv.stats()
        assert st["bytes_peak"] <= 2 * one + 1024 and st["completed"] == 6
        with pytest.raises(_abi.LinonError) as e:
            srv.submit(serving.frame_request(0, camera, wl.settings(), p, 1024, 1024))
        assert e.value.status == _abi.LINON_ENOMEM
        with pytest.raises(_abi.LinonError) as e:
            srv.submit(serving.frame_request(7, camera, wl.settings(), p, 64, 64))
        assert e.value.status == _abi.LINON_EINVAL
    finally:
        srv.stop()


@pytest.mark.gpu
def test_waves_overlap_and_bounded_wait(engine):
    fields = _setup(engine)
    camera = serving.cam.look_at((0.3, 0.2, 3.0))
    long_p = wl.fixed_steps(0.0025, 1600, kahan=True)
    short_p = wl.fixed_steps(0.02, 50, kahan=True, stop_on_hit=True)
    srv = serving.Server(engine, fields, slots=2)
    try:
        rl = srv.submit(serving.frame_request(2, camera, wl.settings(), long_p, 1920, 1080))
        with pytest.raises(_abi.LinonError) as e:
            srv.wait(rl, timeout_ms=0.01)  # still running
        assert e.value.status == _abi.LINON_ETIMEOUT
        rs = srv.submit(serving.frame_request(0, camera, wl.settings(), short_p, 64, 64))
        a, b = srv.wait(rl), srv.wait(rs)
        assert a.status == 0 and b.status == 0
        assert a.wave != b.wave
        assert b.t_done_ms < a.t_done_ms  # the short request did not wait for the long one
        srv.release(rl)
        srv.release(rs)
    finally:
        srv.stop()
