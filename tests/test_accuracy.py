"""Fast-module results against the FP64 oracle on every benchmarked workload (GPU).

Each test renders the workload exactly as bench.py does (fast module, full
size, the benchmark's march parameters), samples seeded pixels, and holds
them to the FP64 oracle (oracle/accuracy.py), with the FP32 oracle's own
error on the same pixels beside it.  Tolerances, stated per test:

  * smooth fields (linear, twist, the scaled Lorenz field): endpoint error
    <= 1e-4 scene units (Euclidean) on every sampled pixel; hit-id mismatch
    outside rounding ties (coplanar faces, facets sharing an edge) <= 0.1%;
    RGBA8 within 1/255 on pixels whose hit ids agree;
  * the point-lens field, whose orbits around the origin are chaotic (the
    FP32 oracle itself is 5e-3 from FP64 at the median): equal accuracy --
    each of the engine's p50 / p90 / p99 endpoint errors within 1e-4 or at
    most 1.25x the FP32 oracle's on the same pixels -- and hit mismatch
    outside ties no more than the FP32 oracle's plus 0.1%;
  * Lyapunov: finite-time exponent and scaled overlay exponent from FP64
    endpoints of each sampled pixel and its four neighbours (the exponent
    within 1e-4 absolute, or no worse than 1.25x the FP32 oracle's error);
    the p95 threshold on the sample within 1e-3 of the FP64 one.
"""
import numpy as np
import pytest
import torch

from linon_gb300 import FramePlanes, _abi, lyapunov, workloads as wl
from linon_gb300.engine import predefined_source

pytestmark = pytest.mark.gpu

SMOOTH_TOL = 1e-4
TIE_FREE_MISMATCH = 1e-3
FIELD_NAMES = {_abi.FIELD_IDS["linear"]: "linear", _abi.FIELD_IDS["twist"]: "twist",
               _abi.FIELD_IDS["lens"]: "lens", _abi.FIELD_IDS["lorenz_scaled"]: "lorenz_scaled"}


@pytest.fixture(scope="module")
def acc():
    from oracle import accuracy
    return accuracy


def _render(engine, w, fid):
    fld = engine.compile_field(predefined_source(fid))
    planes = FramePlanes.allocate(w.width, w.height)
    engine.render(fld, w.camera, w.settings, w.params, planes)
    engine.synchronize()
    torch.cuda.synchronize()
    return planes


def _check_frame(rep, name):
    mism = rep["hit_mismatch"]
    if name == "lens":
        assert rep["equal_accuracy"]["ok"], rep["equal_accuracy"]
        assert mism["other"] <= rep["hit_mismatch_fp32_oracle"]["other"] + TIE_FREE_MISMATCH, mism
    else:
        assert rep["endpoint_err"]["max"] <= SMOOTH_TOL, rep["endpoint_err"]
        assert mism["other"] <= TIE_FREE_MISMATCH, mism
        assert rep["rgba8_vs_fp64"]["max_lsb"] <= 1, rep["rgba8_vs_fp64"]


@pytest.mark.parametrize("name", ["linear", "twist", "lens"])
def test_frames_1080p_fast_vs_fp64(engine, acc, name):
    """1920x1080, h = 0.005 x 4000 steps, Kahan sums: 4000 seeded pixels."""
    w = wl.frames_1080p()
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fid = _abi.FIELD_IDS[name]
    planes = _render(engine, w, fid)
    pix = acc.sample_pixels(w.width, w.height, 4000, seed=11)
    rep = acc.frame_pixels_report(w, fid, planes.sample(pix), pix)
    assert (planes.steps == 4000).all()
    _check_frame(rep, name)


def test_plain_512_twist_fast_vs_fp64(engine, acc):
    """512x512 twist, h = 0.01 x 1000 steps, per-face colours: 4000 pixels."""
    w = wl.plain_small()
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fid = w.fields[0]
    planes = _render(engine, w, fid)
    pix = acc.sample_pixels(w.width, w.height, 4000, seed=5)
    rep = acc.frame_pixels_report(w, fid, planes.sample(pix), pix)
    _check_frame(rep, "twist")


def test_lyapunov_1024_fast_vs_fp64(engine, acc):
    """1024x1024 scaled Lorenz + v0, h = 0.002 x 2000 steps (T = 4), the
    full pipeline with the fast module: 4000 interior centres."""
    w = wl.lyapunov_1024()
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fid = w.fields[0]
    fld = engine.compile_field(predefined_source(fid))
    r = lyapunov.run(engine, fld, w, horizon=w.extra["T"], quantile=w.extra["quantile"])
    centres = acc.sample_pixels(w.width, w.height, 4000, seed=23, border=2)
    idx = torch.as_tensor(centres.astype(np.int64), device="cuda")
    e_ftle = r["ftle"].reshape(-1)[idx].cpu().numpy()
    e_expo = r["exponents"].reshape(-1)[idx].cpu().numpy()
    rep = acc.lyapunov_report(w, fid, centres, e_ftle, e_expo, r["threshold"], r["outline_pixels"], w.extra["T"],
                              engine_px=r["planes"].sample(centres), info=acc.FaceInfo(w.xyz, w.faces))
    _check_frame(rep["frame"], "lorenz_scaled")
    # finite-time exponent: within 1e-4 (absolute) at every quantile, or no
    # worse than 1.25x the FP32 oracle's own error
    assert rep["ftle_equal_accuracy"]["ok"], (rep["ftle_abs_err"], rep["ftle_abs_err_fp32_oracle"])
    assert rep["p95_on_sample"]["abs_diff"] <= 1e-3, rep["p95_on_sample"]
    assert rep["above_p95_agree"] >= 0.995, rep["above_p95_agree"]
    assert rep["overlay_exponent_rel_err"]["p99"] <= 1e-3, rep["overlay_exponent_rel_err"]
    assert rep["overlay_blend_decision_agree"] >= 0.999
    assert rep["outline_pixels_above_engine_threshold_in_fp64"] >= rep["outline_pixels_checked"] - 1


@pytest.mark.parametrize("schedule", [0, 1, 3])
def test_batch_uneven_64_fast_vs_fp64(engine, acc, schedule):
    """The 64 uneven views (Cornell room + four 20,480-triangle icospheres
    behind the BVH, stop at the first hit), rendered by one batched launch
    (schedule 0: the default, one CTA per tile; 1: the persistent queue of
    warp tiles; 3: the persistent queue of CTA tiles): 200 seeded pixels per
    view against the oracle, whose candidate grid returns the brute-force
    loop's hits."""
    w = wl.batch_uneven(64, seed=0)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    flds = [engine.compile_field(predefined_source(fid)) for fid in w.fields]
    views, planes = [], []
    for (W, H, camera, params, fidx) in w.extra["views"]:
        p = FramePlanes.allocate(W, H)
        v = _abi.View()
        v.camera, v.settings, v.params = camera, wl.settings(), params
        v.width, v.height, v.field_index = W, H, fidx
        v.out = p.abi()
        views.append(v)
        planes.append(p)
    tuning = None if schedule == 0 else _abi.BatchTuning(1024, 128, 0, 4, 8, 0, schedule)
    engine.render_batch(flds, views, tuning)
    engine.synchronize()
    torch.cuda.synchronize()
    pix = [acc.sample_pixels(W, H, 200, seed=100 + i) for i, (W, H, *_r) in enumerate(w.extra["views"])]
    eng = [p.sample(px) for p, px in zip(planes, pix)]
    names = {i: FIELD_NAMES[f] for i, f in enumerate(w.fields)}
    rep = acc.batch_report(w, w.extra["views"], eng, pix, names)
    assert set(rep) == {"linear", "twist", "lens"}
    for name, r in rep.items():
        _check_frame(r, name)
        if name != "lens":  # the step of the first hit
            assert r["steps_equal_fp64"] >= 0.99, (name, r["steps_equal_fp64"])
