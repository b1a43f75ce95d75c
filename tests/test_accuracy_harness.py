"""The accuracy checker itself (CPU): the oracle's candidate grid returns the
brute-force loop's results bit for bit, and the per-workload reports behave
as stated when fed the FP32 oracle's own planes in place of the engine's."""
import numpy as np
import pytest

from linon_gb300 import _abi, scene, workloads as wl


@pytest.fixture(scope="module")
def acc():
    from oracle import accuracy
    return accuracy


def _small_batch_scene():
    xyz, faces, rgb = scene.cornell_with_spheres(seed=0, subdivisions=3)
    w = wl.batch_uneven(8, seed=0)
    w.xyz, w.faces, w.face_rgb = xyz, faces, rgb
    return w


@pytest.mark.parametrize("precision", [32, 64])
def test_grid_equals_every_face(oracle, precision):
    # the sphere scene (4 x 1280-facet icospheres in the room): 6 views of the
    # uneven batch, 24 pixels each, all three fields, stop at the first hit
    w = _small_batch_scene()
    rng = np.random.default_rng(3)
    want = ("color", "mapping", "hit_id", "steps") if precision == 32 else ("color", "mapping64", "hit_id", "steps")
    hits = 0
    for (W, H, camera, params, fidx) in w.extra["views"][:6]:
        pix = np.sort(rng.choice(W * H, 24, replace=False)).astype(np.int32)
        args = (w.xyz, w.faces, w.face_rgb, camera, w.settings, params, w.fields[fidx], W, H)
        a = oracle.render(*args, pixels=pix, precision=precision, want=want, accel=True)
        b = oracle.render(*args, pixels=pix, precision=precision, want=want, accel=False)
        for k in a:
            np.testing.assert_array_equal(a[k].view(np.uint8), b[k].view(np.uint8), err_msg=k)
        hits += int((a["hit_id"] >= 0).sum())
    assert hits > 50


def test_grid_equals_every_face_full_frame_and_linear_mode(oracle):
    # the Cornell room alone, a whole frame, and linear mode (segments of
    # length 100 that span the grid: the loop over every face decides)
    w = wl.plain_small(48, 40)
    w.params = wl.fixed_steps(0.02, 200)
    args = (w.xyz, w.faces, w.face_rgb, w.camera, w.settings)
    for lin in (0, 1):
        w.params.linear_mode = lin
        a = oracle.render(*args, w.params, w.fields[0], w.width, w.height, accel=True)
        b = oracle.render(*args, w.params, w.fields[0], w.width, w.height, accel=False)
        for k in a:
            np.testing.assert_array_equal(a[k].view(np.uint8), b[k].view(np.uint8), err_msg=k)


def test_frame_report_of_the_fp32_oracle(oracle, acc):
    w = wl.frames_1080p(240, 135)
    w.params = wl.fixed_steps(0.02, 300, kahan=True)
    fid = _abi.FIELD_IDS["twist"]
    pix = acc.sample_pixels(w.width, w.height, 300, seed=1)
    o64, o32 = acc.oracle_pixels(w, fid, w.width, w.height, w.camera, w.params, pix)
    rep = acc.frame_report(o32, o64, o32, acc.FaceInfo(w.xyz, w.faces))
    assert rep["pixels"] == 300
    assert rep["endpoint_err"] == rep["endpoint_err_fp32_oracle"]
    assert rep["endpoint_err"]["max"] < 1e-4
    assert rep["equal_accuracy"]["ok"] and rep["equal_accuracy"]["ratio_engine_over_fp32"]["p50"] == 1.0
    assert rep["hit_mismatch"] == rep["hit_mismatch_fp32_oracle"]
    assert rep["rgba8_vs_fp64"]["max_lsb"] <= 1
    # a planted error (every endpoint moved by 1e-3) fails the smooth bar and
    # the equal-accuracy comparison
    bad = dict(o32)
    bad["mapping"] = o32["mapping"] + np.float32(1e-3)
    rep = acc.frame_report(bad, o64, o32, acc.FaceInfo(w.xyz, w.faces))
    assert rep["endpoint_err"]["max"] > 1e-4 and not rep["equal_accuracy"]["ok"]


def test_mismatch_classes(acc):
    xyz, faces, _ = scene.cornell_unit()
    info = acc.FaceInfo(xyz, faces)
    # faces 0/1: the two triangles of the floor quad (coplanar); 8/9: the
    # light panel and 6/7: the ceiling (coplanar, disjoint vertex sets);
    # floor 0 vs back wall 10 share the corner vertices (edge graze);
    # hit vs miss is "other"
    m = acc.hit_mismatch(np.array([0, 8, 0, 5, -1]), np.array([1, 6, 10, 5, 3]), info)
    assert m["total"] == pytest.approx(0.8)
    assert m["coplanar_tie"] == pytest.approx(0.4)
    assert m["edge_graze"] == pytest.approx(0.2)
    assert m["other"] == pytest.approx(0.2)


def test_batch_report_pools_views_per_field(oracle, acc):
    w = _small_batch_scene()
    views = [(min(W, 64), min(H, 48), cam, p, f) for (W, H, cam, p, f) in w.extra["views"][:4]]
    pix = [acc.sample_pixels(W, H, 20, seed=i) for i, (W, H, *_r) in enumerate(views)]
    eng = []
    for (W, H, camera, params, fidx), px in zip(views, pix):
        eng.append(oracle.render(w.xyz, w.faces, w.face_rgb, camera, w.settings, params, w.fields[fidx], W, H,
                                 pixels=px, accel=True))
    rep = acc.batch_report(w, views, eng, pix, {0: "linear", 1: "twist", 2: "lens"})
    assert sum(r["views"] for r in rep.values()) == 4
    assert sum(r["pixels"] for r in rep.values()) == 80
    for r in rep.values():
        assert r["equal_accuracy"]["ok"]


def test_lyapunov_report_of_the_fp32_oracle(oracle, acc):
    w = wl.lyapunov_1024(96, 80)
    w.params = wl.fixed_steps(0.01, 300, kahan=True)
    fid = w.fields[0]
    full = oracle.render(w.xyz, w.faces, w.face_rgb, w.camera, w.settings, w.params, fid, w.width, w.height)
    f = oracle.ftle(w.camera, w.params, w.width, w.height, full["mapping"], 3.0)
    _, e = oracle.overlay(full["color"], full["mapping"], w.width, w.height, wl.settings(overlay_mode=1),
                          precision=64)
    centres = acc.sample_pixels(w.width, w.height, 500, seed=2, border=2)
    thr = float(np.quantile(f[1:-1, 1:-1], 0.95))
    outline = oracle.outline_select(f, w.width, w.height, thr)
    rep = acc.lyapunov_report(w, fid, centres, f.ravel()[centres], e.ravel()[centres], thr, outline, 3.0)
    # the outline pixels (extremal pixels above the threshold, image borders
    # included) are above it under the FP64 exponent too
    assert rep["outline_pixels_checked"] >= 1
    assert rep["outline_pixels_above_engine_threshold_in_fp64"] >= rep["outline_pixels_checked"] - 1
    # the FP32 oracle's own maps: the finite-time exponent is the FP32
    # pipeline's (FP32 directions), so its error equals the FP32 column
    assert rep["ftle_abs_err"]["max"] <= rep["ftle_abs_err_fp32_oracle"]["max"] * 1.0001 + 1e-6
    assert rep["overlay_exponent_rel_err"]["p99"] < 1e-3
    assert rep["above_p95_agree"] > 0.98
