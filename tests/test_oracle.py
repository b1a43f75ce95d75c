"""The oracle (C++ restatement of the shader path) against its pins.

Pins, since the reference ships no tests or fixtures for this path:
  * tests/golden/rays.npz, written by a second, independent numpy float32
    restatement (tests/golden/np_restatement.py): bit-exact agreement on the
    transcendental-free fields;
  * known answers of Moeller-Trumbore on hand-built triangles;
  * WGSL quirks the shader relies on (rotateZ drops z, clamp(-1.0, 1.0, x)
    is min(1, x), the fp32 t-loop step count).
"""
from pathlib import Path

import numpy as np
import pytest

from linon_gb300 import _abi, camera as cam, scene, workloads as wl

GOLDEN = Path(__file__).resolve().parent / "golden" / "rays.npz"
FIELDS = ["identity", "linear", "lorenz", "roessler", "translation_x", "mirage_spherical", "mirage_plane"]


def golden_case(name):
    ref_xyz, ref_faces, _, center = scene.cornell_reference()
    unit_xyz, unit_faces, unit_rgb = scene.cornell_unit()
    fname = name.split("_", 1)[1]
    st = wl.settings()
    if name.startswith("reference_"):
        p = _abi.reference_params()
        return dict(xyz=ref_xyz, faces=ref_faces, rgb=None, W=48, H=40, camera=cam.arcball_default(center),
                    settings=st, params=p, field=_abi.FIELD_IDS[fname])
    st.field_weight = 0.75
    p = wl.fixed_steps(0.05, 80, kahan=True)
    return dict(xyz=unit_xyz, faces=unit_faces, rgb=unit_rgb, W=40, H=32, camera=cam.look_at((0.0, 0.0, 3.0)),
                settings=st, params=p, field=_abi.FIELD_IDS[fname])


@pytest.mark.parametrize("name", [f"{k}_{f}" for f in FIELDS for k in ("reference", "steps")])
def test_oracle_matches_golden_bit_exact(oracle, name):
    g = np.load(GOLDEN)
    c = golden_case(name)
    pix = g[f"{name}/pixels"]
    r = oracle.render(c["xyz"], c["faces"], c["rgb"], c["camera"], c["settings"], c["params"], c["field"],
                      c["W"], c["H"], pixels=pix)
    np.testing.assert_array_equal(r["hit_id"], g[f"{name}/hit_id"])
    np.testing.assert_array_equal(r["steps"], g[f"{name}/steps"])
    np.testing.assert_array_equal(r["mapping"].view(np.uint32), g[f"{name}/mapping"].view(np.uint32))
    np.testing.assert_array_equal(r["color"], g[f"{name}/color"])


def test_hit_triangle_known_answers(oracle):
    tri = [0, 0, 0, 1, 0, 0, 0, 1, 0]  # unit right triangle in z = 0
    assert oracle.hit_triangle(tri, [0.25, 0.25, 1.0, 0, 0, -1]) == pytest.approx(1.0)
    assert oracle.hit_triangle(tri, [0.25, 0.25, -2.0, 0, 0, 1]) == pytest.approx(2.0)
    assert oracle.hit_triangle(tri, [0.75, 0.75, 1.0, 0, 0, -1]) == -1.0   # u + v > 1
    assert oracle.hit_triangle(tri, [-0.1, 0.5, 1.0, 0, 0, -1]) == -1.0    # outside
    assert oracle.hit_triangle(tri, [0.25, 0.25, 1.0, 1, 0, 0]) == -1.0    # parallel (|a| < eps)
    assert oracle.hit_triangle(tri, [0.25, 0.25, -1.0, 0, 0, -1]) == -1.0  # behind (t < eps)
    # no back-face culling: both sides hit
    assert oracle.hit_triangle(tri, [0.2, 0.2, 0.5, 0, 0, -1]) == pytest.approx(0.5)
    # edge: u = 0 accepted
    assert oracle.hit_triangle(tri, [0.0, 0.5, 1.0, 0, 0, -1]) == pytest.approx(1.0)


def test_rotate_z_drops_z(oracle):
    # rotateZ's third column is zero (main_view.wgsl:94-100): Rotation field
    # normalize(v0 + rotateZ(v0, PI t)) at t = 0 is normalize(v0 + (vx, vy, 0)).
    x = np.zeros(13, np.float32)
    x[6:9] = (0.0, 0.0, 1.0)
    out = oracle.field_eval(_abi.FIELD_IDS["rotation"], x)
    np.testing.assert_allclose(out[0], [0.0, 0.0, 1.0])
    x[6:9] = (0.6, 0.0, 0.8)
    out = oracle.field_eval(_abi.FIELD_IDS["rotation"], x)
    v = np.array([1.2, 0.0, 0.8])
    np.testing.assert_allclose(out[0], v / np.linalg.norm(v), rtol=1e-6)


def test_t_loop_step_counts(oracle):
    """The fp32 `t <= 5.0` loop (main_view.wgsl:244,265) runs the count a
    float32 accumulation gives, not t_max/h + 1."""
    xyz, faces, _, center = scene.cornell_reference()
    for h in (0.1, 0.05, 0.01, 0.005):
        p = _abi.reference_params()
        p.h_initial = h
        p.adaptive = 0
        t, n = np.float32(0.0), 0
        while t <= np.float32(5.0):
            t = np.float32(t + np.float32(h))
            n += 1
        r = oracle.render(xyz, faces, None, cam.arcball_default(center), wl.settings(), p,
                          _abi.FIELD_IDS["linear"], 8, 8, pixels=[0])
        assert r["steps"][0] == n
    # worked example: 500 steps at h = 0.01 in f32 (exact arithmetic: 501)
    t, n = np.float32(0.0), 0
    while t <= np.float32(5.0):
        t = np.float32(t + np.float32(0.01))
        n += 1
    assert n == 500


def test_fp64_oracle_close_on_smooth_field(oracle):
    w = wl.frames_1080p(64, 36)
    r32 = oracle.render(w.xyz, w.faces, w.face_rgb, w.camera, w.settings, w.params, _abi.FIELD_IDS["twist"],
                        w.width, w.height)
    r64 = oracle.render(w.xyz, w.faces, w.face_rgb, w.camera, w.settings, w.params, _abi.FIELD_IDS["twist"],
                        w.width, w.height, precision=64, want=("mapping64", "hit_id"))
    err = np.abs(r32["mapping"][..., :3] - r64["mapping64"][..., :3]).max()
    assert err < 1e-4
    assert np.mean(r32["hit_id"] != r64["hit_id"]) <= 0.01


def test_outline_select_scans(oracle):
    # hand-made exponent map: the shader's 8 scans pick extremal pixels
    W = H = 9
    e = np.zeros((H, W), np.float32)
    pts = [(1, 1), (7, 1), (1, 7), (7, 7), (4, 2)]
    for x, y in pts:
        e[y, x] = 1.0
    sel = oracle.outline_select(e, W, H, 0.8)
    # bottom-left corner scan maximises (W - x) + y: (1, 7)
    assert tuple(sel[0]) == (1, 7)
    # bottom right maximises x + y: (7, 7)
    assert tuple(sel[2]) == (7, 7)
    # top right maximises x + (H - y): (7, 1)
    assert tuple(sel[4]) == (7, 1)
    # top left maximises (W - x) + (H - y): (1, 1)
    assert tuple(sel[6]) == (1, 1)
    # top middle: first in row-major order
    assert tuple(sel[5]) == (1, 1)
    # middle left: first in column-major order
    assert tuple(sel[7]) == (1, 1)
    # middle right: from the last column
    assert tuple(sel[3]) == (7, 1)
    # bottom middle: from the last row (y = W - 1)
    assert tuple(sel[1]) == (1, 7)
    # nothing above the threshold: all (0, 0)
    assert (oracle.outline_select(np.zeros((H, W), np.float32), W, H, 0.8) == 0).all()


def test_overlay_formula(oracle):
    """Lyapunov overlay: an endpoint map that is linear in x with slope s has
    largest singular value s/2 per central difference... exponent = s."""
    W, H = 12, 10
    xs = np.arange(W, dtype=np.float32)
    mapping = np.zeros((H, W, 4), np.float32)
    mapping[..., 0] = 0.01 * xs[None, :]
    mapping[..., 3] = 1
    rgba = np.full((H, W, 4), 100, np.uint8)
    st = wl.settings(overlay_mode=1, delta=1, scaling=50.0)
    out, e = oracle.overlay(rgba, mapping, W, H, st)
    # G = [0.5*(0.02), 0] -> M = diag(1e-4, 0) -> sqrt(max eig) = 0.01
    expect = np.float32(np.exp(np.float32(50.0) * np.float32(0.01) - np.float32(5.0)))
    assert e[5, 5] == pytest.approx(float(expect), rel=1e-5)
    assert e[0, 0] == 0.0  # border (2 * delta) untouched
    # below the 0.8 threshold: colour passes through
    assert (out[5, 5] == 100).all()
