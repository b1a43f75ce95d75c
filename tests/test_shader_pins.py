"""The oracle against the reference's own shader source.

tests/golden/shader_pins.npz holds outputs of src/main_view.wgsl and
src/overlay.wgsl themselves (with the field bodies of src/functions.rs),
lowered through this package's WGSL front end with the resource bindings
replaced by private variables and run on the host; the script that wrote
it is tests/golden/make_shader_pins.py.  The oracle is a hand restatement
of the same shaders; these tests hold it to the shader text: ray
generation (main_view.wgsl:340-364), the march loop with adaptive
refinement (:229-279), the triangle test and shading (:150-220), the field
bodies and helpers, the high-accuracy source edit (src/main_view.rs:787),
linear mode, the ray samples (:281-314) from the mouse and from the
outline scans (:377-465), and the Lyapunov overlay (overlay.wgsl), both
entry points.
"""
from pathlib import Path

import numpy as np
import pytest

from linon_gb300 import _abi, camera as cam, scene, workloads as wl

PINS = Path(__file__).resolve().parent / "golden" / "shader_pins.npz"
FIELDS = ["identity", "mirage_spherical", "mirage_plane", "mirage_spherical_sigmoid", "mirage_plane_sigmoid",
          "translation_x", "translation_z", "rotation", "lorenz", "roessler"]
# Fields whose march uses +, -, *, /, sqrt only (the colour's specular pow
# aside) are compared bit for bit; the others call the host's sin, cos or
# exp on both sides (bit-exact with one libm, 1e-5 allowed across libms).
EXACT = {"identity", "mirage_plane", "translation_x", "translation_z", "lorenz", "roessler", "mirage_spherical"}
SAMPLE_OFFSETS = np.array([[-1, -1], [0, -1], [1, -1], [1, 0], [1, 1], [0, 1], [-1, 1], [-1, 0]], np.float32)


@pytest.fixture(scope="module")
def pins():
    return np.load(PINS)


def unorm8(c):
    """rgba8unorm store of the shader's float colour (clamp, scale, round
    half to even)."""
    return np.rint(np.clip(c, 0.0, 1.0).astype(np.float32) * np.float32(255.0)).astype(np.uint8)


def main_setup(g):
    xyz, faces, _, center = scene.cornell_reference()
    np.testing.assert_array_equal(xyz, g["scene/xyz"])
    np.testing.assert_array_equal(faces, g["scene/faces"])
    camera = cam.arcball_default(center)
    c = np.array(list(camera.origin) + list(camera.view_direction) + list(camera.up), np.float32)
    np.testing.assert_array_equal(c, g["scene/camera"])
    sf, si = g["main/settings_f"], g["main/settings_i"]
    st = wl.settings(overlay_mode=int(si[0]), delta=int(si[1]), scaling=float(sf[3]))
    st.field_weight = float(sf[0])
    st.mouse_pos[0], st.mouse_pos[1] = float(sf[1]), float(sf[2])
    return xyz, faces, camera, st


def test_scene_is_the_reference_box(pins):
    """scene.cornell_raw equals src/cornell_box.rs's VERTICES and INDICES
    (compared by the fixture script; here through the digest it stored)."""
    import hashlib
    xyz, faces, _ = scene.cornell_raw()
    digest = hashlib.sha256(xyz.astype(np.float32).tobytes() + faces.astype(np.uint32).tobytes()).hexdigest()
    assert digest == str(pins["scene/raw_sha256"])


def pixel_index(gids, W, H):
    return ((H - 1 - gids[:, 1]) * W + gids[:, 0]).astype(np.int32)


def check_mapping(field, got, want):
    if field in EXACT:
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    else:
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-5)


@pytest.mark.parametrize("field", FIELDS)
def test_main_view_frame(oracle, pins, field):
    xyz, faces, camera, st = main_setup(pins)
    gids = pins[f"view/{field}/gids"]
    W, H = 48, 40
    r = oracle.render(xyz, faces, None, camera, st, _abi.reference_params(), _abi.FIELD_IDS[field], W, H,
                      pixels=pixel_index(gids, W, H))
    check_mapping(field, r["mapping"], pins[f"view/{field}/mapping"])
    np.testing.assert_array_equal(r["color"], unorm8(pins[f"view/{field}/color"]))


@pytest.mark.parametrize("field", ["lorenz", "mirage_spherical"])
def test_main_view_high_accuracy(oracle, pins, field):
    xyz, faces, camera, st = main_setup(pins)
    p = _abi.reference_params()
    p.h_initial = 0.001
    gids = pins[f"high/{field}/gids"]
    r = oracle.render(xyz, faces, None, camera, st, p, _abi.FIELD_IDS[field], 48, 40,
                      pixels=pixel_index(gids, 48, 40))
    check_mapping(field, r["mapping"], pins[f"high/{field}/mapping"])
    np.testing.assert_array_equal(r["color"], unorm8(pins[f"high/{field}/color"]))


def test_main_view_linear_mode(oracle, pins):
    xyz, faces, camera, st = main_setup(pins)
    p = _abi.reference_params()
    p.linear_mode = 1
    gids = pins["linear/identity/gids"]
    r = oracle.render(xyz, faces, None, camera, st, p, _abi.FIELD_IDS["identity"], 48, 40,
                      pixels=pixel_index(gids, 48, 40), want=("color",))
    np.testing.assert_array_equal(r["color"], unorm8(pins["linear/identity/color"]))


@pytest.mark.parametrize("field", ["identity", "lorenz", "roessler", "mirage_spherical", "rotation"])
def test_ray_samples_from_mouse(oracle, pins, field):
    _, _, camera, st = main_setup(pins)
    mouse = np.array(st.mouse_pos, np.float32)
    pos = (mouse + np.float32(0.01) * SAMPLE_OFFSETS).astype(np.float32)
    got = oracle.capture(_abi.FIELD_IDS[field], camera, st, _abi.reference_params(), 48, 40, pos, 0.001, 5000, 50,
                         False)
    check_mapping(field, got, pins[f"view/{field}/samples"])


def test_ray_samples_from_outline(oracle, pins):
    _, _, camera, st = main_setup(pins)
    e = pins["outline/lorenz/exponents"]
    S = e.shape[0]
    sel = oracle.outline_select(e, S, S, 0.8, stride=S).astype(np.float32)
    pos = np.stack([sel[:, 0] / np.float32(S - 1), (np.float32(S - 1) - sel[:, 1]) / np.float32(S - 1)],
                   axis=1).astype(np.float32)
    got = oracle.capture(_abi.FIELD_IDS["lorenz"], camera, st, _abi.reference_params(), S, S, pos, 0.001, 5000, 50,
                         False)
    np.testing.assert_array_equal(got.view(np.uint32), pins["outline/lorenz/samples"].view(np.uint32))


@pytest.mark.parametrize("case", ["desktop_d1", "desktop_d2", "web_d1"])
def test_overlay(oracle, pins, case):
    rgba8, mp = pins["overlay/rgba8"], pins["overlay/mapping"]
    H, W = rgba8.shape[:2]
    sf, si = pins[f"overlay/{case}/settings_f"], pins[f"overlay/{case}/settings_i"]
    st = wl.settings(overlay_mode=int(si[0]), delta=int(si[1]), scaling=float(sf[3]))
    e = np.full((H, W), -1.0, np.float32)
    out, e = oracle.overlay(rgba8, mp, W, H, st, srgb=bool(pins[f"overlay/{case}/web"]), exponents=e)
    want_e = pins[f"overlay/{case}/exponents"]
    np.testing.assert_array_equal(e.view(np.uint32), want_e.view(np.uint32))  # -1 where nothing was written
    np.testing.assert_array_equal(out, unorm8(pins[f"overlay/{case}/color"]))


@pytest.mark.gpu
@pytest.mark.parametrize("field", ["identity", "lorenz", "roessler", "translation_x", "mirage_plane"])
def test_engine_equals_shader_source(engine, pins, field):
    """The CUDA engine (precise module, through the C ABI) against the
    shader-source fixtures directly: endpoints bit for bit, colour within
    1/255 (the specular pow is CUDA's)."""
    import torch
    from linon_gb300 import FramePlanes
    from linon_gb300.engine import predefined_source
    xyz, faces, camera, st = main_setup(pins)
    engine.upload_scene(xyz, faces, None, bvh=True)
    fld = engine.compile_field(predefined_source(_abi.FIELD_IDS[field]), precise=True)
    W, H = 48, 40
    planes = FramePlanes.allocate(W, H)
    engine.render(fld, camera, st, _abi.reference_params(), planes)
    engine.synchronize()
    torch.cuda.synchronize()
    pix = pixel_index(pins[f"view/{field}/gids"], W, H)
    mapping = planes.mapping.cpu().numpy().reshape(-1, 4)[pix]
    color = planes.color.cpu().numpy().reshape(-1, 4)[pix]
    np.testing.assert_array_equal(mapping.view(np.uint32), pins[f"view/{field}/mapping"].view(np.uint32))
    want = unorm8(pins[f"view/{field}/color"]).astype(np.int32)
    assert np.abs(color.astype(np.int32) - want).max() <= 1
