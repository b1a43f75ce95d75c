"""Host-side logic: scene preparation, cameras, workloads (CPU)."""
import numpy as np
import pytest

from linon_gb300 import _abi, camera as cam, scene, workloads as wl


def test_cornell_reference_prep():
    """application.rs:105-123 + vertices.rs: one global normalisation after
    negating x and z; bounding box and centre as computed independently."""
    xyz, faces, rgb, center = scene.cornell_reference()
    assert xyz.shape == (72, 3) and faces.shape == (36, 3)
    assert xyz.dtype == np.float32
    lo, hi = xyz.min(axis=0), xyz.max(axis=0)
    np.testing.assert_allclose(lo, [-0.9942, 0.0094, -1.0], atol=1e-4)
    np.testing.assert_allclose(hi, [0.0094, 1.0, 0.0094], atol=1e-4)
    np.testing.assert_allclose(center, [-0.4924, 0.5047, -0.4953], atol=1e-4)
    assert xyz.min() == -1.0 and xyz.max() == 1.0


def test_cornell_faces_follow_quads():
    _, faces, rgb = scene.cornell_raw()
    np.testing.assert_array_equal(faces[:4], [[0, 1, 2], [2, 3, 0], [4, 5, 6], [6, 7, 4]])
    assert faces.max() == 71
    # green (quad 6) and red (quad 7) walls differ from each other and white
    assert tuple(rgb[12]) != tuple(rgb[14]) and tuple(rgb[12]) != tuple(rgb[0])


def test_cornell_unit_is_the_unit_room():
    xyz, _, _ = scene.cornell_unit()
    np.testing.assert_array_equal(xyz.min(axis=0), [-1, -1, -1])
    np.testing.assert_array_equal(xyz.max(axis=0), [1, 1, 1])


def test_icosphere_and_spheres_scene():
    x, f = scene.icosphere(5, 0.3, (0.1, 0.2, 0.3))
    assert len(f) == 20480
    r = np.linalg.norm(x.astype(np.float64) - [0.1, 0.2, 0.3], axis=1)
    np.testing.assert_allclose(r, 0.3, rtol=1e-6)
    a = scene.cornell_with_spheres(seed=0)
    b = scene.cornell_with_spheres(seed=0)
    assert len(a[1]) == 36 + 4 * 20480
    np.testing.assert_array_equal(a[0], b[0])


def test_coplanar_groups():
    xyz, faces, _, _ = scene.cornell_reference()
    g = scene.coplanar_groups(xyz, faces)
    assert g[6] == g[8]      # ceiling and light panel
    assert g[0] == g[2]      # floor and short-block footprint
    assert g[0] != g[6]


def test_arcball_default_matches_reference_construction():
    xyz, faces, _, center = scene.cornell_reference()
    a = cam.Arcball(center, 1.0, (512, 512))
    a.zoom(-1.0, 1.0)
    np.testing.assert_allclose(a.eye_pos(), center + [0, 0, 2], atol=1e-6)
    np.testing.assert_allclose(a.eye_dir(), [0, 0, -1], atol=1e-6)
    np.testing.assert_allclose(a.up_dir(), [0, 1, 0], atol=1e-6)
    c = cam.arcball_default(center)
    np.testing.assert_allclose(list(c.origin)[:3], a.eye_pos(), atol=1e-6)
    # rotating moves the eye on the sphere around the centre
    a.rotate((256, 256), (300, 256))
    assert abs(np.linalg.norm(a.eye_pos() - center) - 2.0) < 1e-4


def _angle(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.arccos(np.clip(np.dot(a, b) / np.linalg.norm(a) / np.linalg.norm(b), -1.0, 1.0)))


def test_arcball_rotate_is_twice_the_ball_angle():
    """Shoemake's arcball (src/arcball.rs rotate): dragging from the ball
    point p to q turns the camera by twice the angle between p and q about
    p x q; a drag that starts and ends at the same point changes nothing."""
    center = np.array([0.5, -0.25, 0.1], np.float32)
    a = cam.Arcball(center, 1.0, (400, 300))
    eye0, dir0, up0 = a.eye_pos(), a.eye_dir(), a.up_dir()
    a.rotate((123, 77), (123, 77))
    np.testing.assert_allclose(a.eye_pos(), eye0, atol=1e-6)
    np.testing.assert_allclose(a.up_dir(), up0, atol=1e-6)
    # horizontal drag through the middle row: ball points (0, 0, 1) and
    # (x, 0, sqrt(1 - x^2)), angle asin(x); the eye turns about the y axis
    x = 0.3
    a.rotate((200, 150), (200 + x * 200, 150))
    np.testing.assert_allclose(_angle(a.eye_dir(), dir0), 2 * np.arcsin(x), atol=2e-6)
    np.testing.assert_allclose(a.up_dir(), up0, atol=1e-6)
    assert abs(np.linalg.norm(a.eye_pos() - center) - 1.0) < 1e-5
    assert abs(a.eye_pos()[1] - eye0[1]) < 1e-6
    # a drag from the centre to the right edge ends on the ball's rim
    # (1, 0, 0): a quarter turn between the ball points, a half turn of
    # the camera
    b = cam.Arcball(center, 1.0, (400, 300))
    b.rotate((200, 150), (400, 150))
    np.testing.assert_allclose(_angle(b.eye_dir(), dir0), np.pi, atol=1e-5)


def test_arcball_zoom_pan_and_resize():
    center = np.array([0.0, 0.0, 0.0], np.float32)
    a = cam.Arcball(center, 2.0, (640, 480))
    a.zoom(0.25, 0.5)  # towards the centre by amount * speed * elapsed
    np.testing.assert_allclose(a.eye_pos(), [0, 0, 0.75], atol=1e-6)
    # pan scales the pixel delta by |translation[3][3]|, which is 1 for a
    # translation matrix (the reference reads the w of the translation
    # column), so a full-width drag moves the view by one unit whatever the
    # zoom; the eye moves against the drag
    a.pan((64, 0))
    np.testing.assert_allclose(a.eye_pos(), [-0.1, 0, 0.75], atol=1e-6)
    np.testing.assert_allclose(a.eye_dir(), [0, 0, -1], atol=1e-6)
    a.pan((0, -48))
    np.testing.assert_allclose(a.eye_pos(), [-0.1, -0.1, 0.75], atol=1e-6)
    a.update_screen(320, 240)
    a.pan((32, 0))
    np.testing.assert_allclose(a.eye_pos(), [-0.2, -0.1, 0.75], atol=1e-6)
    u = a.uniform()
    np.testing.assert_allclose(list(u.origin)[:3], a.eye_pos(), atol=1e-7)


def test_batch_views_seeded():
    v1 = wl.batch_views(64, seed=0)
    v2 = wl.batch_views(64, seed=0)
    assert [(a[0], a[1], a[3].h_initial, a[4]) for a in v1] == [(a[0], a[1], a[3].h_initial, a[4]) for a in v2]
    sides = np.array([(a[0], a[1]) for a in v1])
    assert sides.min() >= 128 and sides.max() <= 1024
    for (_, _, c, p, _) in v1:
        assert abs(np.linalg.norm(list(c.origin)[:3]) - 3.0) < 1e-5
        assert p.max_steps == round(4.0 / p.h_initial)
        assert p.stop_on_hit == 1


def test_fov_params():
    p = cam.fov_params(_abi.reference_params(), 45.0)
    assert p.focal_length == 1.0
    assert p.viewport_height == pytest.approx(2 * np.tan(np.radians(22.5)), rel=1e-6)
