"""Camera construction for the ray-cast pass.

* `arcball_default(center)` is the camera MainView starts with
  (src/main_view.rs:153-155: ArcballCamera::new(center) then zoom(-1, 1),
  src/arcball.rs:33-68): eye = center + (0, 0, 2), looking down -z, up +y.
* `Arcball` restates the Shoemake arcball of src/arcball.rs (rotate, pan,
  zoom) in float32 so interactive clients can drive the engine like the UI.
* `look_at` builds the camera of the benchmark workloads (pinhole with an
  explicit vertical field of view).
"""
from __future__ import annotations

import math

import numpy as np

from . import _abi

REFERENCE_FOCAL = 0.035     # main_view.wgsl:355
REFERENCE_VIEWPORT = 0.025  # main_view.wgsl:356


def make_camera(origin, view_direction, up) -> _abi.Camera:
    c = _abi.Camera()
    for i in range(3):
        c.origin[i] = float(np.float32(origin[i]))
        c.view_direction[i] = float(np.float32(view_direction[i]))
        c.up[i] = float(np.float32(up[i]))
    for i in range(4):
        c.view_matrix[5 * i] = 1.0  # identity, as CameraUniform::moving writes
    return c


def arcball_default(center) -> _abi.Camera:
    c = np.asarray(center, dtype=np.float32)
    eye = (c + np.asarray([0.0, 0.0, 2.0], dtype=np.float32)).astype(np.float32)
    return make_camera(eye, (0.0, 0.0, -1.0), (0.0, 1.0, 0.0))


def look_at(eye, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)) -> _abi.Camera:
    eye = np.asarray(eye, dtype=np.float64)
    d = np.asarray(target, dtype=np.float64) - eye
    d = d / np.linalg.norm(d)
    u = np.asarray(up, dtype=np.float64)
    if abs(float(np.dot(d, u / np.linalg.norm(u)))) > 0.999:
        u = np.array([0.0, 0.0, 1.0]) if abs(d[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
    return make_camera(eye, d, u)


def fov_params(params: _abi.MarchParams, vfov_deg: float) -> _abi.MarchParams:
    """Pinhole with the given vertical field of view: focal 1, viewport 2 tan(fov/2)."""
    params.focal_length = 1.0
    params.viewport_height = float(np.float32(2.0 * math.tan(math.radians(vfov_deg) / 2.0)))
    return params


def _quat_mul(a, b):
    w1, x1, y1, z1 = a
    w2, x2, y2, z2 = b
    return np.array([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2,
                     w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                     w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2,
                     w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2], dtype=np.float32)


def _quat_to_mat4(q):
    w, x, y, z = [float(v) for v in q]
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y), 0],
        [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x), 0],
        [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y), 0],
        [0, 0, 0, 1]], dtype=np.float32)


def _translation(v):
    m = np.eye(4, dtype=np.float32)
    m[:3, 3] = np.asarray(v, dtype=np.float32)
    return m


class Arcball:
    """Shoemake arcball (src/arcball.rs:33-130): camera = translation *
    rotation * center_translation; eye/dir/up from its inverse."""

    def __init__(self, center, zoom_speed: float, screen):
        self.center = np.asarray(center, dtype=np.float32)
        self.translation = _translation((0.0, 0.0, -1.0))
        self.center_translation = _translation(-self.center)
        self.rotation = np.array([1.0, 0.0, 0.0, 0.0], dtype=np.float32)
        self.zoom_speed = np.float32(zoom_speed)
        self.inv_screen = [np.float32(1.0) / np.float32(screen[0]), np.float32(1.0) / np.float32(screen[1])]
        self._update()

    def _update(self):
        self.camera = self.translation @ _quat_to_mat4(self.rotation) @ self.center_translation
        self.inv_camera = np.linalg.inv(self.camera.astype(np.float64)).astype(np.float32)

    def eye_pos(self):
        return self.inv_camera[:3, 3].copy()

    def eye_dir(self):
        d = self.inv_camera @ np.array([0, 0, -1, 0], dtype=np.float32)
        return (d[:3] / np.linalg.norm(d[:3])).astype(np.float32)

    def up_dir(self):
        d = self.inv_camera @ np.array([0, 1, 0, 0], dtype=np.float32)
        return (d[:3] / np.linalg.norm(d[:3])).astype(np.float32)

    @staticmethod
    def _screen_to_arcball(p):
        dist = float(np.dot(p, p))
        if dist <= 1.0:
            return np.array([0.0, p[0], p[1], math.sqrt(1.0 - dist)], dtype=np.float32)
        u = p / np.linalg.norm(p)
        return np.array([0.0, u[0], u[1], 0.0], dtype=np.float32)

    def rotate(self, mouse_prev, mouse_cur):
        def to_ndc(m):
            return np.array([np.clip(m[0] * 2 * self.inv_screen[0] - 1, -1, 1),
                             np.clip(1 - 2 * m[1] * self.inv_screen[1], -1, 1)], dtype=np.float32)
        cur = self._screen_to_arcball(to_ndc(mouse_cur))
        prev = self._screen_to_arcball(to_ndc(mouse_prev))
        self.rotation = _quat_mul(_quat_mul(cur, prev), self.rotation)
        self._update()

    def zoom(self, amount: float, elapsed: float):
        motion = np.array([0.0, 0.0, amount], dtype=np.float32) * self.zoom_speed * np.float32(elapsed)
        self.translation = _translation(motion) @ self.translation
        self._update()

    def pan(self, mouse_delta):
        zoom_dist = abs(float(self.translation[3, 3]))
        delta = np.array([mouse_delta[0] * self.inv_screen[0], -mouse_delta[1] * self.inv_screen[1], 0, 0],
                         dtype=np.float32) * np.float32(zoom_dist)
        motion = self.inv_camera @ delta
        self.center_translation = _translation(motion[:3]) @ self.center_translation
        self._update()

    def update_screen(self, width: float, height: float):
        """The window was resized (src/arcball.rs update_screen)."""
        self.inv_screen = [np.float32(1.0) / np.float32(width), np.float32(1.0) / np.float32(height)]

    def uniform(self) -> _abi.Camera:
        """CameraUniform::moving (src/main_view.rs:21-31)."""
        return make_camera(self.eye_pos(), self.eye_dir(), self.up_dir())
