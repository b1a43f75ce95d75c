"""The workloads the engine is measured and checked on (synthetic, seeded).

* reference_default: the reference application's own first frame (Cornell box
  prepared as src/application.rs:105-123, arcball default camera, the
  shader's t <= 5 loop with h = 0.1 and adaptive refinement, Mirage
  (spherical sigmoid) field, field_weight 1).
* plain_small (512^2, twist, h 0.01, 1000 steps), frames_1080p (1920x1080,
  linear / twist / lens fields, h 0.005, 4000 steps, Kahan sums),
  lyapunov_1024 (1024^2, scaled Lorenz + v0, h 0.002, 2000 steps, T = 4),
  batch_uneven (64 seeded views, 128^2..1024^2 log-uniform, cameras on the
  radius-3 sphere, h in {0.02, 0.01, 0.005}, 4/h steps, Cornell room + four
  20,480-triangle icospheres behind the BVH, stop at the first hit).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field as dfield

import numpy as np

from . import _abi, camera as cam, scene

TWIST = "return rotateY(v0, 0.5 * p.y);"


def settings(field_weight=1.0, mouse=(0.5, 0.6), overlay_mode=0, delta=1, scaling=50.0) -> _abi.Settings:
    s = _abi.Settings()
    s.field_weight = field_weight
    s.mouse_pos[0], s.mouse_pos[1] = mouse
    s.overlay_mode = overlay_mode
    s.central_difference_delta = delta
    s.lyapunov_scaling = scaling
    return s


def fixed_steps(h: float, steps: int, kahan: bool = False, stop_on_hit: bool = False,
                vfov: float = 45.0) -> _abi.MarchParams:
    p = _abi.reference_params()
    p.h_initial = h
    p.max_steps = steps
    p.adaptive = 0
    p.kahan = 1 if kahan else 0
    p.stop_on_hit = 1 if stop_on_hit else 0
    return cam.fov_params(p, vfov)


@dataclass
class Workload:
    name: str
    xyz: np.ndarray
    faces: np.ndarray
    face_rgb: np.ndarray | None
    width: int
    height: int
    camera: _abi.Camera
    settings: _abi.Settings
    params: _abi.MarchParams
    fields: list = dfield(default_factory=list)  # predefined ids
    bvh: bool = True
    extra: dict = dfield(default_factory=dict)


def reference_default(width=512, height=512, field=_abi.FIELD_IDS["mirage_spherical_sigmoid"]) -> Workload:
    xyz, faces, _, center = scene.cornell_reference()
    return Workload("reference_default", xyz, faces, None, width, height, cam.arcball_default(center),
                    settings(), _abi.reference_params(), [field])


def plain_small(width=512, height=512) -> Workload:
    xyz, faces, rgb = scene.cornell_unit()
    return Workload("cornell_512_twist_h0.01x1000", xyz, faces, rgb, width, height,
                    cam.look_at((0.0, 0.0, 3.0)), settings(), fixed_steps(0.01, 1000),
                    [_abi.FIELD_IDS["twist"]])


def frames_1080p(width=1920, height=1080) -> Workload:
    xyz, faces, rgb = scene.cornell_unit()
    return Workload("cornell_1920x1080_linear_twist_lens_h0.005x4000_kahan", xyz, faces, rgb, width, height,
                    cam.look_at((0.0, 0.0, 3.0)), settings(), fixed_steps(0.005, 4000, kahan=True),
                    [_abi.FIELD_IDS["linear"], _abi.FIELD_IDS["twist"], _abi.FIELD_IDS["lens"]])


def lyapunov_1024(width=1024, height=1024) -> Workload:
    xyz, faces, rgb = scene.cornell_unit()
    return Workload("cornell_1024_lorenz_scaled_h0.002x2000_ftle", xyz, faces, rgb, width, height,
                    cam.look_at((0.0, 0.0, 3.0)), settings(overlay_mode=1), fixed_steps(0.002, 2000, kahan=True),
                    [_abi.FIELD_IDS["lorenz_scaled"]], extra={"T": 4.0, "quantile": 0.95})


def batch_views(n_views=64, seed=0, min_side=128, max_side=1024, hs=(0.02, 0.01, 0.005),
                n_fields=3):
    """Seeded view list: (width, height, camera, params, field_index)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_views):
        w, h = [int(round(math.exp(rng.uniform(math.log(min_side), math.log(max_side))))) for _ in range(2)]
        d = rng.normal(size=3)
        eye = 3.0 * d / np.linalg.norm(d)
        step = float(hs[int(rng.integers(len(hs)))])
        steps = int(round(4.0 / step))
        fidx = int(rng.integers(n_fields))
        out.append((w, h, cam.look_at(eye), fixed_steps(step, steps, kahan=True, stop_on_hit=True), fidx))
    return out


def batch_uneven(n_views=64, seed=0) -> Workload:
    xyz, faces, rgb = scene.cornell_with_spheres(seed=seed)
    w = Workload("batch64_uneven_cornell+4icospheres_bvh", xyz, faces, rgb, 0, 0, None, settings(), None,
                 [_abi.FIELD_IDS["linear"], _abi.FIELD_IDS["twist"], _abi.FIELD_IDS["lens"]])
    w.extra["views"] = batch_views(n_views, seed)
    return w
