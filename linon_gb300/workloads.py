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
* obj_scene: an OBJ file (raw Cornell box triangles, a quad torus, a hexagon
  and a pentagon) loaded the way a dropped file is (tobj triangulation,
  normalize_vertices, get_center, arcball default camera), the shader's own
  loop.
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
    p = _abi.shader_params()
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
                    settings(), _abi.shader_params(), [field])


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


def obj_scene_text() -> str:
    """OBJ text of the obj_scene workload: the raw Cornell box (triangles),
    a tilted quad torus inside it, a hexagon on the back wall and a pentagon
    on the floor (fans); two models: "o cornell" and "g torus" (torus,
    hexagon, pentagon), plus a trailing empty object."""
    v, f, _ = scene.cornell_raw()
    tv, tq = scene.torus(center=(278.0, 200.0, 280.0), R=120.0, r=40.0)
    lines = ["# obj_scene: Cornell box, torus, hexagon, pentagon", "o cornell"]
    lines += [f"v {a!r} {b!r} {c!r}" for a, b, c in v.astype(float).tolist()]
    lines += [f"f {a + 1} {b + 1} {c + 1}" for a, b, c in f.tolist()]
    lines.append("g torus")
    lines += [f"v {a!r} {b!r} {c!r}" for a, b, c in tv.astype(float).tolist()]
    lines += ["f " + " ".join(f"{-(len(tv) - k)}" for k in q) for q in tq.tolist()]  # relative indices
    ang = np.arange(6) * np.pi / 3
    hexv = np.stack([278 + 60 * np.cos(ang), 380 + 60 * np.sin(ang), np.full(6, 555.0)], -1)
    lines += [f"v {a!r} {b!r} {c!r}" for a, b, c in hexv.tolist()]
    lines.append("f " + " ".join(str(-6 + k) for k in range(6)))
    ang5 = np.arange(5) * 2 * np.pi / 5
    pentv = np.stack([150 + 50 * np.cos(ang5), np.full(5, 0.5), 420 + 50 * np.sin(ang5)], -1)
    lines += [f"v {a!r} {b!r} {c!r}" for a, b, c in pentv.tolist()]
    lines.append("f " + " ".join(str(-5 + k) for k in range(5)))
    lines.append("o trailing_empty")
    return "\n".join(lines) + "\n"


def obj_scene(width=256, height=192, model: int = 0, text: str | None = None) -> Workload:
    """The OBJ scene as the reference's dropped-file path loads it: the first
    model (\"o cornell\" ends at \"g torus\", so model 0 is the box alone;
    model=1 is the torus with the two panels)."""
    m = scene.parse_obj(text or obj_scene_text(), model=model, normalize=True)
    return Workload(f"obj_scene_model{model}_{width}x{height}", m.xyz, m.faces, None, width, height,
                    cam.arcball_default(m.center), settings(), _abi.shader_params(),
                    [_abi.FIELD_IDS["mirage_spherical_sigmoid"]], extra={"n_models": m.n_models})
