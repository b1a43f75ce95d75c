"""`MainView` with the reference's method names (src/main_view.rs:53-849).

The reference's MainView owns the ray-casting, mapping and output textures,
the exponents buffer, the camera/settings uniforms and the compute
pipelines, and dispatches the ray-cast pass followed by the overlay pass.
This class owns the same state on the GPU (torch CUDA tensors as storage,
every pass through liblinon.so) so a host written against the reference's
MainView finds the same calls:

    reload_shader(new_src, field_function)   # main_view.rs:649-690
    update_settings(settings)                 # :547-550
    update_camera() / update_model(...)       # :460-545
    resize_texture(width, height)             # :552-647
    render()                                  # :831-849
    render_high_accuracy(field_function)      # :778-802 (h = 0.001)
    render_outline_rays(field_function)       # :804-829 (the outline the
                                              #  shader's dead const meant)
"""
from __future__ import annotations

import numpy as np

from . import _abi, camera as cam
from .engine import Engine, FramePlanes, predefined_source


class MainView:
    def __init__(self, engine: Engine, vertices, faces, center, width: int, height: int,
                 discrete_gpu: bool = True, field_function: str | None = None, bvh: bool = True):
        self.engine = engine
        self.downscale_factor = 1 if discrete_gpu else 2  # main_view.rs:93
        self.field_function = field_function or predefined_source(
            _abi.FIELD_IDS["mirage_spherical_sigmoid"])
        self.helpers = None
        self.params = _abi.reference_params()
        self.settings = _abi.Settings()
        self.settings.field_weight = 1.0
        self.settings.mouse_pos[0], self.settings.mouse_pos[1] = 0.5, 0.6
        self.settings.overlay_mode = 0
        self.settings.central_difference_delta = 1
        self.settings.lyapunov_scaling = 50.0
        self.engine.upload_scene(vertices, faces, bvh=bvh)
        self.center = np.asarray(center, dtype=np.float32)
        self.field = self.engine.compile_field(self.field_function)
        self.needs_redraw = True
        self.resize_texture(width, height)

    # ---- textures (main_view.rs:552-647) ----
    def resize_texture(self, width: int, height: int):
        import torch
        w, h = width // self.downscale_factor, height // self.downscale_factor
        self.width, self.height = w, h
        self.ray_casting = FramePlanes.allocate(w, h)
        self.texture = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")
        self.exponents = torch.zeros((h, w), dtype=torch.float32, device="cuda")
        self.ray_samples = torch.zeros((800, 8), dtype=torch.float32, device="cuda")
        self.camera = cam.Arcball(self.center, 1.0, (w, h))
        self.camera.zoom(-1.0, 1.0)
        self.update_camera()

    def update_camera(self):
        self.camera_uniform = self.camera.uniform()
        self.needs_redraw = True

    def update_model(self, vertices, faces, center):
        self.engine.upload_scene(vertices, faces)
        self.center = np.asarray(center, dtype=np.float32)
        self.camera = cam.Arcball(self.center, 1.0, (self.width, self.height))
        self.camera.zoom(-1.0, 1.0)
        self.update_camera()

    def load_obj(self, path, model: int = 0):
        """A dropped .obj file (src/main.rs:139-156): tobj's models[model]
        with triangulation, normalize_vertices and get_center
        (src/application.rs:199-226), then update_model.  Returns the mesh."""
        from . import scene
        mesh = scene.load_obj(path, model=model, normalize=True)
        self.update_model(mesh.xyz, mesh.faces, mesh.center)
        return mesh

    def update_settings(self, settings: _abi.Settings):
        self.settings = settings
        self.needs_redraw = True

    # ---- shader reload (main_view.rs:649-690) ----
    def reload_shader(self, new_src: str | None, field_function: str):
        """Compiles the field; raises LinonCompileError (the reference's
        Err(wgpu::Error)) and keeps the previous field on failure.  `new_src`
        plays the role of the edited main_view.wgsl: its `fn` declarations
        become helpers callable from the field."""
        helpers = new_src if new_src is not None else self.helpers
        field = self.engine.compile_field(field_function, helpers)
        if new_src is not None:
            self.helpers = new_src
        self.field_function = field_function
        self.field = field
        self.needs_redraw = True

    # ---- dispatch (main_view.rs:831-849) ----
    def render(self, params: _abi.MarchParams | None = None):
        p = params or self.params
        self.engine.render(self.field, self.camera_uniform, self.settings, p, self.ray_casting)
        self.engine.overlay(self.settings, self.width, self.height, self.ray_casting.color,
                            self.ray_casting.mapping, self.texture, self.exponents)
        self.engine.capture_reference(self.field, self.camera_uniform, self.settings, p, self.width,
                                      self.height, self.ray_samples)
        self.needs_redraw = False

    def render_high_accuracy(self, field_function: str):
        """Enhance: one frame with h_initial = 0.001 (main_view.rs:778-802)."""
        if field_function != self.field_function:
            self.reload_shader(None, field_function)
        p = _abi.reference_params()
        p.h_initial = 0.001
        self.render(p)

    def render_outline_rays(self, field_function: str, min_exp: float = 0.8):
        """Outline: capture rays at the extremal pixels whose Lyapunov
        exponent is >= min_exp (main_view.wgsl:381-468)."""
        if field_function != self.field_function:
            self.reload_shader(None, field_function)
        self.engine.render(self.field, self.camera_uniform, self.settings, self.params, self.ray_casting)
        s = _abi.Settings.from_buffer_copy(self.settings)
        s.overlay_mode = 1
        self.engine.overlay(s, self.width, self.height, self.ray_casting.color, self.ray_casting.mapping,
                            self.texture, self.exponents)
        _, pos = self.engine.outline_select(self.exponents, self.width, self.height, min_exp)
        self.engine.capture_reference(self.field, self.camera_uniform, self.settings, self.params, self.width,
                                      self.height, self.ray_samples, positions=pos)
        return pos
