"""ctypes view of include/linon.h (the C ABI of liblinon.so).

Structures are byte-compatible with the reference's uniforms
(CameraUniform 112 B, Settings 24 B, RaySample 32 B; src/main_view.rs:12-51).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "liblinon.so"

LINON_OK = 0
LINON_EINVAL = 1
LINON_ECOMPILE = 2
LINON_ECUDA = 3
LINON_ENOMEM = 4
LINON_ETIMEOUT = 5
LINON_ENOSCENE = 6
LINON_EBUSY = 7
LINON_ESTATE = 8
LINON_EIO = 9
LINON_OBJ_NORMALIZE = 1
LINON_COMPILE_PRECISE = 1
LINON_VALIDATE_BATCHED = 2
LINON_MAX_BATCH_FIELDS = 8

FIELD_IDS = {
    "custom": 0, "mirage_spherical": 1, "mirage_plane": 2, "mirage_spherical_sigmoid": 3,
    "mirage_plane_sigmoid": 4, "translation_x": 5, "translation_z": 6, "rotation": 7,
    "lorenz": 8, "roessler": 9, "identity": 10, "linear": 11, "twist": 12, "lens": 13,
    "lorenz_scaled": 14,
}
FIELD_COUNT = 15


class Camera(C.Structure):
    _fields_ = [("origin", C.c_float * 4), ("view_direction", C.c_float * 4),
                ("up", C.c_float * 4), ("view_matrix", C.c_float * 16)]


class Settings(C.Structure):
    _fields_ = [("field_weight", C.c_float), ("mouse_pos", C.c_float * 2),
                ("overlay_mode", C.c_int32), ("central_difference_delta", C.c_int32),
                ("lyapunov_scaling", C.c_float)]


class RaySample(C.Structure):
    _fields_ = [("position", C.c_float * 4), ("color", C.c_float * 4)]


class MarchParams(C.Structure):
    _fields_ = [("h_initial", C.c_float), ("t_max", C.c_float), ("max_steps", C.c_int32),
                ("adaptive", C.c_int32), ("h_fine", C.c_float), ("h_fine_above", C.c_float),
                ("stop_on_hit", C.c_int32), ("kahan", C.c_int32), ("focal_length", C.c_float),
                ("viewport_height", C.c_float), ("linear_mode", C.c_int32), ("reserved", C.c_int32)]


class Frame(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("color", C.c_void_p),
                ("mapping", C.c_void_p), ("hit_id", C.c_void_p), ("steps", C.c_void_p)]


class View(C.Structure):
    _fields_ = [("camera", Camera), ("settings", Settings), ("params", MarchParams),
                ("width", C.c_int32), ("height", C.c_int32), ("field_index", C.c_int32),
                ("reserved", C.c_int32), ("out", Frame)]


class BatchTuning(C.Structure):
    _fields_ = [("quantum", C.c_int32), ("block_threads", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("tile_w", C.c_int32), ("tile_h", C.c_int32), ("refill_below", C.c_int32),
                ("schedule", C.c_int32)]


LINON_REQ_FRAME, LINON_REQ_OVERLAY, LINON_REQ_CAPTURE = 0, 1, 2


class Request(C.Structure):
    _fields_ = [("kind", C.c_int32), ("field_index", C.c_int32), ("camera", Camera), ("settings", Settings),
                ("params", MarchParams), ("width", C.c_int32), ("height", C.c_int32),
                ("fp64_overlay", C.c_int32), ("n_rays", C.c_int32), ("n_steps", C.c_int32),
                ("record_every", C.c_int32), ("h", C.c_float), ("reserved", C.c_int32),
                ("pos_xy", C.c_void_p)]


class ServeConfig(C.Structure):
    _fields_ = [("hbm_budget", C.c_size_t), ("slots", C.c_int32), ("max_wave", C.c_int32),
                ("tuning", BatchTuning)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int32), ("kind", C.c_int32), ("t_submit_ms", C.c_double),
                ("t_admit_ms", C.c_double), ("t_done_ms", C.c_double), ("ray_steps", C.c_int64),
                ("frame", Frame), ("overlay", C.c_void_p), ("exponents", C.c_void_p), ("paths", C.c_void_p),
                ("n_points", C.c_int32), ("wave", C.c_int32)]


class ServeStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("waves", C.c_uint64), ("bytes_in_use", C.c_size_t), ("bytes_peak", C.c_size_t)]


assert C.sizeof(Camera) == 112 and C.sizeof(Settings) == 24 and C.sizeof(RaySample) == 32
assert C.sizeof(MarchParams) == 48

vp, i32, sz, cp = C.c_void_p, C.c_int32, C.c_size_t, C.c_char_p
P = C.POINTER

# name -> (restype, argtypes); every symbol declared in include/linon.h
PROTOTYPES = {
    "linon_abi_version": (C.c_int, []),
    "linon_last_error": (cp, []),
    "linon_status_string": (cp, [C.c_int]),
    "linon_predefined_source": (cp, [C.c_int]),
    "linon_predefined_name": (cp, [C.c_int]),
    "linon_march_params_reference": (None, [P(MarchParams)]),
    "linon_create": (C.c_int, [C.c_int, sz, P(vp)]),
    "linon_destroy": (C.c_int, [vp]),
    "linon_set_stream": (C.c_int, [vp, vp]),
    "linon_synchronize": (C.c_int, [vp]),
    "linon_device_bytes": (sz, [vp]),
    "linon_scene_upload": (C.c_int, [vp, vp, C.c_uint32, vp, C.c_uint32, vp, C.c_int]),
    "linon_scene_info": (C.c_int, [vp, P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)]),
    "linon_obj_load": (C.c_int, [C.c_char_p, C.c_uint32, C.c_uint32, P(vp)]),
    "linon_obj_parse": (C.c_int, [C.c_char_p, sz, C.c_char_p, C.c_uint32, C.c_uint32, P(vp)]),
    "linon_mesh_info": (C.c_int, [vp, P(C.c_uint32), P(C.c_uint32), P(C.c_uint32), P(C.c_float)]),
    "linon_mesh_positions": (P(C.c_float), [vp]),
    "linon_mesh_faces": (P(C.c_uint32), [vp]),
    "linon_mesh_free": (None, [vp]),
    "linon_normalize_vertices": (C.c_int, [vp, sz, P(C.c_float)]),
    "linon_field_compile": (C.c_int, [vp, cp, cp, C.c_int, P(vp), C.c_char_p, sz]),
    "linon_field_release": (C.c_int, [vp, vp]),
    "linon_field_flops": (C.c_int, [vp, P(i32), P(i32)]),
    "linon_field_pair_state": (C.c_int, [vp]),
    "linon_field_cuda_source": (cp, [vp]),
    "linon_field_validate": (C.c_int, [cp, cp, C.c_int, C.c_char_p, sz]),
    "linon_wgsl_translate": (C.c_int, [cp, cp, C.c_char_p, sz, C.c_char_p, sz]),
    "linon_render": (C.c_int, [vp, vp, P(Camera), P(Settings), P(MarchParams), P(Frame)]),
    "linon_render_rows": (C.c_int, [vp, vp, P(Camera), P(Settings), P(MarchParams), P(Frame), i32, i32]),
    "linon_field_eval": (C.c_int, [vp, vp, vp, vp, C.c_int64]),
    "linon_render_host": (C.c_int, [vp, vp, P(Camera), P(Settings), P(MarchParams), i32, i32,
                                    vp, vp, vp, vp]),
    "linon_overlay": (C.c_int, [vp, P(Settings), i32, i32, vp, vp, vp, vp, C.c_int, C.c_int]),
    "linon_ftle": (C.c_int, [vp, P(Camera), P(MarchParams), i32, i32, vp, C.c_float, vp]),
    "linon_capture_reference": (C.c_int, [vp, vp, P(Camera), P(Settings), P(MarchParams), i32,
                                          i32, vp, vp]),
    "linon_capture_paths": (C.c_int, [vp, vp, P(Camera), P(Settings), P(MarchParams), i32, i32,
                                      vp, i32, C.c_float, i32, i32, vp]),
    "linon_capture_paths_noalloc": (C.c_int, [vp, vp, P(Camera), P(Settings), P(MarchParams), i32, i32,
                                              vp, i32, C.c_float, i32, i32, vp]),
    "linon_outline_select": (C.c_int, [vp, vp, i32, i32, C.c_float, vp, vp]),
    "linon_exponent_quantile": (C.c_int, [vp, vp, i32, i32, i32, C.c_double, P(C.c_float)]),
    "linon_outline_indices": (C.c_int, [vp, sz]),
    "linon_render_batch": (C.c_int, [vp, vp, i32, vp, i32, vp]),
    "linon_render_views_plain": (C.c_int, [vp, vp, i32, vp, i32]),
    "linon_autotune_batch": (C.c_int, [vp, vp, i32, vp, i32, P(BatchTuning), P(C.c_double)]),
    "linon_probe_fp32_peak": (C.c_int, [vp, P(C.c_double)]),
    "linon_check_bounded_wait": (C.c_int, [vp, i32]),
    "linon_serve_start": (C.c_int, [vp, vp, i32, P(ServeConfig), P(vp)]),
    "linon_serve_submit": (C.c_int, [vp, P(Request), P(C.c_uint64)]),
    "linon_serve_poll": (C.c_int, [vp, C.c_uint64, P(Result)]),
    "linon_serve_wait": (C.c_int, [vp, C.c_uint64, C.c_double, P(Result)]),
    "linon_serve_copy": (C.c_int, [vp, C.c_uint64, i32, vp, sz]),
    "linon_serve_release": (C.c_int, [vp, C.c_uint64]),
    "linon_serve_stats": (C.c_int, [vp, P(ServeStats)]),
    "linon_serve_stop": (C.c_int, [vp]),
}

_lib = None
ABI_VERSION = 2  # include/linon.h LINON_ABI_VERSION (struct layouts of this file)


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads liblinon.so (building it first if it is missing) and binds the ABI."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        from . import build as _build
        _build.build()
    lib = C.CDLL(str(p))
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.linon_abi_version() != ABI_VERSION:
        raise RuntimeError(f"{p}: ABI version {lib.linon_abi_version()}, these bindings expect {ABI_VERSION} "
                           "(rebuild with python -m linon_gb300.build)")
    if path is None:
        _lib = lib
    return lib


class LinonError(RuntimeError):
    """A non-zero status from the C ABI, with linon_last_error()'s message."""

    def __init__(self, status: int, message: str):
        super().__init__(f"linon status {status}: {message}")
        self.status = status
        self.message = message


class LinonCompileError(LinonError):
    """Field source rejected (the reference's reload_shader Err, main_view.rs:676-678)."""


def check(status: int) -> None:
    if status != LINON_OK:
        msg = load().linon_last_error().decode(errors="replace")
        if status == LINON_ECOMPILE:
            raise LinonCompileError(status, msg)
        raise LinonError(status, msg)


def reference_params() -> MarchParams:
    p = MarchParams()
    load().linon_march_params_reference(C.byref(p))
    return p


def shader_params() -> MarchParams:
    """The shader's own march constants, filled in Python without loading
    liblinon.so: h = 0.1 (main_view.wgsl:241), the t <= 5 loop (:244),
    adaptive refinement to h = 0.001 above h = 0.002 (:252-253), focal
    length 0.035 and viewport height 0.025 (:355-356).  Equal field for
    field to linon_march_params_reference (a CPU test holds them equal);
    the workload builders use it so that the CPU reference leg never maps
    the engine library."""
    p = MarchParams()
    p.h_initial, p.t_max, p.max_steps, p.adaptive = 0.1, 5.0, 0, 1
    p.h_fine, p.h_fine_above = 0.001, 0.002
    p.stop_on_hit, p.kahan, p.linear_mode, p.reserved = 0, 0, 0, 0
    p.focal_length, p.viewport_height = 0.035, 0.025
    return p
