"""ctypes wrapper of the oracle library (oracle/_build/liblinon_oracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the oracle the CUDA engine is compared
against; never as the thing measured or shipped.  The oracle is the C++ restatement of the shader
path in oracle/linon_oracle.hpp, pinned bit for bit against the reference's
shader source lowered on the host (tests/golden/make_shader_pins.py writes the
fixtures, tests/test_shader_pins.py checks them); the reference's runtime,
WGSL through a graphics API, is not available where this runs.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liblinon_oracle.so"
_lib = None


def build() -> Path:
    r = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
        vp = C.c_void_p
        _lib.oracle_render.argtypes = [C.c_int, vp, C.c_int, vp, C.c_int, vp, vp, vp, vp, C.c_int, C.c_int,
                                       C.c_int, vp, C.c_int64, vp, vp, vp, vp, vp, C.c_int, C.c_int]
        _lib.oracle_count_ops.argtypes = [vp, C.c_int, vp, C.c_int, vp, vp, vp, C.c_int, C.c_int, C.c_int,
                                          vp, C.c_int, vp, vp]
        _lib.oracle_count_field.argtypes = [C.c_int, vp, vp]
        _lib.oracle_count_live_ops.argtypes = [vp, C.c_int, vp, C.c_int, vp, vp, vp, C.c_int, C.c_int, C.c_int,
                                               vp, C.c_int, C.c_int, C.c_int, vp]
        _lib.oracle_field_eval.argtypes = [C.c_int, C.c_int, vp, C.c_int64, vp, vp]
        _lib.oracle_hit_triangle.argtypes = [vp, vp]
        _lib.oracle_hit_triangle.restype = C.c_float
        _lib.oracle_primary_dirs.argtypes = [vp, vp, C.c_int, C.c_int, vp, C.c_int, vp]
        _lib.oracle_primary_dirs64.argtypes = [vp, vp, C.c_int, C.c_int, vp, C.c_int, vp]
        _lib.oracle_overlay.argtypes = [C.c_int, vp, vp, C.c_int, C.c_int, vp, C.c_int, vp, vp, C.c_int]
        _lib.oracle_ftle.argtypes = [vp, vp, C.c_int, C.c_int, vp, C.c_double, vp]
        _lib.oracle_capture.argtypes = [C.c_int, C.c_int, vp, vp, vp, C.c_int, C.c_int, vp, C.c_int, C.c_float,
                                        C.c_int, C.c_int, C.c_int, vp]
        _lib.oracle_outline_select.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_float, vp, vp]
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def render(xyz, faces, face_rgb, camera, settings, params, field_id, width, height, pixels=None,
           precision=32, threads=0, want=("color", "mapping", "hit_id", "steps"), accel=False):
    """Renders the frame (or the listed pixel indices row*W+x) on the CPU.
    accel: test each segment against the faces listed by the oracle's
    candidate grid instead of every face (equal results; for large scenes)."""
    xyz = np.ascontiguousarray(xyz, np.float32)
    faces = np.ascontiguousarray(faces, np.uint32)
    rgb = None if face_rgb is None else np.ascontiguousarray(face_rgb, np.float32)
    n = width * height if pixels is None else len(pixels)
    pix = None if pixels is None else np.ascontiguousarray(pixels, np.int32)
    out = {}
    if "color" in want:
        out["color"] = np.zeros((n, 4), np.uint8)
    if "mapping" in want:
        out["mapping"] = np.zeros((n, 4), np.float32)
    if "mapping64" in want:
        out["mapping64"] = np.zeros((n, 4), np.float64)
    if "hit_id" in want:
        out["hit_id"] = np.zeros(n, np.int32)
    if "steps" in want:
        out["steps"] = np.zeros(n, np.int32)
    st = lib().oracle_render(precision, _p(xyz), len(xyz), _p(faces), len(faces), _p(rgb), C.addressof(camera),
                             C.addressof(settings), C.addressof(params), field_id, width, height, _p(pix),
                             0 if pix is None else len(pix), _p(out.get("color")), _p(out.get("mapping")),
                             _p(out.get("mapping64")), _p(out.get("hit_id")), _p(out.get("steps")), threads,
                             1 if accel else 0)
    assert st == 0
    if pixels is None:
        for k, v in list(out.items()):
            out[k] = v.reshape((height, width) + v.shape[1:])
    return out


def count_ops(xyz, faces, camera, settings, params, field_id, width, height, pixels):
    xyz = np.ascontiguousarray(xyz, np.float32)
    faces = np.ascontiguousarray(faces, np.uint32)
    pix = np.ascontiguousarray(pixels, np.int32)
    out = np.zeros((len(pix), 6), np.int64)
    steps = np.zeros(len(pix), np.int32)
    lib().oracle_count_ops(_p(xyz), len(xyz), _p(faces), len(faces), C.addressof(camera), C.addressof(settings),
                           C.addressof(params), field_id, width, height, _p(pix), len(pix), _p(out), _p(steps))
    return out, steps


def count_live_ops(xyz, faces, camera, settings, params, field_id, width, height, pixels, steps_a=64,
                   steps_b=128):
    """Algorithmic FP32 operations per accepted step at each listed pixel:
    the operations the endpoint depends on, without loop-invariant work or
    products by launch constants (oracle_count_live_ops).  Returns a float
    array [n, 7]: add, mul, div, sqrt, transcendental, free, cmp."""
    xyz = np.ascontiguousarray(xyz, np.float32)
    faces = np.ascontiguousarray(faces, np.uint32)
    pix = np.ascontiguousarray(pixels, np.int32)
    out = np.zeros((len(pix), 8), np.float64)
    st = lib().oracle_count_live_ops(_p(xyz), len(xyz), _p(faces), len(faces), C.addressof(camera),
                                     C.addressof(settings), C.addressof(params), field_id, width, height, _p(pix),
                                     len(pix), steps_a, steps_b, _p(out))
    assert st == 0, st
    return out[:, :7]


def count_field(field_id, inputs13):
    x = np.ascontiguousarray(inputs13, np.float32)
    out = np.zeros(6, np.int64)
    lib().oracle_count_field(field_id, _p(x), _p(out))
    return out


def field_eval(field_id, inputs, precision=32):
    x = np.ascontiguousarray(inputs, np.float32).reshape(-1, 13)
    if precision == 64:
        out = np.zeros((len(x), 3), np.float64)
        lib().oracle_field_eval(64, field_id, _p(x), len(x), None, _p(out))
    else:
        out = np.zeros((len(x), 3), np.float32)
        lib().oracle_field_eval(32, field_id, _p(x), len(x), _p(out), None)
    return out


def hit_triangle(tri9, ray6) -> float:
    a = np.ascontiguousarray(tri9, np.float32)
    b = np.ascontiguousarray(ray6, np.float32)
    return float(lib().oracle_hit_triangle(_p(a), _p(b)))


def primary_dirs(camera, params, width, height, pixels, precision=32):
    pix = np.ascontiguousarray(pixels, np.int32)
    if precision == 64:
        out = np.zeros((len(pix), 3), np.float64)
        lib().oracle_primary_dirs64(C.addressof(camera), C.addressof(params), width, height, _p(pix), len(pix),
                                    _p(out))
        return out
    out = np.zeros((len(pix), 3), np.float32)
    lib().oracle_primary_dirs(C.addressof(camera), C.addressof(params), width, height, _p(pix), len(pix), _p(out))
    return out


def overlay(rgba8, mapping, width, height, settings, srgb=False, precision=32, exponents=None):
    rgba8 = np.ascontiguousarray(rgba8, np.uint8)
    mapping = np.ascontiguousarray(mapping, np.float32)
    out = np.zeros((height, width, 4), np.uint8)
    e = np.zeros((height, width), np.float32) if exponents is None else exponents
    lib().oracle_overlay(precision, _p(rgba8), _p(mapping), width, height, C.addressof(settings), 1 if srgb else 0,
                         _p(out), _p(e), 0)
    return out, e


def ftle(camera, params, width, height, mapping, T):
    mapping = np.ascontiguousarray(mapping, np.float32)
    out = np.zeros((height, width), np.float32)
    lib().oracle_ftle(C.addressof(camera), C.addressof(params), width, height, _p(mapping), float(T), _p(out))
    return out


def capture(field_id, camera, settings, params, width, height, pos_xy, h, n_steps, every, record_final,
            precision=32):
    pos = np.ascontiguousarray(pos_xy, np.float32).reshape(-1, 2)
    npts = -(-n_steps // every) + (1 if record_final else 0)
    out = np.zeros((len(pos), npts, 4), np.float32)
    lib().oracle_capture(precision, field_id, C.addressof(camera), C.addressof(settings), C.addressof(params),
                         width, height, _p(pos), len(pos), float(h), n_steps, every, 1 if record_final else 0,
                         _p(out))
    return out


def outline_select(exponents, width, height, min_exp, stride=None):
    e = np.ascontiguousarray(exponents, np.float32)
    px = np.zeros(8, np.int32)
    py = np.zeros(8, np.int32)
    lib().oracle_outline_select(_p(e), width, height, width if stride is None else stride, float(min_exp),
                                _p(px), _p(py))
    return np.stack([px, py], axis=1)


def max_threads() -> int:
    return int(lib().oracle_max_threads())
