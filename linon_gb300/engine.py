"""Python host API over the C ABI.

`Engine` wraps a linon_ctx (one CUDA device, one stream, the resident scene,
compiled fields); `Field` is a compiled field function.  Frame planes are
torch CUDA tensors (torch is used for device memory and streams only); every
compute call goes through liblinon.so, and a missing library or GPU raises
instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import check, load


@dataclass
class FramePlanes:
    """Device output planes of one frame (row 0 = top, as the storage texture)."""
    width: int
    height: int
    color: "object"    # torch.uint8 [H, W, 4]
    mapping: "object"  # torch.float32 [H, W, 4]
    hit_id: "object"   # torch.int32 [H, W]
    steps: "object"    # torch.int32 [H, W]

    @staticmethod
    def allocate(width: int, height: int, device="cuda"):
        import torch
        return FramePlanes(width, height,
                           torch.empty((height, width, 4), dtype=torch.uint8, device=device),
                           torch.empty((height, width, 4), dtype=torch.float32, device=device),
                           torch.empty((height, width), dtype=torch.int32, device=device),
                           torch.empty((height, width), dtype=torch.int32, device=device))

    def sample(self, pixels) -> dict:
        """The planes at pixel indices row*W+x, gathered on the device and
        copied to the host as numpy arrays."""
        import torch
        idx = torch.as_tensor(np.asarray(pixels, np.int64), device=self.mapping.device)
        out = {}
        for k in ("color", "mapping", "hit_id", "steps"):
            t = getattr(self, k)
            if t is not None:
                out[k] = t.reshape(self.width * self.height, -1)[idx].squeeze(-1).cpu().numpy()
        return out

    def abi(self) -> _abi.Frame:
        f = _abi.Frame()
        f.width, f.height = self.width, self.height
        f.color = self.color.data_ptr() if self.color is not None else None
        f.mapping = self.mapping.data_ptr() if self.mapping is not None else None
        f.hit_id = self.hit_id.data_ptr() if self.hit_id is not None else None
        f.steps = self.steps.data_ptr() if self.steps is not None else None
        return f


class Field:
    """A compiled field function (linon_field_compile)."""

    def __init__(self, engine: "Engine", handle: int, body: str, precise: bool):
        self.engine = engine
        self.handle = C.c_void_p(handle)
        self.body = body
        self.precise = precise

    def flops(self):
        a, t = C.c_int32(), C.c_int32()
        check(load().linon_field_flops(self.handle, C.byref(a), C.byref(t)))
        return a.value, t.value

    def pair_state(self) -> int:
        """linon_field_pair_state: 1 fixed-step renders run two rays per
        thread, 0 not tried yet, -1 one ray per thread."""
        return int(load().linon_field_pair_state(self.handle))

    def cuda_source(self) -> str:
        return load().linon_field_cuda_source(self.handle).decode()

    def release(self):
        if self.handle:
            load().linon_field_release(self.engine.ctx, self.handle)
            self.handle = C.c_void_p()


class Engine:
    """One linon context on one CUDA device."""

    def __init__(self, device: int = 0, hbm_budget: int = 0, stream=None):
        import torch
        self._torch = torch
        self.lib = load()
        self.device = device
        ctx = C.c_void_p()
        check(self.lib.linon_create(device, hbm_budget, C.byref(ctx)))
        self.ctx = ctx
        # The engine enqueues on a torch stream of its own; every call is
        # fenced against torch's current stream on entry and exit, so tensors
        # torch produced are ready and results are ordered for torch users.
        self.stream = None
        self.set_stream(stream if stream is not None else torch.cuda.Stream(device=device))

    def close(self):
        if self.ctx:
            self.lib.linon_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream):
        """stream: a torch.cuda.Stream (the engine's queue from now on)."""
        self.stream = stream
        # torch's default stream is the legacy default stream (handle 0); the
        # ABI reads NULL as "the context's own stream", so pass
        # cudaStreamLegacy (1) for it
        raw = stream.cuda_stream if stream.cuda_stream else 1
        check(self.lib.linon_set_stream(self.ctx, C.c_void_p(raw)))

    def _call(self, name, *args):
        cur = self._torch.cuda.current_stream(self.device)
        fenced = cur.cuda_stream != self.stream.cuda_stream
        if fenced:
            self.stream.wait_stream(cur)
        check(getattr(self.lib, name)(*args))
        if fenced:
            cur.wait_stream(self.stream)

    def synchronize(self):
        check(self.lib.linon_synchronize(self.ctx))

    def device_bytes(self) -> int:
        return int(self.lib.linon_device_bytes(self.ctx))

    # ---- scene (MainView::update_model) ----
    def upload_scene(self, xyz, faces, face_rgb=None, bvh: bool = True):
        xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
        faces = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1, 3)
        rgb = None if face_rgb is None else np.ascontiguousarray(face_rgb, dtype=np.float32).reshape(-1, 3)
        check(self.lib.linon_scene_upload(
            self.ctx, xyz.ctypes.data, len(xyz), faces.ctypes.data, len(faces),
            rgb.ctypes.data if rgb is not None else None, 1 if bvh else 0))

    def scene_info(self):
        f, n, d = C.c_uint32(), C.c_uint32(), C.c_uint32()
        check(self.lib.linon_scene_info(self.ctx, C.byref(f), C.byref(n), C.byref(d)))
        return {"faces": f.value, "nodes": n.value, "max_depth": d.value}

    # ---- fields (MainView::reload_shader) ----
    def compile_field(self, body: str, helpers: str | None = None, precise: bool = False) -> Field:
        log = C.create_string_buffer(1 << 16)
        h = C.c_void_p()
        st = self.lib.linon_field_compile(self.ctx, body.encode(), helpers.encode() if helpers else None,
                                          _abi.LINON_COMPILE_PRECISE if precise else 0, C.byref(h), log,
                                          len(log))
        if st != _abi.LINON_OK:
            msg = log.value.decode(errors="replace") or self.lib.linon_last_error().decode()
            if st == _abi.LINON_ECOMPILE:
                raise _abi.LinonCompileError(st, msg)
            raise _abi.LinonError(st, msg)
        return Field(self, h.value, body, precise)

    def predefined(self, name_or_id, precise: bool = False) -> Field:
        fid = name_or_id if isinstance(name_or_id, int) else _abi.FIELD_IDS[name_or_id]
        return self.compile_field(predefined_source(fid), precise=precise)

    # ---- the two dispatches of MainView::render ----
    def render(self, field: Field, camera, settings, params, frame: FramePlanes):
        f = frame.abi()
        self._call("linon_render", self.ctx, field.handle, C.byref(camera), C.byref(settings),
                                    C.byref(params), C.byref(f))

    def render_rows(self, field: Field, camera, settings, params, frame: FramePlanes, row0: int, row1: int):
        """Rows [row0, row1) of the frame (linon_render_rows)."""
        f = frame.abi()
        self._call("linon_render_rows", self.ctx, field.handle, C.byref(camera), C.byref(settings),
                   C.byref(params), C.byref(f), int(row0), int(row1))

    def field_eval(self, field: Field, inputs):
        """Evaluates the field at n points (torch CUDA tensor [n, 13]) -> [n, 3]."""
        import torch
        x = inputs.contiguous().to(torch.float32)
        out = torch.empty((x.shape[0], 3), dtype=torch.float32, device=x.device)
        self._call("linon_field_eval", self.ctx, field.handle, x.data_ptr(), out.data_ptr(), x.shape[0])
        return out

    def render_host(self, field: Field, camera, settings, params, width: int, height: int,
                    color=True, mapping=True, hit_id=True, steps=True):
        """Renders into host numpy arrays (copies inside the call)."""
        out = {}
        ptr = {}
        for name, on, shape, dt in (("color", color, (height, width, 4), np.uint8),
                                    ("mapping", mapping, (height, width, 4), np.float32),
                                    ("hit_id", hit_id, (height, width), np.int32),
                                    ("steps", steps, (height, width), np.int32)):
            if on is True:
                out[name] = np.empty(shape, dtype=dt)
            elif on is not None and on is not False:
                out[name] = on
            ptr[name] = out[name].ctypes.data if name in out else None
        self._call("linon_render_host", self.ctx, field.handle, C.byref(camera), C.byref(settings),
                                         C.byref(params), width, height, ptr["color"], ptr["mapping"],
                                         ptr["hit_id"], ptr["steps"])
        return out

    def overlay(self, settings, width, height, ray_casting, mapping, target, exponents=None,
                srgb=False, fp64=False):
        self._call("linon_overlay", self.ctx, C.byref(settings), width, height, ray_casting.data_ptr(),
                                     mapping.data_ptr() if mapping is not None else None,
                                     target.data_ptr(), exponents.data_ptr() if exponents is not None else None,
                                     1 if srgb else 0, 1 if fp64 else 0)

    def ftle(self, camera, params, width, height, mapping, horizon, exponents):
        self._call("linon_ftle", self.ctx, C.byref(camera), C.byref(params), width, height,
                                  mapping.data_ptr(), float(horizon), exponents.data_ptr())

    # ---- path capture (sample_rays) ----
    def capture_reference(self, field: Field, camera, settings, params, width, height, out,
                          positions=None):
        pos = None
        if positions is not None:
            pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(8, 2)
        self._call("linon_capture_reference", self.ctx, field.handle, C.byref(camera), C.byref(settings),
                                               C.byref(params), width, height,
                                               pos.ctypes.data if pos is not None else None,
                                               out.data_ptr())

    def capture_paths(self, field: Field, camera, settings, params, width, height, pos_xy, h, n_steps,
                      record_every, out):
        pos = np.ascontiguousarray(pos_xy, dtype=np.float32).reshape(-1, 2)
        self._call("linon_capture_paths", self.ctx, field.handle, C.byref(camera), C.byref(settings),
                                           C.byref(params), width, height, pos.ctypes.data, len(pos),
                                           float(h), int(n_steps), int(record_every), out.data_ptr())

    # ---- outline rays ----
    def outline_select(self, exponents, width, height, min_exp=0.8):
        pix = np.zeros((8, 2), dtype=np.int32)
        pos = np.zeros((8, 2), dtype=np.float32)
        self._call("linon_outline_select", self.ctx, exponents.data_ptr(), width, height, float(min_exp),
                                            pix.ctypes.data, pos.ctypes.data)
        return pix, pos

    def exponent_quantile(self, exponents, width, height, q, border=0):
        out = C.c_float()
        self._call("linon_exponent_quantile", self.ctx, exponents.data_ptr(), width, height, border,
                                               float(q), C.byref(out))
        return out.value

    # ---- batches ----
    def _batch_args(self, fields, views):
        fa = (C.c_void_p * len(fields))(*[f.handle.value for f in fields])
        va = (_abi.View * len(views))(*views)
        return fa, va

    def render_batch(self, fields, views, tuning: _abi.BatchTuning | None = None):
        fa, va = self._batch_args(fields, views)
        self._call("linon_render_batch", self.ctx, fa, len(fields), va, len(views),
                                          C.byref(tuning) if tuning is not None else None)

    def render_views_plain(self, fields, views):
        fa, va = self._batch_args(fields, views)
        self._call("linon_render_views_plain", self.ctx, fa, len(fields), va, len(views))

    def autotune_batch(self, fields, views):
        fa, va = self._batch_args(fields, views)
        t = _abi.BatchTuning()
        ms = C.c_double()
        self._call("linon_autotune_batch", self.ctx, fa, len(fields), va, len(views), C.byref(t),
                                            C.byref(ms))
        return t, ms.value

    def probe_fp32_peak(self) -> float:
        v = C.c_double()
        check(self.lib.linon_probe_fp32_peak(self.ctx, C.byref(v)))
        return v.value

    def check_bounded_wait(self, polls: int = 4096) -> int:
        """linon_check_bounded_wait: the raw status (LINON_ETIMEOUT when the
        device's bounded wait ran out and was reported)."""
        return int(self.lib.linon_check_bounded_wait(self.ctx, int(polls)))


def predefined_source(fid: int) -> str:
    s = load().linon_predefined_source(int(fid))
    if s is None:
        raise ValueError(f"no predefined field {fid}")
    return s.decode()


def predefined_name(fid: int) -> str:
    return load().linon_predefined_name(int(fid)).decode()


def validate_field(body: str, helpers: str | None = None, precise: bool = False, batched: bool = False) -> str:
    """Front end + NVRTC compile without a GPU; returns the compiler report.
    batched: also compile the batched kernels (linon_render_batch) with it."""
    log = C.create_string_buffer(1 << 18)
    flags = (_abi.LINON_COMPILE_PRECISE if precise else 0) | (_abi.LINON_VALIDATE_BATCHED if batched else 0)
    st = load().linon_field_validate(body.encode(), helpers.encode() if helpers else None, flags, log, len(log))
    if st != _abi.LINON_OK:
        raise _abi.LinonCompileError(st, log.value.decode(errors="replace"))
    return log.value.decode(errors="replace")


def translate_wgsl(body: str, helpers: str | None = None) -> str:
    """WGSL field body -> CUDA C (front end only, no GPU)."""
    out = C.create_string_buffer(1 << 20)
    log = C.create_string_buffer(1 << 16)
    st = load().linon_wgsl_translate(body.encode(), helpers.encode() if helpers else None, out, len(out),
                                     log, len(log))
    if st != _abi.LINON_OK:
        raise _abi.LinonCompileError(st, log.value.decode(errors="replace"))
    return out.value.decode()


def outline_indices() -> np.ndarray:
    """The outline mesh index list of src/ray_samples.rs:42-49 as [n,3] uint16."""
    n = load().linon_outline_indices(None, 0)
    buf = np.zeros(n, dtype=np.uint16)
    got = load().linon_outline_indices(buf.ctypes.data, n)
    if got < 0:
        check(-got)
    return buf.reshape(-1, 3)
