"""linon_capture_paths_noalloc: ray-path capture that allocates nothing.

Callers that cannot allocate device memory (an interactive click handler with
a frame budget, a host with a fixed memory budget) use this variant; it stages
the ray start positions in a fixed array inside the library instead of the
context's scratch buffer.  Checked here through the C ABI against
linon_capture_paths on two calls in a row (the second with fewer rays, so
stale positions from the first call are present in the shared array), plus
the size limit and the image-size checks both entry points share.  This file
sorts last so that a run stopping at the first failure has already run every
other test.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from linon_gb300 import _abi, workloads as wl
from linon_gb300.engine import predefined_source

pytestmark = pytest.mark.gpu


def _call(lib, engine, fld, w, pos, h, n_steps, every, out):
    pos = np.ascontiguousarray(pos, np.float32)
    return lib.linon_capture_paths_noalloc(engine.ctx, fld.handle, C.byref(w.camera), C.byref(w.settings),
                                           C.byref(w.params), w.width, w.height, pos.ctypes.data, len(pos),
                                           float(h), int(n_steps), int(every), out.data_ptr())


def test_noalloc_capture_matches_capture_paths(engine):
    lib = _abi.load()
    w = wl.plain_small(256, 256)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fld = engine.compile_field(predefined_source(_abi.FIELD_IDS["lorenz_scaled"]))
    rng = np.random.default_rng(21)
    for n_rays, n_steps, every, h in ((300, 257, 5, 0.01), (37, 400, 1, 0.005)):
        pos = rng.uniform(0.1, 0.9, size=(n_rays, 2)).astype(np.float32)
        n_pts = -(-n_steps // every) + 1
        ref = torch.zeros((n_rays, n_pts, 4), dtype=torch.float32, device="cuda")
        engine.capture_paths(fld, w.camera, w.settings, w.params, w.width, w.height, pos, h, n_steps, every, ref)
        engine.synchronize()
        before = engine.device_bytes()
        got = torch.full((n_rays, n_pts, 4), float("nan"), dtype=torch.float32, device="cuda")
        assert _call(lib, engine, fld, w, pos, h, n_steps, every, got) == _abi.LINON_OK
        engine.synchronize()
        torch.cuda.synchronize()
        assert engine.device_bytes() == before  # the context grew no buffer
        np.testing.assert_array_equal(got.cpu().numpy(), ref.cpu().numpy())


def test_noalloc_rejects_more_rays_than_the_array_holds(engine):
    lib = _abi.load()
    w = wl.plain_small(64, 64)
    fld = engine.compile_field(predefined_source(_abi.FIELD_IDS["linear"]))
    n = 16384 + 1
    pos = np.full((n, 2), 0.5, np.float32)
    out = torch.zeros((1, 4), dtype=torch.float32, device="cuda")  # never written
    st = _call(lib, engine, fld, w, pos, 0.01, 10, 1, out)
    assert st == _abi.LINON_EINVAL
    assert b"16384" in lib.linon_last_error()


def test_noalloc_checks_image_size_like_capture_paths(engine):
    # 65535 x 65535 is within the per-side limit but above 2^31-1 pixels:
    # both entry points reject it before any work is queued
    lib = _abi.load()
    w = wl.plain_small(64, 64)
    fld = engine.compile_field(predefined_source(_abi.FIELD_IDS["linear"]))
    w.width = w.height = 65535
    pos = np.full((4, 2), 0.5, np.float32)
    out = torch.zeros((1, 4), dtype=torch.float32, device="cuda")  # never written
    assert _call(lib, engine, fld, w, pos, 0.01, 10, 1, out) == _abi.LINON_EINVAL
    msg = lib.linon_last_error()
    st = lib.linon_capture_paths(engine.ctx, fld.handle, C.byref(w.camera), C.byref(w.settings), C.byref(w.params),
                                 w.width, w.height, pos.ctypes.data, len(pos), 0.01, 10, 1, out.data_ptr())
    assert st == _abi.LINON_EINVAL
    assert lib.linon_last_error() == msg
