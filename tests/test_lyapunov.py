"""The Lyapunov pipeline (overlay, finite-time exponent, p95 threshold,
outline pixels, outline capture) against the oracle (GPU)."""
import numpy as np
import pytest
import torch

from linon_gb300 import _abi, lyapunov, workloads as wl
from linon_gb300.engine import predefined_source

pytestmark = pytest.mark.gpu


def test_pipeline_matches_oracle(engine, oracle):
    w = wl.lyapunov_1024(128, 128)
    w.params = wl.fixed_steps(0.01, 300, kahan=True)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fld = engine.compile_field(predefined_source(_abi.FIELD_IDS["lorenz_scaled"]), precise=True)
    r = lyapunov.run(engine, fld, w, horizon=3.0, quantile=0.95, timings=True)
    mapping = r["planes"].mapping.cpu().numpy()
    # the render is the precise module: bit-exact endpoints
    o = oracle.render(w.xyz, w.faces, w.face_rgb, w.camera, w.settings, w.params, _abi.FIELD_IDS["lorenz_scaled"],
                      128, 128)
    np.testing.assert_array_equal(mapping.view(np.uint32), o["mapping"].view(np.uint32))
    # finite-time exponent (FP64) and its 95th percentile over the interior
    ftle = r["ftle"].cpu().numpy()
    np.testing.assert_allclose(ftle, oracle.ftle(w.camera, w.params, 128, 128, mapping, 3.0), rtol=1e-6, atol=1e-6)
    inner = np.sort(ftle[1:-1, 1:-1].ravel())
    assert r["threshold"] == inner[int(np.floor(0.95 * (len(inner) - 1)))]
    # outline pixels: the shader's 8 scans over the thresholded map
    np.testing.assert_array_equal(r["outline_pixels"], oracle.outline_select(ftle, 128, 128, r["threshold"]))
    # outline capture: 8 rays x 100 samples at those positions
    got = r["samples"].cpu().numpy().reshape(8, 100, 8)
    ref = oracle.capture(_abi.FIELD_IDS["lorenz_scaled"], w.camera, w.settings, w.params, 128, 128,
                         r["outline_positions"], 0.001, 5000, 50, False)
    np.testing.assert_array_equal(got[:, :, :4], ref)
    assert r["indices"].shape == (1584, 3)
    assert set(r["ms"]) == {"render", "overlay_fp64", "ftle_fp64", "quantile", "outline_select", "outline_capture"}
