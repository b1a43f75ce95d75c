"""Scenes loaded from OBJ files, rendered through the C ABI (GPU).

The obj_scene workload (raw Cornell box triangles, a quad torus, a hexagon
and a pentagon; normalised and centred as the reference's dropped-file path
does) goes through linon_obj_parse -> linon_scene_upload (BVH) ->
linon_render.  Bars: precise modules bit-exact to the FP32 oracle on the
transcendental-free fields (colour within 1/255, the specular pow), BVH ==
brute force bit-exact, and the MainView mirror's load_obj path renders.
"""
import numpy as np
import pytest
import torch

from linon_gb300 import FramePlanes, _abi, workloads as wl
from linon_gb300.engine import predefined_source

pytestmark = pytest.mark.gpu


def render(engine, w, fld):
    f = FramePlanes.allocate(w.width, w.height)
    engine.render(fld, w.camera, w.settings, w.params, f)
    torch.cuda.synchronize()
    engine.synchronize()
    return {k: getattr(f, k).cpu().numpy() for k in ("color", "mapping", "hit_id", "steps")}


@pytest.mark.parametrize("model", [0, 1])
@pytest.mark.parametrize("name", ["linear", "mirage_spherical", "identity"])
def test_obj_scene_precise_bit_exact(engine, oracle, model, name):
    w = wl.obj_scene(128, 96, model=model)
    engine.upload_scene(w.xyz, w.faces, None, bvh=True)
    fld = engine.compile_field(predefined_source(_abi.FIELD_IDS[name]), precise=True)
    g = render(engine, w, fld)
    o = oracle.render(w.xyz, w.faces, None, w.camera, w.settings, w.params, _abi.FIELD_IDS[name], w.width,
                      w.height, want=("color", "mapping", "hit_id", "steps"))
    np.testing.assert_array_equal(g["hit_id"], o["hit_id"])
    np.testing.assert_array_equal(g["steps"], o["steps"])
    np.testing.assert_array_equal(g["mapping"].view(np.uint32), o["mapping"].view(np.uint32))
    assert np.abs(g["color"].astype(int) - o["color"].astype(int)).max() <= 1
    assert (g["hit_id"] >= 0).mean() > 0.1  # the frame sees geometry


def test_obj_scene_bvh_equals_brute_force(engine):
    w = wl.obj_scene(200, 150, model=1)
    w.params = wl.fixed_steps(0.01, 400)
    fld = engine.compile_field(wl.TWIST)
    engine.upload_scene(w.xyz, w.faces, None, bvh=False)
    a = render(engine, w, fld)
    engine.upload_scene(w.xyz, w.faces, None, bvh=True)
    assert engine.scene_info()["nodes"] > 1
    b = render(engine, w, fld)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])


def test_main_view_load_obj(engine, tmp_path):
    from linon_gb300 import scene
    from linon_gb300.main_view import MainView
    p = tmp_path / "scene.obj"
    p.write_text(wl.obj_scene_text())
    xyz, faces, _, center = scene.cornell_reference()
    mv = MainView(engine, xyz, faces, center, 64, 48)
    mesh = mv.load_obj(p)
    assert mesh.n_models == 3 and mesh.faces.shape == (36, 3)
    np.testing.assert_array_equal(mv.center, mesh.center)
    mv.render()
    torch.cuda.synchronize()
    assert engine.scene_info()["faces"] == 36
