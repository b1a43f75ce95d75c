"""Writes tests/golden/shader_pins.npz: outputs of the reference's own
shaders (src/main_view.wgsl, src/overlay.wgsl, with the field bodies of
src/functions.rs), run on the host.

Neither wgpu nor a graphics stack exists here, so the shader text itself is
lowered: each resource binding is replaced by a module-scope var<private>
holding the data the application would bind (a texture store becomes an
assignment to a private variable, a texture load an indexed read, a
runtime-sized array a fixed-size one), the entry point becomes a function
of its invocation id, and the reference's own linon helpers keep their
bodies under a `ref_` prefix (the front end predeclares its own).  The
result goes through this package's WGSL front end, is compiled for the host
with g++ (no FMA contraction) and is run once per invocation with fresh
private state.  Every substitution is a literal string replacement that
must match; a changed reference fails loudly.

Run from the repository root, where the reference sources are present:
    python tests/golden/make_shader_pins.py <path of the linon source tree>
"""
from __future__ import annotations

import ctypes as C
import re
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from linon_gb300 import translate_wgsl  # noqa: E402
from linon_gb300 import scene  # noqa: E402

RT = ROOT / "linon_gb300" / "csrc" / "device" / "wgsl_rt.cuh"
REF_HELPERS = ["rotateX", "rotateY", "rotateZ", "translate", "refraction_index", "refraction",
               "point_plane_distance", "sigmoid", "PI"]
FIELD_LINE = ("fn field_function(p_prev: vec3<f32>, p: vec3<f32>, v0: vec3<f32>, v: vec3<f32>, t: f32)"
              " -> vec3<f32> { return v; }")


def sub1(text: str, old: str, new: str) -> str:
    """Literal replacement that must match exactly once."""
    n = text.count(old)
    if n != 1:
        raise SystemExit(f"expected one occurrence of {old!r}, found {n}")
    return text.replace(old, new)


def suball(text: str, old: str, new: str) -> str:
    if old not in text:
        raise SystemExit(f"expected {old!r}")
    return text.replace(old, new)


def rename_helpers(text: str) -> str:
    for name in REF_HELPERS:
        text = re.sub(rf"\b{name}\b", "ref_" + name, text)
    return text


def predefined_bodies(ref: Path) -> dict:
    """Field bodies of PredefinedFunction::to_code (src/functions.rs): the
    Rust string literals, unescaped."""
    src = (ref / "src" / "functions.rs").read_text()
    code = src[src.index("fn to_code"):]
    out = {}
    for m in re.finditer(r'Self::(\w+)\s*=>\s*"((?:[^"\\]|\\.)*)"', code):
        body = re.sub(r"\\\n\s*", "", m.group(2))  # line continuations
        body = body.replace('\\"', '"').replace("\\n", "\n").replace("\\\\", "\\")
        out[m.group(1)] = body
    return out


def rust_array(src: str, name: str, dtype) -> np.ndarray:
    """The literal `pub const NAME: [T; N] = [...];` of a Rust file."""
    m = re.search(rf"pub const {name}: \[\w+; (\d+)\] = \[(.*?)\];", src, re.S)
    if not m:
        raise SystemExit(f"no array {name}")
    items = [t for t in re.sub(r"//[^\n]*", "", m.group(2)).replace("\n", " ").split(",") if t.strip()]
    a = np.array([float(t) for t in items], dtype)
    if len(a) != int(m.group(1)):
        raise SystemExit(f"{name}: {len(a)} items, declared {m.group(1)}")
    return a


def scene_digest(ref: Path) -> str:
    """src/cornell_box.rs's VERTICES and INDICES must equal this package's
    raw Cornell box (scene.cornell_raw); returns the SHA-256 of their bytes,
    which the tests check against the package without the reference."""
    import hashlib
    src = (ref / "src" / "cornell_box.rs").read_text()
    v = rust_array(src, "VERTICES", np.float32).reshape(-1, 3)
    f = rust_array(src, "INDICES", np.float64).astype(np.uint32).reshape(-1, 3)
    xyz, faces, _ = scene.cornell_raw()
    if not (np.array_equal(v, xyz) and np.array_equal(f, faces)):
        raise SystemExit("scene.cornell_raw differs from src/cornell_box.rs")
    return hashlib.sha256(v.tobytes() + f.tobytes()).hexdigest()


def f32s(a) -> str:
    return ", ".join(repr(float(np.float32(x))) for x in np.asarray(a, np.float32).ravel())


# Sizes of the runtime-sized arrays once they are fixed-size private arrays.
MAX_VERTICES, MAX_FACES, MAX_TEXELS = 256, 256, 4096


def main_view_module(ref: Path, high_accuracy=False, outline=False, linear=False) -> str:
    """src/main_view.wgsl with its bindings made private (see the module
    docstring); the variants are the application's own source edits
    (src/main_view.rs:787 for high accuracy, :811 for outline rays) and the
    linear_mode constant."""
    s = (ref / "src" / "main_view.wgsl").read_text()
    s = sub1(s, FIELD_LINE, "")  # the field body is translated as the field function
    if high_accuracy:
        s = sub1(s, "let h_initial = 0.1;", "let h_initial = 0.001;")
    if outline:
        s = sub1(s, "const sample_outline_rays: bool = false;", "const sample_outline_rays: bool = true;")
    if linear:
        s = sub1(s, "const linear_mode: bool = false;", "const linear_mode: bool = true;")
    s = sub1(s, "@group(0) @binding(0)\nvar ttarget: texture_storage_2d<rgba8unorm, write>;",
             "var<private> pin_color: vec4<f32>;\nvar<private> pin_size: vec2<u32>;\n"
             "var<private> pin_n_faces: u32;")
    s = sub1(s, "@group(0) @binding(1)\nvar mapping: texture_storage_2d<rgba32float, write>;",
             "var<private> pin_mapping: vec4<f32>;")
    s = sub1(s, "@group(0) @binding(2)\nvar<uniform> camera: Camera;", "var<private> camera: Camera;")
    s = sub1(s, "@group(0) @binding(3)\nvar<uniform> settings: Settings;", "var<private> settings: Settings;")
    s = sub1(s, "    data: array<f32>,", f"    data: array<f32, {MAX_TEXELS}>,")
    s = sub1(s, "@group(0) @binding(4)\nvar<storage, read> exponents: Exponents;",
             "var<private> exponents: Exponents;")
    s = sub1(s, "    data: array<Vertex>,", f"    data: array<Vertex, {MAX_VERTICES}>,")
    s = sub1(s, "@group(1) @binding(0)\nvar<storage, read> vertices: Vertices;", "var<private> vertices: Vertices;")
    s = sub1(s, "    data: array<Face>,", f"    data: array<Face, {MAX_FACES}>,")
    s = sub1(s, "@group(1) @binding(1)\nvar<storage, read> faces: Faces;", "var<private> faces: Faces;")
    s = sub1(s, "@group(2) @binding(0)\nvar<storage, read_write> ray_samples: RaySamples;",
             "var<private> ray_samples: RaySamples;")
    s = sub1(s, "arrayLength(&faces.data)", "pin_n_faces")
    s = sub1(s, "textureDimensions(ttarget)", "pin_size")
    s = sub1(s, "textureStore(ttarget, coords, color);", "pin_color = color;")
    s = sub1(s, "textureStore(ttarget, coords, result.color);", "pin_color = result.color;")
    s = sub1(s, "textureStore(mapping, coords, result.mapping_point);", "pin_mapping = result.mapping_point;")
    s = sub1(s, "@compute @workgroup_size(8, 8)\nfn main_view(@builtin(global_invocation_id) gid: vec3<u32>)",
             "fn main_view(gid: vec3<u32>)")
    return rename_helpers(s)


def overlay_module(ref: Path) -> str:
    """src/overlay.wgsl with its bindings made private; both entry points
    become functions of the invocation id."""
    s = (ref / "src" / "overlay.wgsl").read_text()
    s = sub1(s, "@group(0) @binding(0)\nvar ray_casting: texture_2d<f32>;",
             f"struct PinTexels {{ data: array<vec4<f32>, {MAX_TEXELS}>, }};\n"
             "var<private> pin_ray_casting: PinTexels;\nvar<private> pin_size: vec2<u32>;\n"
             "fn pin_load_color(c: vec2<i32>) -> vec4<f32> {\n"
             "    return pin_ray_casting.data[c.y * i32(pin_size.x) + c.x];\n}\n"
             "fn pin_load_mapping(c: vec2<i32>) -> vec4<f32> {\n"
             "    return pin_mapping.data[c.y * i32(pin_size.x) + c.x];\n}")
    s = sub1(s, "@group(0) @binding(1)\nvar mapping: texture_2d<f32>;", "var<private> pin_mapping: PinTexels;")
    s = sub1(s, "@group(0) @binding(2)\nvar ttarget: texture_storage_2d<rgba8unorm, write>;",
             "var<private> pin_color: vec4<f32>;")
    s = sub1(s, "@group(0) @binding(3)\nvar<uniform> settings: Settings;", "var<private> settings: Settings;")
    s = sub1(s, "    data: array<f32>,", f"    data: array<f32, {MAX_TEXELS}>,")
    s = sub1(s, "@group(0) @binding(4)\nvar<storage, read_write> exponents: Exponents;",
             "var<private> exponents: Exponents;")
    s = sub1(s, "textureLoad(ray_casting, coords, 0)", "pin_load_color(coords)")
    s = re.sub(r"textureLoad\(mapping, (coords [+-] vec2<i32>\([^;]*?\)), 0\)", r"pin_load_mapping(\1)", s)
    if "textureLoad" in s:
        raise SystemExit("unreplaced textureLoad in src/overlay.wgsl")
    s = suball(s, "textureDimensions(ttarget)", "pin_size")
    s = sub1(s, "textureStore(ttarget, coords, color);", "pin_color = color;")
    s = sub1(s, "textureStore(ttarget, coords, vec4<f32>(srgb_from_linear(color.rgb), color.a));",
             "pin_color = vec4<f32>(srgb_from_linear(color.rgb), color.a);")
    for entry in ("overlay_desktop", "overlay_web"):
        s = sub1(s, f"@compute @workgroup_size(8, 8)\nfn {entry}(@builtin(global_invocation_id) gid: vec3<u32>)",
                 f"fn {entry}(gid: vec3<u32>)")
    return rename_helpers(s)


HARNESS = r"""
#include <memory>
using namespace linon_user;
typedef ::wgsl::vec<float, 4> f4;

static void load_scene(Private& pv, const float* cam, const float* st, const int* sti, const float* verts,
                       int nv, const unsigned* faces, int nf, const float* exps, int ne, int W, int H) {
  pv.u_camera.m_origin = f4(cam[0], cam[1], cam[2], cam[3]);
  pv.u_camera.m_view_direction = f4(cam[4], cam[5], cam[6], cam[7]);
  pv.u_camera.m_up = f4(cam[8], cam[9], cam[10], cam[11]);
  pv.u_settings = s_Settings(st[0], st[1], st[2], sti[0], sti[1], st[3]);
  for (int k = 0; k < nv; ++k) pv.u_vertices.m_data[k] = s_Vertex(verts[3 * k], verts[3 * k + 1], verts[3 * k + 2]);
  for (int k = 0; k < nf; ++k) pv.u_faces.m_data[k] = s_Face(faces[3 * k], faces[3 * k + 1], faces[3 * k + 2]);
  for (int k = 0; k < ne; ++k) pv.u_exponents.m_data[k] = exps[k];
  pv.u_pin_size = ::wgsl::vec<unsigned, 2>(unsigned(W), unsigned(H));
  pv.u_pin_n_faces = unsigned(nf);
}

// One main_view invocation per gid, each with fresh private state.
extern "C" void pin_main_view(const float* cam, const float* st, const int* sti, const float* verts, int nv,
                              const unsigned* faces, int nf, const float* exps, int ne, int W, int H,
                              const int* gids, int n, float* color, float* mapping, float* samples) {
  for (int i = 0; i < n; ++i) {
    std::unique_ptr<Private> pv(new Private());
    load_scene(*pv, cam, st, sti, verts, nv, faces, nf, exps, ne, W, H);
    const unsigned gx = unsigned(gids[2 * i]), gy = unsigned(gids[2 * i + 1]);
    u_main_view(*pv, ::wgsl::vec<unsigned, 3>(gx, gy, 0u));
    const f4 c = pv->u_pin_color, m = pv->u_pin_mapping;
    const float cv[8] = {c.x, c.y, c.z, c.w, m.x, m.y, m.z, m.w};
    for (int k = 0; k < 4; ++k) { color[4 * i + k] = cv[k]; mapping[4 * i + k] = cv[4 + k]; }
    if (samples && gy == 0 && gx < 8)
      for (int k = 0; k < 100; ++k) {
        const f4 p = pv->u_ray_samples.m_data[int(gx) * 100 + k].m_position;
        float* o = samples + (size_t(i) * 100 + k) * 4;
        o[0] = p.x; o[1] = p.y; o[2] = p.z; o[3] = p.w;
      }
  }
}
"""

OVERLAY_HARNESS = r"""
#include <memory>
using namespace linon_user;
typedef ::wgsl::vec<float, 4> f4;

// One overlay invocation per pixel (web: the sRGB entry point); exponents
// holds what the invocation wrote at its own index (-1: nothing).
extern "C" void pin_overlay(const float* st, const int* sti, const float* rc, const float* map, int W, int H,
                            int web, float* color, float* expo) {
  std::unique_ptr<Private> base(new Private());
  base->u_settings = s_Settings(st[0], st[1], st[2], sti[0], sti[1], st[3]);
  for (int k = 0; k < W * H; ++k) {
    base->u_pin_ray_casting.m_data[k] = f4(rc[4 * k], rc[4 * k + 1], rc[4 * k + 2], rc[4 * k + 3]);
    base->u_pin_mapping.m_data[k] = f4(map[4 * k], map[4 * k + 1], map[4 * k + 2], map[4 * k + 3]);
  }
  base->u_pin_size = ::wgsl::vec<unsigned, 2>(unsigned(W), unsigned(H));
  for (int k = 0; k < W * H; ++k) base->u_exponents.m_data[k] = -1.0f;
  for (int gy = 0; gy < H; ++gy)
    for (int gx = 0; gx < W; ++gx) {
      std::unique_ptr<Private> pv(new Private(*base));
      if (web) u_overlay_web(*pv, ::wgsl::vec<unsigned, 3>(unsigned(gx), unsigned(gy), 0u));
      else u_overlay_desktop(*pv, ::wgsl::vec<unsigned, 3>(unsigned(gx), unsigned(gy), 0u));
      const int row = H - gy - 1, pix = row * W + gx;
      const f4 c = pv->u_pin_color;
      color[4 * pix] = c.x; color[4 * pix + 1] = c.y; color[4 * pix + 2] = c.z; color[4 * pix + 3] = c.w;
      expo[pix] = pv->u_exponents.m_data[H * row + gx];
    }
}
"""


def compile_host(cpp: str, harness: str, tag: str):
    d = Path(tempfile.mkdtemp(prefix=f"linon_pin_{tag}_"))
    (d / "m.cpp").write_text("\n".join([f'#include "{RT}"', cpp, harness]))
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-shared", "-fPIC", "-o", str(d / "m.so"),
                        str(d / "m.cpp")], capture_output=True, text=True)
    if r.returncode != 0:
        raise SystemExit(r.stderr[-4000:])
    return C.CDLL(str(d / "m.so"))


def ptr(a):
    return a.ctypes.data_as(C.c_void_p)


# Field bodies by this package's field names; "identity" is the shader's
# own placeholder body.
FIELDS = {"identity": None, "mirage_spherical": "MirageSpherical", "mirage_plane": "MiragePlane",
          "mirage_spherical_sigmoid": "MirageSphericalSigmoid", "mirage_plane_sigmoid": "MiragePlaneSigmoid",
          "translation_x": "TranslationX", "translation_z": "TranslationZ", "rotation": "Rotation",
          "lorenz": "LorenzAttractor", "roessler": "RoesslerAttractor"}
SAMPLED = ("identity", "lorenz", "roessler", "mirage_spherical", "rotation")


def scene_arrays():
    from linon_gb300 import camera as cam
    xyz, faces, _, center = scene.cornell_reference()
    c = cam.arcball_default(center)
    camera = np.array(list(c.origin) + list(c.view_direction) + list(c.up), np.float32)
    return np.ascontiguousarray(xyz, np.float32), np.ascontiguousarray(faces, np.uint32), camera


def run_main_view(lib, camera, settings_f, settings_i, xyz, faces, exps, W, H, gids, samples: bool):
    n = len(gids)
    color = np.zeros((n, 4), np.float32)
    mapping = np.zeros((n, 4), np.float32)
    smp = np.zeros((n, 100, 4), np.float32) if samples else None
    e = np.ascontiguousarray(exps, np.float32)
    g = np.ascontiguousarray(gids, np.int32)
    lib.pin_main_view(ptr(camera), ptr(settings_f), ptr(settings_i), ptr(xyz), len(xyz), ptr(faces), len(faces),
                      ptr(e), len(e), W, H, ptr(g), n, ptr(color), ptr(mapping),
                      ptr(smp) if samples else None)
    return color, mapping, smp


def outline_exponents(W, H):
    """A ring of exponents >= 0.8 around the image centre (the outline scans
    find its extreme points), below 0.8 elsewhere."""
    y, x = np.mgrid[0:H, 0:W].astype(np.float32)
    r = np.hypot(x - 0.45 * W, y - 0.55 * H)
    return np.where(np.abs(r - 0.3 * min(W, H)) < 2.0, 1.0, 0.3).astype(np.float32)


def main():
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_shader_pins.py <path of the linon source tree>")
    ref = Path(sys.argv[1])
    bodies = predefined_bodies(ref)
    xyz, faces, camera = scene_arrays()
    if len(xyz) > MAX_VERTICES or len(faces) > MAX_FACES:
        raise SystemExit("scene larger than the fixed arrays")
    rng = np.random.default_rng(77)
    settings_f = np.array([1.0, 0.3, 0.6, 0.0], np.float32)  # field_weight, mouse x, mouse y, lyapunov_scaling
    settings_i = np.array([0, 1], np.int32)                 # overlay_mode, central_difference_delta
    data = {"scene/xyz": xyz, "scene/faces": faces, "scene/camera": camera,
            "scene/raw_sha256": np.array(scene_digest(ref)),
            "main/settings_f": settings_f, "main/settings_i": settings_i}
    sample_gids = np.array([[x, 0] for x in range(8)], np.int32)

    def pixels(W, H, n):
        k = rng.choice(W * H, size=n, replace=False)
        return np.stack([k % W, k // W], axis=1).astype(np.int32)

    def module(variant, field):
        body = "return v;" if FIELDS[field] is None else rename_helpers(bodies[FIELDS[field]])
        return compile_host(translate_wgsl(body, main_view_module(ref, **variant)), HARNESS, field)

    empty = np.zeros(1, np.float32)
    for field in FIELDS:
        lib = module({}, field)
        W, H = 48, 40
        gids = np.concatenate([pixels(W, H, 24), sample_gids]) if field in SAMPLED else pixels(W, H, 24)
        color, mapping, smp = run_main_view(lib, camera, settings_f, settings_i, xyz, faces, empty, W, H, gids,
                                            samples=field in SAMPLED)
        data.update({f"view/{field}/gids": gids, f"view/{field}/color": color, f"view/{field}/mapping": mapping})
        if smp is not None:
            data[f"view/{field}/samples"] = smp[-8:]
        if field in ("lorenz", "mirage_spherical"):
            lib = module({"high_accuracy": True}, field)
            gids = pixels(W, H, 6)
            color, mapping, _ = run_main_view(lib, camera, settings_f, settings_i, xyz, faces, empty, W, H, gids,
                                              samples=False)
            data.update({f"high/{field}/gids": gids, f"high/{field}/color": color,
                         f"high/{field}/mapping": mapping})
        print("main_view", field, flush=True)
    lib = module({"linear": True}, "identity")
    gids = pixels(48, 40, 24)
    color, _, _ = run_main_view(lib, camera, settings_f, settings_i, xyz, faces, empty, 48, 40, gids, samples=False)
    data.update({"linear/identity/gids": gids, "linear/identity/color": color})
    # outline rays: a square frame (the scans index exponents y * height + x)
    S = 32
    exps = outline_exponents(S, S)
    lib = module({"outline": True}, "lorenz")
    _, _, smp = run_main_view(lib, camera, settings_f, settings_i, xyz, faces, exps.ravel(), S, S, sample_gids,
                              samples=True)
    data.update({"outline/lorenz/exponents": exps, "outline/lorenz/samples": smp})

    # overlay: random colours and a smooth endpoint map; the scalings put
    # about half of the exponents above the 0.8 blend threshold
    olib = compile_host(translate_wgsl("return v;", overlay_module(ref)), OVERLAY_HARNESS, "overlay")
    W, H = 40, 40
    rgba8 = rng.integers(0, 256, size=(H, W, 4), dtype=np.uint8)
    y, x = np.mgrid[0:H, 0:W].astype(np.float32) / np.float32(W)
    mp = np.stack([np.sin(3 * x) * np.cos(2 * y), x * y + 0.2 * np.sin(9 * x), np.cos(4 * y) + x,
                   np.ones_like(x)], axis=-1).astype(np.float32)
    rc = (rgba8.astype(np.float32) / np.float32(255.0)).astype(np.float32)
    data.update({"overlay/rgba8": rgba8, "overlay/mapping": mp})
    for name, web, delta, scaling in (("desktop_d1", 0, 1, 60.0), ("desktop_d2", 0, 2, 30.0), ("web_d1", 1, 1, 60.0)):
        st_f = np.array([1.0, 0.0, 0.0, scaling], np.float32)
        st_i = np.array([1, delta], np.int32)
        color = np.zeros((H, W, 4), np.float32)
        expo = np.zeros((H, W), np.float32)
        olib.pin_overlay(ptr(st_f), ptr(st_i), ptr(np.ascontiguousarray(rc)), ptr(mp), W, H, web, ptr(color),
                         ptr(expo))
        data.update({f"overlay/{name}/settings_f": st_f, f"overlay/{name}/settings_i": st_i,
                     f"overlay/{name}/web": np.int32(web), f"overlay/{name}/color": color,
                     f"overlay/{name}/exponents": expo})
    out = Path(__file__).resolve().parent / "shader_pins.npz"
    np.savez_compressed(out, **data)
    print("wrote", out, sum(v.nbytes for v in data.values()), "bytes uncompressed")


if __name__ == "__main__":
    main()
