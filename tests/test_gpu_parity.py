"""CUDA engine vs the oracle, through the C ABI (GPU).

Bars (written per test):
  * LINON_COMPILE_PRECISE modules are op-for-op the FP32 restatement: for
    fields whose arithmetic is + - * / sqrt only, every plane is bit-exact
    (colour within 1/255: the specular pow is CUDA's powf vs the C library's).
  * Fields with transcendental calls (CUDA's sinf/expf/powf vs the C
    library's) agree to FP32 tolerance: hit ids on >= 99% of pixels, endpoint
    difference small except on the pixels whose hit differs.
  * Fast modules (FMA contraction) are held to the FP64 oracle: endpoint
    error <= 1e-4 scene units and hit-id mismatch <= 0.1% on smooth fields.
  * BVH traversal == brute force (bit-exact, same module).
"""
import numpy as np
import pytest
import torch

from linon_gb300 import FramePlanes, _abi, camera as cam, scene, workloads as wl
from linon_gb300.engine import predefined_source, validate_field

pytestmark = pytest.mark.gpu

EXACT_FIELDS = ["identity", "linear", "lorenz", "roessler", "translation_x", "mirage_spherical", "mirage_plane"]
TRANSC_FIELDS = ["twist", "rotation", "mirage_spherical_sigmoid", "lens"]

_fields = {}


def field(engine, name, precise):
    key = (name, precise)
    if key not in _fields:
        _fields[key] = engine.compile_field(predefined_source(_abi.FIELD_IDS[name]), precise=precise)
    return _fields[key]


def gpu_render(engine, w, fld, width=None, height=None, params=None, settings=None, camera=None):
    W, H = width or w.width, height or w.height
    f = FramePlanes.allocate(W, H)
    engine.render(fld, camera or w.camera, settings or w.settings, params or w.params, f)
    torch.cuda.synchronize()
    engine.synchronize()
    return {k: getattr(f, k).cpu().numpy() for k in ("color", "mapping", "hit_id", "steps")}


def oracle_render(oracle, w, fid, width, height, params=None, settings=None, camera=None, precision=32):
    want = ("color", "mapping", "hit_id", "steps") if precision == 32 else ("mapping64", "hit_id", "steps")
    return oracle.render(w.xyz, w.faces, w.face_rgb, camera or w.camera, settings or w.settings, params or w.params,
                         fid, width, height, precision=precision, want=want)


def steps_case():
    w = wl.plain_small(96, 64)
    w.settings.field_weight = 0.75
    w.params = wl.fixed_steps(0.05, 80, kahan=True)
    return w


def ref_case():
    return wl.reference_default(96, 64)


def assert_exact(g, o, color_tol=1):
    """Bit-exact hit ids, step counts and endpoints; a NaN matches a NaN of
    any sign or payload (CUDA's arithmetic makes 0x7fffffff, the host's
    0x7fc00000 or its negation; WGSL gives NaNs no bit pattern)."""
    np.testing.assert_array_equal(g["hit_id"], o["hit_id"])
    np.testing.assert_array_equal(g["steps"], o["steps"])
    gn, on = np.isnan(g["mapping"]), np.isnan(o["mapping"])
    np.testing.assert_array_equal(gn, on)
    np.testing.assert_array_equal(np.where(gn, 0, g["mapping"].view(np.uint32)), np.where(on, 0, o["mapping"].view(np.uint32)))
    assert np.abs(g["color"].astype(int) - o["color"].astype(int)).max() <= color_tol


def long_steps_case():
    """Steps of 0.37 (segments longer than the cell lists reach, so the BVH
    walk tests them) and of 1.9 (a segment can cross the whole room)."""
    w = wl.plain_small(80, 60)
    w.params = wl.fixed_steps(0.37, 12, kahan=False)
    return w


@pytest.mark.parametrize("bvh", [False, True])
@pytest.mark.parametrize("case", ["steps", "reference", "long_steps", "room_steps"])
@pytest.mark.parametrize("name", EXACT_FIELDS)
def test_precise_bit_exact(engine, oracle, name, case, bvh):
    if case in ("long_steps", "room_steps"):
        w = long_steps_case()
        if case == "room_steps":
            w.params = wl.fixed_steps(1.9, 4, kahan=True)
    else:
        w = steps_case() if case == "steps" else ref_case()
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=bvh)
    g = gpu_render(engine, w, field(engine, name, True))
    o = oracle_render(oracle, w, _abi.FIELD_IDS[name], w.width, w.height)
    assert_exact(g, o)


@pytest.mark.parametrize("weight", [0.0, 1.0, 1.5])
@pytest.mark.parametrize("view", ["degenerate_up", "from_inside", "grazing"])
@pytest.mark.parametrize("name", ["lorenz", "translation_x"])
def test_precise_cameras_and_weights(engine, oracle, name, view, weight):
    """Field weights 0 (straight rays), 1 (the blend-free kernel variant) and
    1.5 (extrapolation), with a camera whose up vector is its view direction
    (the shader's basis is NaN: every ray is NaN), one inside the room, and
    one grazing the floor; precise module bit-exact to the FP32 oracle."""
    from linon_gb300 import camera as cam
    w = wl.plain_small(72, 40)
    w.params = wl.fixed_steps(0.03, 90, kahan=True)
    w.settings.field_weight = weight
    if view == "degenerate_up":
        w.camera = cam.make_camera((0.0, 3.0, 0.0), (0.0, -1.0, 0.0), (0.0, -1.0, 0.0))
    elif view == "from_inside":
        w.camera = cam.make_camera((0.1, -0.2, 0.3), (0.2, 0.3, -0.93), (0.0, 1.0, 0.0))
    else:
        w.camera = cam.make_camera((-0.9, -0.999, 0.9), (0.7, 0.0005, -0.7), (0.0, 1.0, 0.0))
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    g = gpu_render(engine, w, field(engine, name, True))
    o = oracle_render(oracle, w, _abi.FIELD_IDS[name], 72, 40)
    assert_exact(g, o)
    if view == "degenerate_up":
        assert np.isnan(g["mapping"][..., :3]).all()


@pytest.mark.parametrize("name", TRANSC_FIELDS)
def test_precise_transcendental_fields_close(engine, oracle, name):
    w = steps_case()
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    g = gpu_render(engine, w, field(engine, name, True))
    o = oracle_render(oracle, w, _abi.FIELD_IDS[name], w.width, w.height)
    same = g["hit_id"] == o["hit_id"]
    assert same.mean() >= 0.99
    np.testing.assert_array_equal(g["steps"], o["steps"])
    d = np.abs(g["mapping"][..., :3] - o["mapping"][..., :3]).max(axis=-1)
    tol = 1e-2 if name == "lens" else 1e-4  # lens orbits are chaotic near the origin
    assert np.percentile(d[same], 99) <= tol


@pytest.mark.parametrize("precise", [True, False])
def test_reference_default_frame(engine, oracle, precise):
    """The reference application's first frame: the Cornell box as
    application.rs prepares it, the arcball default camera, the spherical
    sigmoid mirage field, the shader's t <= 5 loop (h = 0.1, adaptive), at
    200x150.

    The shader's refinement test (diff > 10 * last_diff) compares velocity
    changes that, away from the heated region, are rounding noise: the FP32
    and FP64 oracles agree on the step count of only ~0.2% of these pixels
    (median 82 vs 1342 steps) while agreeing on 99.8% of hit ids.  Step counts
    are therefore held exactly only for the precise module (op-for-op the
    FP32 oracle; exp differs in the last bit, so >= 98% of pixels); the fast
    module (FMA) is held to what survives rounding: hit ids on >= 98% of
    pixels and endpoints within 0.12 at the 99th percentile: one coarse step
    (0.1, the spread of the last step past t = 5) plus 20%; the FP32 and FP64
    oracles differ by 0.084 there."""
    w = wl.reference_default(200, 150)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    g = gpu_render(engine, w, field(engine, "mirage_spherical_sigmoid", precise))
    o = oracle_render(oracle, w, _abi.FIELD_IDS["mirage_spherical_sigmoid"], w.width, w.height)
    hit_ok = np.mean(g["hit_id"] == o["hit_id"])
    assert hit_ok >= (0.99 if precise else 0.98), hit_ok
    d = np.abs(g["mapping"][..., :3] - o["mapping"][..., :3]).max(axis=-1)
    if precise:
        steps_ok = np.mean(g["steps"] == o["steps"])
        assert steps_ok >= 0.98, steps_ok
        same = (g["steps"] == o["steps"]) & (g["hit_id"] == o["hit_id"])
        assert np.percentile(d[same], 99) <= 1e-4
    else:
        assert np.percentile(d, 99) <= 0.12, np.percentile(d, 99)
    assert (o["steps"] >= 51).all() and (g["steps"] >= 51).all()  # t <= 5 at h <= 0.1


@pytest.mark.parametrize("name", ["linear", "twist", "lens"])
def test_fast_vs_fp64_1080p(engine, oracle, name):
    """The 1080p workload (h = 0.005, 4000 steps, Kahan sums), fast module,
    full frame on the GPU, 4000 random pixels against the FP64 oracle.
    Bars: endpoint error <= 1e-4 scene units on smooth fields; hit-id
    mismatch <= 0.1% excluding coplanar ties (light panel / ceiling, block
    footprints / floor: which of two coplanar faces a ray meets is a rounding
    tie).  The lens field's rays are captured into orbits around the origin,
    a chaotic region where FP32 and FP64 separate; its error is recorded, not
    bounded at 1e-4."""
    w = wl.frames_1080p()
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    g = gpu_render(engine, w, field(engine, name, False))
    rng = np.random.default_rng(11)
    pix = np.sort(rng.choice(w.width * w.height, 4000, replace=False)).astype(np.int32)
    o = oracle.render(w.xyz, w.faces, w.face_rgb, w.camera, w.settings, w.params, _abi.FIELD_IDS[name], w.width,
                      w.height, pixels=pix, precision=64, want=("mapping64", "hit_id", "steps"))
    gm = g["mapping"].reshape(-1, 4)[pix, :3].astype(np.float64)
    gh = g["hit_id"].ravel()[pix]
    err = np.abs(gm - o["mapping64"][:, :3]).max(axis=-1)
    groups = scene.coplanar_groups(w.xyz, w.faces)
    diff = gh != o["hit_id"]
    tie = diff & (gh >= 0) & (o["hit_id"] >= 0)
    tie[tie] = groups[gh[tie]] == groups[o["hit_id"][tie]]
    assert np.mean(diff & ~tie) <= 0.001
    assert (g["steps"] == 4000).all()
    if name == "lens":
        assert np.percentile(err, 50) < 0.05
    else:
        assert err.max() <= 1e-4, err.max()


def test_plain_small_512_config(engine, oracle):
    """The 512x512 twist workload (h = 0.01, 1000 steps, per-face colours):
    the precise module against the FP32 oracle and the fast module within
    1e-4 of the FP64 oracle, on 2000 seeded pixels of the full frame (hit
    mismatch <= 0.1% outside coplanar ties)."""
    w = wl.plain_small()
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    rng = np.random.default_rng(5)
    pix = np.sort(rng.choice(w.width * w.height, 2000, replace=False)).astype(np.int32)
    fid = _abi.FIELD_IDS["twist"]
    gp = gpu_render(engine, w, field(engine, "twist", True))
    o32 = oracle.render(w.xyz, w.faces, w.face_rgb, w.camera, w.settings, w.params, fid, w.width, w.height,
                        pixels=pix, want=("color", "mapping", "hit_id", "steps"))
    # sin/cos are CUDA's in the module and the C library's in the oracle
    # (last-bit differences): hit ids on >= 99.5% of the pixels, endpoints of
    # the agreeing pixels within 1e-5
    same = gp["hit_id"].ravel()[pix] == o32["hit_id"]
    assert same.mean() >= 0.995, same.mean()
    np.testing.assert_array_equal(gp["steps"].ravel()[pix], o32["steps"])
    d32 = np.abs(gp["mapping"].reshape(-1, 4)[pix, :3] - o32["mapping"][:, :3]).max(-1)
    assert np.percentile(d32[same], 99) <= 1e-5, np.percentile(d32[same], 99)
    gf = gpu_render(engine, w, field(engine, "twist", False))
    o64 = oracle.render(w.xyz, w.faces, w.face_rgb, w.camera, w.settings, w.params, fid, w.width, w.height,
                        pixels=pix, precision=64, want=("mapping64", "hit_id", "steps"))
    err = np.abs(gf["mapping"].reshape(-1, 4)[pix, :3].astype(np.float64) - o64["mapping64"][:, :3]).max(-1)
    gh = gf["hit_id"].ravel()[pix]
    groups = scene.coplanar_groups(w.xyz, w.faces)
    diff = gh != o64["hit_id"]
    tie = diff & (gh >= 0) & (o64["hit_id"] >= 0)
    tie[tie] = groups[gh[tie]] == groups[o64["hit_id"][tie]]
    assert np.mean(diff & ~tie) <= 0.001
    assert err.max() <= 1e-4, err.max()
    assert (gf["steps"] == 1000).all()


def test_fast_math_accuracy(engine):
    """Fast modules' sin/cos (one Cody-Waite reduction by 2 pi, then the
    special-function unit on r = x - k 2 pi) and constant-exponent pow
    against FP64.  Bars: < 5e-7 absolute for |t| <= 3000 (the unit's
    documented 2^-21.41 on [-pi, pi] plus the reduced argument's 1.3e-7);
    < 1e-6 for |t| < 2^22, where the rounding of t / (2 pi) can leave |r| a
    little above pi, outside the unit's most accurate range."""
    body = "return vec3<f32>(sin(t), cos(t), pow(p.x, 1.5));"
    fld = engine.compile_field(body)
    n = 1 << 18
    rng = np.random.default_rng(2)
    x = np.zeros((n, 13), np.float32)
    small = n // 2 + n // 4
    x[:, 12] = np.concatenate([rng.uniform(-4, 4, n // 2), rng.uniform(-3000, 3000, n // 4),
                               rng.uniform(-4.0e6, 4.0e6, n // 4)]).astype(np.float32)
    x[:, 3] = rng.uniform(0, 50, n).astype(np.float32)
    out = engine.field_eval(fld, torch.from_numpy(x).cuda()).cpu().numpy().astype(np.float64)
    t = x[:, 12].astype(np.float64)
    es, ec = np.abs(out[:, 0] - np.sin(t)), np.abs(out[:, 1] - np.cos(t))
    assert es[:small].max() <= 5e-7 and ec[:small].max() <= 5e-7, (es[:small].max(), ec[:small].max())
    assert es.max() <= 1e-6 and ec.max() <= 1e-6, (es.max(), ec.max())
    ref = x[:, 3].astype(np.float64) ** 1.5
    assert (np.abs(out[:, 2] - ref) / np.maximum(ref, 1e-30)).max() <= 3.6e-7


@pytest.mark.parametrize("name", ["twist", "lens", "lorenz_scaled"])
def test_bvh_equals_brute_force_cornell(engine, name):
    """BVH culling + safe-ball skipping vs the plain loop over all faces, on
    fields whose rays travel far from (twist), orbit near (lens) and swirl
    around (scaled Lorenz) the geometry."""
    w = wl.plain_small(256, 256)
    fld = field(engine, name, False)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=False)
    a = gpu_render(engine, w, fld)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    assert engine.scene_info()["nodes"] > 1
    b = gpu_render(engine, w, fld)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])


def test_bvh_equals_brute_force_spheres(engine):
    xyz, faces, rgb = scene.cornell_with_spheres(seed=0)
    assert len(faces) == 36 + 4 * 20480
    views = wl.batch_views(3, seed=1, min_side=96, max_side=128)
    fld = field(engine, "twist", False)
    for W, H, camera, params, _ in views:
        params.stop_on_hit = 1
        w = wl.Workload("v", xyz, faces, rgb, W, H, camera, wl.settings(), params)
        engine.upload_scene(xyz, faces, rgb, bvh=False)
        a = gpu_render(engine, w, fld)
        engine.upload_scene(xyz, faces, rgb, bvh=True)
        b = gpu_render(engine, w, fld)
        for k in a:
            np.testing.assert_array_equal(a[k], b[k])


def degenerate_scene():
    """The Cornell room plus triangles that stress culling and ties: two equal
    vertices, three collinear ones, a point, a 1e-4 triangle, a 1e-5 sliver
    across the room, a large slanted triangle through it, and a second copy
    of a wall face (equal hits: the lower face index wins)."""
    room = scene.cornell_unit()
    a, b = np.array([-0.3, -0.2, 0.1]), np.array([0.4, 0.3, -0.2])
    c = np.array([0.1, 0.0, 0.0])
    tris = [
        [a, a, b],
        [a, b, (a + b) / 2],
        [a, a, a],
        [c, c + [1e-4, 0, 0], c + [0, 1e-4, 0]],
        [[-0.9, 0.2, -0.5], [0.9, 0.2, 0.5], [0.9, 0.2 + 1e-5, 0.5]],
        [[-0.95, -0.9, -0.8], [0.9, -0.2, -0.9], [0.1, 0.95, 0.7]],
        list(room[0][room[1][4]].astype(np.float64)),
    ]
    x = np.array([v for t in tris for v in t], np.float32)
    f = np.arange(len(x), dtype=np.uint32).reshape(-1, 3)
    rgb = np.linspace(0.2, 0.9, 3 * len(f), dtype=np.float32).reshape(-1, 3)
    return scene.merge(room, (x, f, rgb))


@pytest.mark.parametrize("name", ["twist", "lens", "lorenz_scaled"])
def test_bvh_equals_brute_force_degenerate_triangles(engine, oracle, name):
    """On the degenerate scene: the BVH path equals the loop over every face
    (fast module), and for the transcendental-free field the precise module
    equals the FP32 oracle bit for bit (hit ids, step counts, endpoints)."""
    xyz, faces, rgb = degenerate_scene()
    w = wl.plain_small(160, 120)
    w.xyz, w.faces, w.face_rgb = xyz, faces, rgb
    w.params = wl.fixed_steps(0.01, 400, kahan=True)
    fld = field(engine, name, False)
    engine.upload_scene(xyz, faces, rgb, bvh=False)
    a = gpu_render(engine, w, fld)
    engine.upload_scene(xyz, faces, rgb, bvh=True)
    assert engine.scene_info()["nodes"] > 1
    b = gpu_render(engine, w, fld)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    if name == "lorenz_scaled":  # op-for-op (sin, cos and pow are library calls on both sides)
        g = gpu_render(engine, w, field(engine, name, True))
        o = oracle_render(oracle, w, _abi.FIELD_IDS[name], 160, 120)
        assert_exact(g, o)


@pytest.mark.parametrize("size", [(1, 1), (2, 2), (33, 17), (7, 130)])
def test_odd_and_tiny_sizes(engine, oracle, size):
    W, H = size
    w = steps_case()
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    g = gpu_render(engine, w, field(engine, "linear", True), W, H)
    o = oracle_render(oracle, w, _abi.FIELD_IDS["linear"], W, H)
    np.testing.assert_array_equal(g["hit_id"], o["hit_id"])
    np.testing.assert_array_equal(np.isnan(g["mapping"]), np.isnan(o["mapping"]))
    m = ~np.isnan(o["mapping"])
    np.testing.assert_array_equal(g["mapping"][m], o["mapping"][m])


def test_frame_size_limits(engine, oracle):
    """The largest accepted width (65535) renders like the oracle; sizes
    beyond the limits (65536 per side, 2^31 - 1 pixels, zero) are rejected
    with LINON_EINVAL before any output pointer is touched."""
    import ctypes as C
    w = steps_case()
    w.params = wl.fixed_steps(0.05, 8)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fld = field(engine, "linear", True)
    g = gpu_render(engine, w, fld, 65535, 2)
    cols = np.r_[0:64, 32000:32064, 65471:65535]
    pix = np.concatenate([cols, 65535 + cols]).astype(np.int32)
    o = oracle.render(w.xyz, w.faces, w.face_rgb, w.camera, w.settings, w.params, _abi.FIELD_IDS["linear"], 65535, 2,
                      pixels=pix, want=("mapping", "hit_id", "steps"))
    np.testing.assert_array_equal(g["hit_id"].ravel()[pix], o["hit_id"])
    np.testing.assert_array_equal(g["mapping"].reshape(-1, 4)[pix].view(np.uint32), o["mapping"].view(np.uint32))
    lib = _abi.load()
    for W, H in ((65536, 1), (1, 65536), (65535, 65535), (0, 5), (5, -1)):
        f = _abi.Frame()
        f.width, f.height = W, H  # null planes: only the size check may run
        st = lib.linon_render(engine.ctx, fld.handle, C.byref(w.camera), C.byref(w.settings), C.byref(w.params),
                              C.byref(f))
        assert st == _abi.LINON_EINVAL, (W, H, st)


def test_empty_scene_and_linear_mode(engine, oracle):
    w = steps_case()
    engine.upload_scene(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32), None, bvh=True)
    g = gpu_render(engine, w, field(engine, "linear", True))
    assert (g["hit_id"] == -1).all()
    assert (g["color"][..., :3] == 0).all() and (g["color"][..., 3] == 255).all()
    # linear_mode (main_view.wgsl:368-370): one straight ray, max distance 100
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    p = wl.fixed_steps(0.05, 80)
    p.linear_mode = 1
    g = gpu_render(engine, w, field(engine, "linear", True), params=p)
    o = oracle_render(oracle, w, _abi.FIELD_IDS["linear"], w.width, w.height, params=p)
    np.testing.assert_array_equal(g["hit_id"], o["hit_id"])
    assert np.abs(g["color"].astype(int) - o["color"].astype(int)).max() <= 1


def test_render_host_matches_device(engine):
    w = steps_case()
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fld = field(engine, "lorenz", True)
    d = gpu_render(engine, w, fld)
    h = engine.render_host(fld, w.camera, w.settings, w.params, w.width, w.height)
    for k in d:
        np.testing.assert_array_equal(d[k], h[k])


@pytest.mark.parametrize("name", ["twist", "lens"])
@pytest.mark.parametrize("size", [(1920, 1080), (640, 417), (513, 1031)])
def test_render_host_bands_match_device(engine, size, name):
    """Frames of >= 2^18 pixels go to the host in row bands rendered on two
    streams while earlier bands are copied: every plane equals the one-launch
    device render (band edges at multiples of 16 rows, ragged last band); the
    1080p lens frame runs two rays per thread in both."""
    w = wl.frames_1080p(*size)
    w.params = wl.fixed_steps(0.01, 300, kahan=True)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fld = field(engine, name, False)
    d = gpu_render(engine, w, fld)
    h = engine.render_host(fld, w.camera, w.settings, w.params, w.width, w.height)
    if name == "lens" and size == (1920, 1080):
        assert fld.pair_state() == 1
    for k in d:
        np.testing.assert_array_equal(d[k], h[k])


def test_compile_error_through_engine(engine):
    with pytest.raises(_abi.LinonCompileError) as e:
        engine.compile_field("return nope;")
    assert "nope" in e.value.message
    with pytest.raises(_abi.LinonCompileError):
        engine.compile_field(predefined_source(0))  # Custom: empty body


@pytest.mark.parametrize("fp64", [False, True])
@pytest.mark.parametrize("srgb", [False, True])
def test_overlay_matches_oracle(engine, oracle, fp64, srgb):
    w = wl.lyapunov_1024(128, 128)
    w.params = wl.fixed_steps(0.01, 300, kahan=True)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    g = gpu_render(engine, w, field(engine, "lorenz_scaled", False))
    st = wl.settings(overlay_mode=1, delta=2, scaling=50.0)
    target = torch.empty((128, 128, 4), dtype=torch.uint8, device="cuda")
    expo = torch.zeros((128, 128), dtype=torch.float32, device="cuda")
    color = torch.from_numpy(g["color"]).cuda()
    mapping = torch.from_numpy(g["mapping"]).cuda()
    engine.overlay(st, 128, 128, color, mapping, target, expo, srgb=srgb, fp64=fp64)
    torch.cuda.synchronize()
    o_rgba, o_e = oracle.overlay(g["color"], g["mapping"], 128, 128, st, srgb=srgb, precision=64 if fp64 else 32)
    e = expo.cpu().numpy()
    np.testing.assert_allclose(e, o_e, rtol=1e-5, atol=1e-6)
    assert np.abs(target.cpu().numpy().astype(int) - o_rgba.astype(int)).max() <= 1


@pytest.mark.parametrize("fp64,srgb", [(True, False), (False, True)])
@pytest.mark.parametrize("delta", [1, 9, 10, 30])
def test_overlay_border_widths_match_oracle(engine, oracle, delta, fp64, srgb):
    """A non-square frame (96x40) with central-difference deltas whose 2*delta
    border leaves a few interior rows (9), none (10: rows 20..19) or covers
    the frame (30); both overlay modes; the exponents buffer is pre-filled
    with a sentinel, which border pixels keep in the engine as in the
    oracle."""
    w = wl.lyapunov_1024(96, 40)
    w.params = wl.fixed_steps(0.01, 150, kahan=True)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    g = gpu_render(engine, w, field(engine, "lorenz_scaled", False))
    color = torch.from_numpy(g["color"]).cuda()
    mapping = torch.from_numpy(g["mapping"]).cuda()
    for mode in (0, 1):
        st = wl.settings(overlay_mode=mode, delta=delta, scaling=50.0)
        target = torch.empty((40, 96, 4), dtype=torch.uint8, device="cuda")
        expo = torch.full((40, 96), -7.0, dtype=torch.float32, device="cuda")
        engine.overlay(st, 96, 40, color, mapping, target, expo, srgb=srgb, fp64=fp64)
        torch.cuda.synchronize()
        o_e = np.full((40, 96), -7.0, np.float32)
        o_rgba, o_e = oracle.overlay(g["color"], g["mapping"], 96, 40, st, srgb=srgb, precision=64 if fp64 else 32,
                                     exponents=o_e)
        np.testing.assert_allclose(expo.cpu().numpy(), o_e, rtol=1e-5, atol=1e-6)
        assert np.abs(target.cpu().numpy().astype(int) - o_rgba.astype(int)).max() <= 1


def test_ftle_matches_oracle(engine, oracle):
    w = wl.lyapunov_1024(96, 96)
    w.params = wl.fixed_steps(0.01, 200, kahan=True)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    g = gpu_render(engine, w, field(engine, "lorenz_scaled", False))
    mapping = torch.from_numpy(g["mapping"]).cuda()
    out = torch.empty((96, 96), dtype=torch.float32, device="cuda")
    engine.ftle(w.camera, w.params, 96, 96, mapping, 2.0, out)
    torch.cuda.synchronize()
    o = oracle.ftle(w.camera, w.params, 96, 96, g["mapping"], 2.0)
    np.testing.assert_allclose(out.cpu().numpy(), o, rtol=1e-6, atol=1e-6)


def test_capture_reference_matches_oracle(engine, oracle):
    w = ref_case()
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fld = field(engine, "lorenz", True)
    out = torch.zeros((800, 8), dtype=torch.float32, device="cuda")
    engine.capture_reference(fld, w.camera, w.settings, w.params, w.width, w.height, out)
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(8, 100, 8)
    ring = np.array([(-1, -1), (0, -1), (1, -1), (1, 0), (1, 1), (0, 1), (-1, 1), (-1, 0)], np.float32)
    pos = (np.float32([0.5, 0.6]) + np.float32(0.01) * ring).astype(np.float32)
    o = oracle.capture(_abi.FIELD_IDS["lorenz"], w.camera, w.settings, w.params, w.width, w.height, pos,
                       0.001, 5000, 50, False)
    np.testing.assert_array_equal(got[:, :, :4], o)
    assert (got[:, :, 7] == 0.5).all()
    np.testing.assert_array_equal(got[1, 0, 4:7], [0.5, 0.5, 0.0])


@pytest.mark.parametrize("n_steps,every", [(301, 7), (300, 1), (5, 10), (0, 3), (49, 49), (50, 49)])
def test_capture_paths_matches_oracle(engine, oracle, n_steps, every):
    """Recorded points every `every` steps from step 0, plus the final
    point: a step count that `every` does not divide, every step, fewer
    steps than `every`, no step, and `every` equal to the step count or one
    below it; bit-exact with the oracle (precise module)."""
    w = wl.plain_small(64, 64)
    fld = field(engine, "translation_x", True)
    rng = np.random.default_rng(3)
    pos = rng.uniform(0.2, 0.8, size=(37, 2)).astype(np.float32)
    npts = -(-n_steps // every) + 1
    out = torch.zeros((37, npts, 4), dtype=torch.float32, device="cuda")
    engine.capture_paths(fld, w.camera, w.settings, w.params, 64, 64, pos, 0.01, n_steps, every, out)
    torch.cuda.synchronize()
    o = oracle.capture(_abi.FIELD_IDS["translation_x"], w.camera, w.settings, w.params, 64, 64, pos, 0.01,
                       n_steps, every, True)
    np.testing.assert_array_equal(out.cpu().numpy(), o)


@pytest.mark.parametrize("shape", [(64, 64), (96, 48), (1, 1), (5, 3)])
def test_outline_select_matches_oracle(engine, oracle, shape):
    W, H = shape
    rng = np.random.default_rng(W * 7 + H)
    for density in (0.0, 0.01, 0.3, -1.0):
        e = (rng.random((H, W)) < abs(density)).astype(np.float32) * rng.uniform(0.8, 2.0, size=(H, W)).astype(
            np.float32)
        if density < 0:  # NaN (never selected), +inf (selected), -inf and a value just below the bar
            special = np.array([np.nan, np.inf, -np.inf, np.float32(0.8) - np.float32(1e-7)], np.float32)
            e = special[rng.integers(0, 4, size=(H, W))]
        t = torch.from_numpy(e).cuda()
        pix, pos = engine.outline_select(t, W, H, 0.8)
        o = oracle.outline_select(e, W, H, 0.8)
        np.testing.assert_array_equal(pix, o)


def test_quantile_matches_numpy(engine):
    rng = np.random.default_rng(5)
    e = rng.standard_normal((200, 300)).astype(np.float32)
    t = torch.from_numpy(e).cuda()
    for q in (0.0, 0.5, 0.95, 1.0):
        got = engine.exponent_quantile(t, 300, 200, q, border=3)
        inner = np.sort(e[3:-3, 3:-3].ravel())
        assert got == inner[int(np.floor(q * (len(inner) - 1)))]


def test_quantile_with_infinities_nans_and_signed_zeros(engine):
    """Exponent maps hold -inf (isolated pixels of the finite-time
    exponent), +inf and NaN of either sign; the quantile is numpy's sorted
    value at floor(q (n - 1)) with every NaN last and -0.0 equal to +0.0."""
    rng = np.random.default_rng(11)
    e = rng.standard_normal((60, 70)).astype(np.float32)
    flat = e.reshape(-1)
    idx = rng.permutation(flat.size)
    flat[idx[:40]] = -np.inf
    flat[idx[40:60]] = np.inf
    flat[idx[60:80]] = np.nan
    flat[idx[80:100]] = -np.float32(np.nan)
    flat[idx[100:130]] = 0.0
    flat[idx[130:160]] = -0.0
    assert np.signbit(flat[idx[80:100]]).all()
    t = torch.from_numpy(e).cuda()
    for border in (0, 2):
        inner = np.sort(e[border:60 - border, border:70 - border].ravel())
        for q in (0.0, 0.004, 0.25, 0.5, 0.9, 0.97, 0.99, 1.0):
            got = engine.exponent_quantile(t, 70, 60, q, border=border)
            want = inner[int(np.floor(q * (len(inner) - 1)))]
            assert (np.isnan(got) and np.isnan(want)) or got == want, (border, q, got, want)


@pytest.mark.parametrize("shape", [(1, 1), (2, 1), (1, 3), (5, 4)])
def test_ftle_tiny_frames_match_oracle(engine, oracle, shape):
    """Frames of one pixel (no neighbour: -inf; its ray direction is NaN as in
    the shader) and frames one pixel wide or high."""
    W, H = shape
    w = wl.lyapunov_1024(W, H)
    w.params = wl.fixed_steps(0.01, 50, kahan=True)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    g = gpu_render(engine, w, field(engine, "lorenz_scaled", False))
    mapping = torch.from_numpy(g["mapping"]).cuda()
    out = torch.empty((H, W), dtype=torch.float32, device="cuda")
    engine.ftle(w.camera, w.params, W, H, mapping, 0.5, out)
    torch.cuda.synchronize()
    o = oracle.ftle(w.camera, w.params, W, H, g["mapping"], 0.5)
    np.testing.assert_allclose(out.cpu().numpy(), o, rtol=1e-6, atol=1e-6)


def batch_setup(engine, precise, n=6, seed=4):
    xyz, faces, rgb = scene.cornell_with_spheres(seed=seed, subdivisions=2)
    engine.upload_scene(xyz, faces, rgb, bvh=True)
    names = ["linear", "twist", "lorenz_scaled"]
    flds = [field(engine, nme, precise) for nme in names]
    views, planes = [], []
    for (W, H, camera, params, fidx) in wl.batch_views(n, seed=seed, min_side=24, max_side=90, n_fields=3):
        params.max_steps = min(params.max_steps, 200)
        fp = FramePlanes.allocate(W, H)
        v = _abi.View()
        v.camera = camera
        v.settings = wl.settings()
        v.params = params
        v.width, v.height, v.field_index = W, H, fidx
        v.out = fp.abi()
        views.append(v)
        planes.append(fp)
    return flds, views, planes


def snapshot(planes):
    torch.cuda.synchronize()
    return [{k: getattr(p, k).cpu().numpy().copy() for k in ("color", "mapping", "hit_id", "steps")} for p in planes]


BATCH_FORMS = [(1, 0), (1, 8), (2, 0), (3, 0)]  # (schedule, refill_below)


@pytest.mark.parametrize("precise", [True, False])
@pytest.mark.parametrize("schedule,refill", BATCH_FORMS)
def test_batch_equals_plain(engine, precise, schedule, refill):
    """The four batched forms against one plain launch per view: the
    persistent queue of whole-warp tiles (schedule 1, refill_below 0), the
    persistent queue that refills lanes mid-ray (refill_below 8, a quantum of
    16 steps), one CTA per tile of every view (schedule 2) and the
    persistent queue of CTA tiles (schedule 3)."""
    flds, views, planes = batch_setup(engine, precise)
    engine.render_views_plain(flds, views)
    a = snapshot(planes)
    for p in planes:
        for k in ("color", "mapping", "hit_id", "steps"):
            getattr(p, k).zero_()
    tuning = _abi.BatchTuning(16, 64, 0, 8, 4, refill, schedule)
    engine.render_batch(flds, views, tuning)
    engine.synchronize()
    b = snapshot(planes)
    for x, y in zip(a, b):
        if precise:  # op-for-op modules: bit-exact
            for k in x:
                np.testing.assert_array_equal(x[k], y[k])
        else:
            # fast modules: FMA contraction may differ between the two
            # kernels' inlining contexts, so hold them to FP32 tolerance
            assert np.mean(x["hit_id"] != y["hit_id"]) <= 0.005
            same = (x["hit_id"] == y["hit_id"]) & (x["steps"] == y["steps"])
            assert same.mean() >= 0.99
            d = np.abs(x["mapping"] - y["mapping"]).max(axis=-1)
            assert np.percentile(d[same], 99) <= 1e-4


@pytest.mark.parametrize("schedule,refill", BATCH_FORMS)
def test_batch_tiny_and_mixed_views_equal_plain(engine, schedule, refill):
    """Views smaller than one tile or one warp (1x1, 1x37, 33x1, 7x5), one
    just past a tile edge (17x16), and mixed march parameters in one batch:
    fixed steps with Kahan sums and stop at the first hit, a single step,
    linear mode, the shader's own adaptive t-loop.  Precise modules, every
    batched form bit-exact against one plain launch per view."""
    xyz, faces, rgb = scene.cornell_with_spheres(seed=5, subdivisions=1)
    engine.upload_scene(xyz, faces, rgb, bvh=True)
    flds = [field(engine, nme, True) for nme in ("linear", "twist", "lorenz_scaled")]
    cams = wl.batch_views(7, seed=21, min_side=20, max_side=40, n_fields=3)
    sizes = [(1, 1), (1, 37), (33, 1), (7, 5), (17, 16), (40, 3), (9, 9)]
    plist = [wl.fixed_steps(0.02, 150, kahan=True, stop_on_hit=True), wl.fixed_steps(0.05, 1, kahan=True),
             wl.fixed_steps(0.02, 120, kahan=False), _abi.shader_params(), wl.fixed_steps(0.01, 90, kahan=True),
             wl.fixed_steps(0.02, 60, kahan=True, stop_on_hit=True), wl.fixed_steps(0.02, 80, kahan=True)]
    plist[2].linear_mode = 1
    views, planes = [], []
    for i, ((W, H), (_w, _h, camera, _p, fidx), params) in enumerate(zip(sizes, cams, plist)):
        fp = FramePlanes.allocate(W, H)
        v = _abi.View()
        v.camera, v.settings, v.params = camera, wl.settings(), params
        v.width, v.height, v.field_index = W, H, i % 3
        v.out = fp.abi()
        views.append(v)
        planes.append(fp)
    engine.render_views_plain(flds, views)
    a = snapshot(planes)
    for p in planes:
        for k in ("color", "mapping", "hit_id", "steps"):
            getattr(p, k).fill_(7)
    engine.render_batch(flds, views, _abi.BatchTuning(16, 64, 0, 8, 4, refill, schedule))
    engine.synchronize()
    for i, (x, y) in enumerate(zip(a, snapshot(planes))):
        for k in x:
            np.testing.assert_array_equal(x[k], y[k], err_msg=f"view {i} {sizes[i]} {k}")


@pytest.mark.parametrize("schedule,refill", BATCH_FORMS)
def test_batch_eight_fields_equals_plain(engine, schedule, refill):
    """The most fields one batch takes (LINON_MAX_BATCH_FIELDS = 8), one view
    per field plus two more: the per-CTA field choice of the tile schedules
    and the per-warp choice of the warp queues (one march loop per field in
    each) pick the right field.  Precise modules, bit-exact against
    one plain launch per view."""
    xyz, faces, rgb = scene.cornell_with_spheres(seed=2, subdivisions=1)
    engine.upload_scene(xyz, faces, rgb, bvh=True)
    # (no "identity": it returns v, which equals linear's v0 on straight rays)
    names = ["linear", "twist", "lens", "lorenz_scaled", "mirage_spherical", "rotation",
             "translation_x", "mirage_plane"]
    assert len(names) == _abi.LINON_MAX_BATCH_FIELDS
    flds = [field(engine, nme, True) for nme in names]
    views, planes = [], []
    specs = wl.batch_views(10, seed=11, min_side=20, max_side=70, n_fields=8)
    for i, (W, H, camera, params, fidx) in enumerate(specs):
        params.max_steps = min(params.max_steps, 120)
        fp = FramePlanes.allocate(W, H)
        v = _abi.View()
        v.camera, v.settings, v.params = camera, wl.settings(), params
        v.width, v.height = W, H
        v.field_index = i if i < 8 else fidx  # every field at least once
        v.out = fp.abi()
        views.append(v)
        planes.append(fp)
    engine.render_views_plain(flds, views)
    a = snapshot(planes)
    for p in planes:
        for k in ("color", "mapping", "hit_id", "steps"):
            getattr(p, k).zero_()
    engine.render_batch(flds, views, _abi.BatchTuning(16, 64, 0, 8, 4, refill, schedule))
    engine.synchronize()
    for x, y in zip(a, snapshot(planes)):
        for k in x:
            np.testing.assert_array_equal(x[k], y[k])


def test_batch_alone_equals_in_mix(engine):
    flds, views, planes = batch_setup(engine, True, n=5)
    engine.render_batch(flds, views[:1])
    alone = snapshot(planes[:1])[0]
    for p in planes:
        p.hit_id.fill_(-7)
    engine.render_batch(flds, views)
    engine.synchronize()
    mixed = snapshot(planes[:1])[0]
    for k in alone:
        np.testing.assert_array_equal(alone[k], mixed[k])


def test_batch_graph_replay_and_tuning(engine):
    flds, views, planes = batch_setup(engine, False, n=4)
    engine.render_batch(flds, views)
    first = snapshot(planes)
    engine.render_batch(flds, views)  # replays the captured graph
    second = snapshot(planes)
    for x, y in zip(first, second):
        for k in x:
            np.testing.assert_array_equal(x[k], y[k])
    t, ms = engine.autotune_batch(flds, views)
    assert ms > 0 and (t.schedule in (2, 3) or (t.schedule == 1 and t.quantum in (256, 1024, 4096)
                                                and t.refill_below in (0, 8)))
    # the tuned launch gives the default one's planes (fast modules: the two
    # batched kernels may contract FMAs differently, so to FP32 tolerance)
    engine.render_batch(flds, views, t)
    for x, y in zip(first, snapshot(planes)):
        assert np.mean(x["hit_id"] != y["hit_id"]) <= 0.005
        same = (x["hit_id"] == y["hit_id"]) & (x["steps"] == y["steps"])
        assert same.mean() >= 0.99
        d = np.abs(x["mapping"] - y["mapping"]).max(axis=-1)
        assert np.percentile(d[same], 99) <= 1e-4


def test_bounded_device_wait_reports_timeout(engine):
    """Failure path of the bounded mbarrier wait: one CTA waits on a barrier
    nothing completes; the wait runs out after its poll budget, the kernel
    flags it and returns, the host reads LINON_ETIMEOUT, and the context
    renders normally afterwards (the error word is cleared)."""
    import time
    t0 = time.perf_counter()
    assert engine.check_bounded_wait(2000) == _abi.LINON_ETIMEOUT
    assert time.perf_counter() - t0 < 10.0
    assert "flags 1" in engine.lib.linon_last_error().decode()
    assert engine.lib.linon_synchronize(engine.ctx) == _abi.LINON_OK
    with pytest.raises(_abi.LinonError):
        _abi.check(engine.check_bounded_wait(0))  # polls out of range
    w = wl.plain_small(32, 24)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fld = field(engine, "twist", True)
    planes = FramePlanes.allocate(w.width, w.height)
    engine.render(fld, w.camera, w.settings, wl.fixed_steps(0.05, 20), planes)
    engine.synchronize()
    assert int(planes.steps.sum().item()) == 20 * 32 * 24


def test_row_shards_equal_whole_frame(engine):
    """One frame split by rows (sharding.shard_rows, halo 2 * delta): each
    band rendered with linon_render_rows and overlaid alone gives the whole
    frame's planes, overlay and exponents on its owned rows, bit for bit
    (the bands run one after another on this GPU, each one rank's work)."""
    from linon_gb300 import sharding
    w = wl.lyapunov_1024(96, 80)
    params = wl.fixed_steps(0.01, 100, kahan=True)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fld = field(engine, "lorenz_scaled", False)
    delta = 2
    st = wl.settings(overlay_mode=1, delta=delta, scaling=20.0)
    full = FramePlanes.allocate(w.width, w.height)
    engine.render(fld, w.camera, st, params, full)
    t_full = torch.empty_like(full.color)
    e_full = torch.zeros((w.height, w.width), dtype=torch.float32, device="cuda")
    engine.overlay(st, w.width, w.height, full.color, full.mapping, t_full, e_full, fp64=True)
    engine.synchronize()
    ref = {k: getattr(full, k).cpu().numpy() for k in ("color", "mapping", "hit_id", "steps")}
    t_ref, e_ref = t_full.cpu().numpy(), e_full.cpu().numpy()
    for world in (2, 3):
        for band in sharding.shard_rows(w.height, world, 2 * delta):
            # each band with buffers of its own, as on its own rank (a band's
            # overlay also writes its halo rows, with border values)
            planes = FramePlanes.allocate(w.width, w.height)
            tgt = torch.zeros_like(full.color)
            ex = torch.zeros_like(e_full)
            o0, o1 = sharding.overlay_band(engine, fld, w.camera, st, params, planes, tgt, ex, band)
            engine.synchronize()
            for k in ref:
                np.testing.assert_array_equal(getattr(planes, k)[o0:o1].cpu().numpy(), ref[k][o0:o1])
            np.testing.assert_array_equal(tgt[o0:o1].cpu().numpy(), t_ref[o0:o1])
            np.testing.assert_array_equal(ex[o0:o1].cpu().numpy(), e_ref[o0:o1])
    with pytest.raises(_abi.LinonError):
        engine.render_rows(fld, w.camera, st, params, full, 10, 5)
    engine.render_rows(fld, w.camera, st, params, full, 7, 7)  # empty range: nothing to do


def test_private_state_is_per_ray(engine):
    """var<private> lives for one ray: a field that counts its calls and
    turns back after 40 of them (10 RK4 steps) brings every ray of a
    20-step march back to the eye, in the per-frame kernel and in a batch
    next to a stateless field (one CTA per tile, the queue of warp tiles,
    a lane-refilling request, which then takes the queue of warp tiles, and
    the queue of CTA tiles)."""
    helpers = "var<private> calls: u32 = 0u;"
    body = "calls += 1u;\nif (calls > 40u) { return -v0; }\nreturn v0;"
    w = wl.plain_small(40, 30)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    params = wl.fixed_steps(0.05, 20, kahan=True)
    fld = engine.compile_field(body, helpers)
    planes = FramePlanes.allocate(w.width, w.height)
    engine.render(fld, w.camera, w.settings, params, planes)
    engine.synchronize()
    eye = np.array(list(w.camera.origin)[:3], np.float32)
    ends = planes.mapping.cpu().numpy()[..., :3]
    assert np.abs(ends - eye).max() < 1e-4
    # batched next to a stateless field: per-view plain launches = batch
    flds = [fld, field(engine, "linear", False)]
    views, outs = [], []
    for k in range(4):
        fp = FramePlanes.allocate(24 + 8 * k, 16 + 4 * k)
        v = _abi.View()
        v.camera, v.settings, v.params = w.camera, w.settings, params
        v.width, v.height, v.field_index = fp.width, fp.height, k % 2
        v.out = fp.abi()
        views.append(v)
        outs.append(fp)
    engine.render_views_plain(flds, views)
    a = snapshot(outs)
    for tuning in (None, _abi.BatchTuning(1024, 128, 0, 4, 8, 0, 1), _abi.BatchTuning(16, 128, 0, 4, 8, 8, 1),
                   _abi.BatchTuning(0, 0, 0, 0, 0, 0, 3)):
        for fp in outs:
            fp.mapping.zero_()
        engine.render_batch(flds, views, tuning)
        engine.synchronize()
        b = snapshot(outs)
        for k, (x, y) in enumerate(zip(a, b)):
            np.testing.assert_allclose(y["mapping"], x["mapping"], rtol=0, atol=1e-5)
            if k % 2 == 0:
                assert np.abs(y["mapping"][..., :3] - eye).max() < 1e-4


def test_hbm_budget_admission():
    from linon_gb300 import Engine
    e = Engine(0, hbm_budget=1 << 20)
    try:
        xyz, faces, rgb = scene.cornell_with_spheres(seed=0)
        with pytest.raises(_abi.LinonError) as err:
            e.upload_scene(xyz, faces, rgb)
        assert err.value.status == _abi.LINON_ENOMEM
        e.upload_scene(*scene.cornell_unit())
    finally:
        e.close()


def test_main_view_mirror(engine):
    from linon_gb300.main_view import MainView
    xyz, faces, _, center = scene.cornell_reference()
    mv = MainView(engine, xyz, faces, center, 64, 48)
    mv.render()
    mv.reload_shader(None, predefined_source(_abi.FIELD_IDS["rotation"]))
    with pytest.raises(_abi.LinonCompileError):
        mv.reload_shader(None, "return undefined;")
    mv.render_high_accuracy(mv.field_function)
    pos = mv.render_outline_rays(mv.field_function)
    torch.cuda.synchronize()
    assert pos.shape == (8, 2)
    assert mv.texture.shape == (48, 64, 4)


PAIR_BUILTIN_BODIES = [
    # lane-wise builtins of the pair runtime: sin, cos, abs, clamp, exp, sqrt,
    # inverseSqrt, min, max, floor, length, sigmoid, cross, translate, pow
    "let w = vec3<f32>(sin(p.x), abs(p.y) - 0.5, clamp(p.z, -0.3, 0.3));\n"
    "return normalize(v0 + 0.2 * w * exp(-dot(p, p)));",
    "let r = sqrt(dot(p, p) + 0.25);\n"
    "let s = max(min(inverseSqrt(r), 1.5), 0.2);\n"
    "return normalize(v - 0.03 * cross(p, v0) * s + 0.01 * floor(2.0 * p));",
    "let q = translate(p, 0.1, -0.2, 0.05);\n"
    "return normalize(v + 0.02 * q * sigmoid(length(q) - 1.0) / pow(dot(q, q) + 0.1, 1.5));",
    # vector forms on unevaluated products (2.0 * p) and vector sqrt/exp/sin/cos
    "return normalize(v + 0.02 * abs(2.0 * p) - 0.01 * max(2.0 * p, v0) + 0.01 * min(0.5 * p, v0)\n"
    "    + 0.01 * clamp(3.0 * p, vec3<f32>(-0.3), vec3<f32>(0.3)) + 0.005 * sqrt(abs(p)) * exp(-p)\n"
    "    + 0.005 * sin(2.0 * p) * cos(p));",
    # mix, distance, fract, sign, tan, log, exp2, atan2, reflect, smoothstep, step
    "let m = mix(v, v0, 0.25) + 0.01 * mix(p, v0, vec3<f32>(0.3, 0.2, 0.1));\n"
    "let s = 0.01 * (fract(3.0 * p) + 0.5 * sign(p)) + 0.002 * vec3<f32>(tan(0.3 * p.x), log(1.0 + dot(p, p)),\n"
    "    exp2(-abs(p.z)));\n"
    "let r = 0.01 * reflect(p, v0) + 0.01 * smoothstep(vec3<f32>(-1.0), vec3<f32>(1.0), p)\n"
    "    + 0.005 * step(vec3<f32>(0.1), p) + 0.001 * vec3<f32>(atan2(p.y, p.x + 2.0), distance(p, v0), 0.0);\n"
    "return normalize(m + s + r);",
]


@pytest.mark.parametrize("body", range(len(PAIR_BUILTIN_BODIES)))
def test_pair_kernel_user_fields_match_one_ray_kernel(engine, body, monkeypatch):
    """User fields built from the pair runtime's lane-wise builtins, two rays
    per thread against one ray per thread (fast modules): endpoints within
    FP32 rounding, hit ids equal but for rounding ties."""
    src = PAIR_BUILTIN_BODIES[body]
    w = wl.frames_1080p(161, 97)
    w.params = wl.fixed_steps(0.005, 600, kahan=True)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fld = engine.compile_field(src)
    assert "pair form: compiles" in validate_field(src)
    monkeypatch.setenv("LINON_RAY_PAIRS", "1")
    g2 = gpu_render(engine, w, fld)
    assert fld.pair_state() == 1
    monkeypatch.setenv("LINON_RAY_PAIRS", "0")
    g1 = gpu_render(engine, w, fld)
    monkeypatch.delenv("LINON_RAY_PAIRS")
    same = g2["hit_id"] == g1["hit_id"]
    assert same.mean() >= 0.995, same.mean()
    d = np.linalg.norm(g2["mapping"][..., :3].astype(np.float64) - g1["mapping"][..., :3], axis=-1)
    assert np.percentile(d, 99) <= 1e-4, np.percentile(d, 99)


@pytest.mark.parametrize("name", ["linear", "twist", "lens", "lorenz_scaled", "lorenz", "roessler", "translation_x"])
def test_pair_kernel_matches_one_ray_kernel(engine, name, monkeypatch):
    """Two rays per thread (fixed step budget, fast module) against one ray
    per thread on the same frame: an odd width (the last pixel pair has one
    lane outside the image) and a band of rows (linon_render_rows).  The two
    kernels round every operation alike except where the one-ray kernel's
    compiler contracts a multiply-add differently from the pair kernel's
    explicit packed FMAs, so endpoints agree to FP32 rounding (smooth fields
    within 1e-4 at the 99.9th percentile; the chaotic lens orbits and the
    unscaled Lorenz field's fast, far-flung paths at the median) and hit ids
    and colours agree except on rounding ties."""
    w = wl.frames_1080p(241, 135)
    w.params = wl.fixed_steps(0.005, 800, kahan=True)
    engine.upload_scene(w.xyz, w.faces, w.face_rgb, bvh=True)
    fld = engine.compile_field(predefined_source(_abi.FIELD_IDS[name]))
    monkeypatch.setenv("LINON_RAY_PAIRS", "1")
    g2 = gpu_render(engine, w, fld)
    assert fld.pair_state() == 1
    monkeypatch.setenv("LINON_RAY_PAIRS", "0")
    g1 = gpu_render(engine, w, fld)
    monkeypatch.setenv("LINON_RAY_PAIRS", "1")
    assert (g2["steps"] == 800).all() and (g1["steps"] == 800).all()
    same = g2["hit_id"] == g1["hit_id"]
    assert same.mean() >= 0.995, same.mean()
    d = np.linalg.norm(g2["mapping"][..., :3].astype(np.float64) - g1["mapping"][..., :3], axis=-1)
    if name in ("lens", "lorenz"):
        assert np.median(d) <= 1e-4, np.median(d)
    else:
        assert np.percentile(d, 99.9) <= 1e-4, np.percentile(d, 99.9)
    dc = np.abs(g2["color"].astype(int) - g1["color"].astype(int))[same].max()
    assert dc <= 1, dc
    assert (g2["color"][..., 3] == 255).all()
    # a band of rows gives the whole frame's rows bit for bit
    band = FramePlanes.allocate(w.width, w.height)
    engine.render_rows(fld, w.camera, w.settings, w.params, band, 37, 101)
    torch.cuda.synchronize()
    engine.synchronize()
    monkeypatch.delenv("LINON_RAY_PAIRS")
    for k in ("color", "mapping", "hit_id", "steps"):
        np.testing.assert_array_equal(getattr(band, k).cpu().numpy()[37:101], g2[k][37:101], err_msg=k)
