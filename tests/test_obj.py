"""OBJ scene ingestion (CPU): the native loader against the restatement of
tobj's load_obj in oracle/obj_restatement.py, plus the reference's
normalize_vertices / get_center.

Bars: positions bit-identical (float32 bit patterns), triangles and model
counts identical, and the same inputs rejected.
"""
import numpy as np
import pytest

from linon_gb300 import _abi, scene
from oracle import obj_restatement as ref


def native(text, model=0, normalize=False, mtl_dir=None):
    return scene.parse_obj(text, model=model, normalize=normalize, mtl_dir=mtl_dir)


def same(text, model=0, mtl_dir=None):
    """Both loaders agree: identical output, or both reject."""
    try:
        want = ref.load(text, model, mtl_dir)
    except ref.ObjError:
        with pytest.raises(_abi.LinonError):
            native(text, model, mtl_dir=mtl_dir)
        return None
    got = native(text, model, mtl_dir=mtl_dir)
    xyz, tris, n_models = want
    np.testing.assert_array_equal(got.xyz.view(np.uint32), xyz.view(np.uint32))
    np.testing.assert_array_equal(got.faces, tris)
    assert got.n_models == n_models
    return got


QUADS = """# two quads and a pentagon
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 0.5 1.5 0
f 1 2 3 4
f 4 3 5
f 1 2 3 5 4
"""


def test_triangulation_fans():
    m = same(QUADS)
    np.testing.assert_array_equal(m.faces, [[0, 1, 2], [0, 2, 3], [3, 2, 4], [0, 1, 2], [0, 2, 4], [0, 4, 3]])


def test_first_reference_order_and_unreferenced_vertices():
    # vertex 3 is never referenced; the positions follow first reference
    m = same("v 0 0 0\nv 1 0 0\nv 9 9 9\nv 0 1 0\nf 4 1 2\n")
    np.testing.assert_array_equal(m.xyz, [[0, 1, 0], [0, 0, 0], [1, 0, 0]])
    np.testing.assert_array_equal(m.faces, [[0, 1, 2]])


def test_index_forms_and_relative_indices():
    text = ("v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvn 0 0 1\n"
            "f 1/1/1 2/2/1 3//1\nf -3 -2/-1 -1//-1\nf +1 +2 +3\n")
    m = same(text)
    np.testing.assert_array_equal(m.faces, [[0, 1, 2]] * 3)


def test_points_and_lines_become_zero_area_triangles():
    m = same("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1\nl 1 2\nf 2 3\n")
    np.testing.assert_array_equal(m.faces, [[0, 0, 0], [0, 1, 1], [1, 2, 2]])


def test_forward_reference_inside_a_model():
    # a face may name a position defined later in the same model
    same("f 1 2 3\nv 0 0 0\nv 1 0 0\nv 0 1 0\n")


@pytest.mark.parametrize("text", [
    "v 0 0\n",                                  # short vertex
    "v 0 0 zero\n",                             # bad number
    "v 0 0 0\nf 1 1 2\n",                       # position out of range
    "v 0 0 0\nf 0 1 1\n",                       # index 0 is "missing"
    "v 0 0 0\nf -2 1 1\n",                      # relative before the start
    "v 0 0 0\nf 1/1/1/1 1 1\n",                 # four parts
    "v 0 0 0\nf 1 1 1 # comment\n",             # '#' is not an index
    "v 0 0 0\nvt 0 0\nf 1/2 1 1\n",             # texcoord out of range
    "v 0 0 0\nvn 0 0 1\nf 1//3 1 1\n",          # normal out of range
    "v 0 0 0\nf\n",                             # face without vertices
    "v 0 0 0\nusemtl\n",                        # usemtl without a name
    "v 0 0 0\nf 1.0 1 1\n",                     # non-integer index
    "v 0 0 0\nf 99999999999999999999 1 1\n",    # index overflow
])
def test_rejected(text):
    assert same(text) is None


def test_absent_texcoords_and_normals_are_not_checked():
    # texture / normal references are only checked when that list exists
    m = same("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1/7 2/8 3/9/4\n")
    assert m.faces.shape == (1, 3)


@pytest.mark.parametrize("tok,ok", [
    ("1", True), ("-1.5", True), ("+2.25", True), (".5", True), ("5.", True), ("1e3", True), ("1.E-3", True),
    ("1e50", True), ("-1e50", True), ("1e-50", True), ("1e-40", True), ("3.4028235e38", True),
    ("3.40282357e38", True), ("3.4028236e38", True), ("inf", True), ("-Infinity", True), ("NaN", True),
    ("0.1", True), ("16777217", True), ("1.00000005960464477539062500", True),
    ("1e", False), (".", False), ("e5", False), ("0x10", False), ("1_0", False), ("--1", False),
    ("+-1", False), ("nan(1)", False), ("1.5f", False), ("infinit", False), ("", False),
])
def test_float_grammar_and_rounding(tok, ok):
    text = f"v {tok or '+'} 0 0\nf 1 1 1\n"
    m = same(text)
    assert (m is not None) == ok
    if ok:
        want = ref.f32_from_str(tok)
        assert m.xyz[0, 0].view(np.uint32) == want.view(np.uint32) or (np.isnan(want) and np.isnan(m.xyz[0, 0]))


def test_midpoint_rounds_to_even():
    # 1 + 2^-24 is exactly halfway between 1 and the next float: ties to even -> 1
    assert ref.f32_from_str("1.000000059604644775390625") == np.float32(1.0)
    m = native("v 1.000000059604644775390625 0 0\nf 1 1 1\n")
    assert m.xyz[0, 0] == np.float32(1.0)


def test_models_split_at_objects_and_groups():
    text = ("o first\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n"
            "g second\nv 0 0 1\nf 1 2 4\nf 2 3 4\n"
            "o empty\ng third\nf 4 3 2\n")
    for k in range(3):
        m = same(text, model=k)
        assert m.n_models == 3
    assert same(text, model=3) is None
    # names before any face do not start a model; a trailing empty model counts
    m = same("o a\no b\nv 0 0 0\nf 1 1 1\no c\n")
    assert m.n_models == 2


def test_usemtl_splits_only_on_known_material_changes(tmp_path):
    (tmp_path / "m.mtl").write_text("newmtl red\nKd 1 0 0\nnewmtl  blue \nKd 0 0 1\n")
    text = ("mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nv 0 0 1\n"
            "usemtl red\nf 1 2 3\nusemtl red\nf 1 2 4\n"      # same material: no split
            "usemtl blue\nf 2 3 4\n"                           # split
            "usemtl nowhere\nf 1 3 4\nusemtl also_missing\nf 1 2 3\n")  # unknown -> none, then none: no split
    for k in range(3):
        same(text, model=k, mtl_dir=tmp_path)
    assert native(text, mtl_dir=tmp_path).n_models == 3
    # without the material file every name is unknown: one model
    assert native(text).n_models == 1
    assert same(text) is not None
    # the file loader finds the .mtl next to the .obj
    p = tmp_path / "scene.obj"
    p.write_text(text)
    assert scene.load_obj(p, normalize=False).n_models == 3


def test_crlf_tabs_and_comments():
    text = "# header\r\nv\t0 0 0\r\nv 1 0 0 0.5 0.5 0.5\r\n\r\nv 0 1 0\r\n  f 1 2 3  \r\n#f 3 2 1\r\nfoo bar\r\n"
    m = same(text)
    np.testing.assert_array_equal(m.faces, [[0, 1, 2]])


def _fuzz_text(rng):
    lines = []
    n_v = n_vt = n_vn = 0
    for _ in range(int(rng.integers(20, 120))):
        r = rng.random()
        if r < 0.35:
            vals = rng.normal(0, 10, 3)
            fmt = rng.integers(0, 4)
            toks = [f"{x:.{int(rng.integers(1, 12))}g}" if fmt else repr(float(np.float32(x))) for x in vals]
            if fmt == 3:
                toks = [f"{x:.6e}" for x in vals]
            lines.append("v " + " ".join(toks))
            n_v += 1
        elif r < 0.42:
            lines.append(f"vt {rng.random():.4f} {rng.random():.4f}")
            n_vt += 1
        elif r < 0.48:
            lines.append(f"vn {rng.normal():.4f} {rng.normal():.4f} {rng.normal():.4f}")
            n_vn += 1
        elif r < 0.85 and n_v:
            k = int(rng.choice([1, 2, 3, 3, 3, 4, 4, 5, 7]))
            refs = []
            for _ in range(k):
                v = int(rng.integers(1, n_v + 1))
                if rng.random() < 0.01:
                    v = n_v + 1                           # occasionally one past the end
                if rng.random() < 0.3:
                    v = v - n_v - 1                       # relative form
                form = rng.integers(0, 4)
                vt = int(rng.integers(1, n_vt + 1)) if n_vt else 1
                vn = int(rng.integers(1, n_vn + 1)) if n_vn else 1
                refs.append([f"{v}", f"{v}/{vt}", f"{v}//{vn}", f"{v}/{vt}/{vn}"][form])
            lines.append(("l " if k == 2 and rng.random() < 0.5 else "f ") + " ".join(refs))
        elif r < 0.9:
            lines.append(f"{rng.choice(['o', 'g'])} part{int(rng.integers(0, 5))}")
        elif r < 0.94:
            lines.append(f"usemtl mat{int(rng.integers(0, 3))}")
        elif r < 0.97:
            lines.append("# comment")
        else:
            lines.append("s off")
    return "\n".join(lines) + "\n"


def test_fuzz_against_restatement(tmp_path):
    (tmp_path / "lib.mtl").write_text("newmtl mat0\nnewmtl mat1\n")
    rng = np.random.default_rng(1234)
    accepted = 0
    for _ in range(300):
        text = _fuzz_text(rng)
        if rng.random() < 0.5:
            text = "mtllib lib.mtl\n" + text
        n_models = None
        try:
            n_models = ref.load(text, 0, tmp_path)[2]
        except ref.ObjError:
            pass
        for k in range(min(n_models or 1, 3)):
            if same(text, model=k, mtl_dir=tmp_path) is not None:
                accepted += 1
    assert accepted > 100  # the fuzz exercises the accepting path, not only errors


def test_normalize_matches_reference_and_restatement():
    rng = np.random.default_rng(5)
    v = rng.normal(0, 50, (500, 3)).astype(np.float32)
    got, c = scene.normalize_vertices_native(v)
    want = ref.normalize_vertices(v)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    np.testing.assert_array_equal(c.view(np.uint32), ref.get_center(want).view(np.uint32))
    # the package's numpy mirror agrees too
    np.testing.assert_array_equal(scene.normalize_vertices(v).view(np.uint32), want.view(np.uint32))


def test_normalize_nan_and_flat():
    v = np.array([[np.nan, 1, 2], [3, 4, 5]], np.float32)
    got, c = scene.normalize_vertices_native(v)
    want = ref.normalize_vertices(v)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.isnan(c[0]) and np.isnan(ref.get_center(want)[0])
    flat, _ = scene.normalize_vertices_native(np.ones((2, 3), np.float32))
    assert not np.isfinite(flat).any()  # (x-min)/(max-min) with max == min


def test_load_obj_normalizes_like_load_model(tmp_path):
    """The Cornell box written as an OBJ and dropped: the loaded scene is the
    reference's normalize_vertices + get_center of the raw coordinates."""
    v, f, _ = scene.cornell_raw()
    p = tmp_path / "cornell.obj"
    p.write_text(scene.to_obj(v, f))
    m = scene.load_obj(p)
    want = ref.normalize_vertices(v)
    np.testing.assert_array_equal(m.xyz.view(np.uint32), want.view(np.uint32))
    np.testing.assert_array_equal(m.faces, f)
    np.testing.assert_array_equal(m.center.view(np.uint32), ref.get_center(want).view(np.uint32))


def test_unreadable_file(tmp_path):
    with pytest.raises(_abi.LinonError) as e:
        scene.load_obj(tmp_path / "missing.obj")
    assert e.value.status == _abi.LINON_EIO


def test_large_mesh_parses(tmp_path):
    import time
    xyz, faces = scene.icosphere(6)  # 40,962 vertices, 81,920 triangles
    text = scene.to_obj(xyz, faces)
    t0 = time.perf_counter()
    m = native(text)
    dt = time.perf_counter() - t0
    assert m.faces.shape == (81920, 3) and len(m.xyz) == len(xyz)
    # positions are renumbered in first-reference order; the triangles' corners are the same
    tri = np.asarray(xyz, np.float32)[np.asarray(faces)]
    np.testing.assert_array_equal(m.xyz[m.faces].view(np.uint32), tri.view(np.uint32))
    assert dt < 5.0, dt
