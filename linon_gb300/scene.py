"""Scene inputs: the Cornell box, vertex normalisation, icospheres.

The Cornell box is the public Cornell Program of Computer Graphics
measurement set, in the vertex/face order of src/cornell_box.rs:1-163 (18
quads, two triangles each, so face indices match the reference's).  The
preparation of src/application.rs:105-123 (negate x and z, then one global
min/max normalisation, src/vertices.rs:3-17) and the bounding-box centre of
src/vertices.rs:19-57 are restated in float32 arithmetic.
"""
from __future__ import annotations

import numpy as np

# Quads as (name, 4 vertices); each becomes triangles (a,b,c), (c,d,a),
# the index pattern of src/cornell_box.rs:102-163.
CORNELL_QUADS = [
    ("floor", [(552.8, 0.0, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, 559.2), (549.6, 0.0, 559.2)]),
    ("floor", [(130.0, 0.0, 65.0), (82.0, 0.0, 225.0), (240.0, 0.0, 272.0), (290.0, 0.0, 114.0)]),
    ("floor", [(423.0, 0.0, 247.0), (265.0, 0.0, 296.0), (314.0, 0.0, 456.0), (472.0, 0.0, 406.0)]),
    ("ceiling", [(556.0, 548.8, 0.0), (556.0, 548.8, 559.2), (0.0, 548.8, 559.2), (0.0, 548.8, 0.0)]),
    ("light", [(343.0, 548.8, 227.0), (343.0, 548.8, 332.0), (213.0, 548.8, 332.0), (213.0, 548.8, 227.0)]),
    ("back", [(549.6, 0.0, 559.2), (0.0, 0.0, 559.2), (0.0, 548.8, 559.2), (556.0, 548.8, 559.2)]),
    ("green", [(0.0, 0.0, 559.2), (0.0, 0.0, 0.0), (0.0, 548.8, 0.0), (0.0, 548.8, 559.2)]),
    ("red", [(552.8, 0.0, 0.0), (549.6, 0.0, 559.2), (556.0, 548.8, 559.2), (556.0, 548.8, 0.0)]),
    ("short", [(130.0, 165.0, 65.0), (82.0, 165.0, 225.0), (240.0, 165.0, 272.0), (290.0, 165.0, 114.0)]),
    ("short", [(290.0, 0.0, 114.0), (290.0, 165.0, 114.0), (240.0, 165.0, 272.0), (240.0, 0.0, 272.0)]),
    ("short", [(130.0, 0.0, 65.0), (130.0, 165.0, 65.0), (290.0, 165.0, 114.0), (290.0, 0.0, 114.0)]),
    ("short", [(82.0, 0.0, 225.0), (82.0, 165.0, 225.0), (130.0, 165.0, 65.0), (130.0, 0.0, 65.0)]),
    ("short", [(240.0, 0.0, 272.0), (240.0, 165.0, 272.0), (82.0, 165.0, 225.0), (82.0, 0.0, 225.0)]),
    ("tall", [(423.0, 330.0, 247.0), (265.0, 330.0, 296.0), (314.0, 330.0, 456.0), (472.0, 330.0, 406.0)]),
    ("tall", [(423.0, 0.0, 247.0), (423.0, 330.0, 247.0), (472.0, 330.0, 406.0), (472.0, 0.0, 406.0)]),
    ("tall", [(472.0, 0.0, 406.0), (472.0, 330.0, 406.0), (314.0, 330.0, 456.0), (314.0, 0.0, 456.0)]),
    ("tall", [(314.0, 0.0, 456.0), (314.0, 330.0, 456.0), (265.0, 330.0, 296.0), (265.0, 0.0, 296.0)]),
    ("tall", [(265.0, 0.0, 296.0), (265.0, 330.0, 296.0), (423.0, 330.0, 247.0), (423.0, 0.0, 247.0)]),
]

# Diffuse reflectances of the published Cornell box (white / red / green).
_WHITE = (0.725, 0.71, 0.68)
_RGB = {"red": (0.63, 0.065, 0.05), "green": (0.14, 0.45, 0.091), "light": (1.0, 1.0, 1.0)}


def cornell_raw():
    """Raw Cornell box: (vertices float32 [72,3], faces uint32 [36,3], face_rgb float32 [36,3])."""
    verts, faces, rgb = [], [], []
    for q, (name, quad) in enumerate(CORNELL_QUADS):
        verts.extend(quad)
        b = 4 * q
        faces.append((b, b + 1, b + 2))
        faces.append((b + 2, b + 3, b))
        c = _RGB.get(name, _WHITE)
        rgb.extend([c, c])
    return (np.asarray(verts, dtype=np.float32), np.asarray(faces, dtype=np.uint32),
            np.asarray(rgb, dtype=np.float32))


def normalize_vertices(v: np.ndarray) -> np.ndarray:
    """src/vertices.rs:3-17: one global min/max over all coordinates, float32 ops."""
    v = np.asarray(v, dtype=np.float32)
    lo, hi = np.float32(v.min()), np.float32(v.max())
    out = (v - lo) / (hi - lo)
    return (out * np.float32(2.0) - np.float32(1.0)).astype(np.float32)


def normalize_per_axis(v: np.ndarray) -> np.ndarray:
    """Per-axis min/max normalisation to [-1,1]^3 (float32 ops)."""
    v = np.asarray(v, dtype=np.float32)
    lo, hi = v.min(axis=0), v.max(axis=0)
    out = (v - lo) / (hi - lo)
    return (out * np.float32(2.0) - np.float32(1.0)).astype(np.float32)


def get_center(v: np.ndarray) -> np.ndarray:
    """src/vertices.rs:19-57: centre of the axis-aligned bounding box (float32)."""
    v = np.asarray(v, dtype=np.float32).reshape(-1, 3)
    return ((v.min(axis=0) + v.max(axis=0)) / np.float32(2.0)).astype(np.float32)


def cornell_reference():
    """The scene the reference application builds (src/application.rs:105-123):
    x and z negated, then normalize_vertices.  Returns (xyz, faces, face_rgb, center)."""
    v, f, rgb = cornell_raw()
    v = v.copy()
    v[:, 0] = -v[:, 0]
    v[:, 2] = -v[:, 2]
    v = normalize_vertices(v)
    return v, f, rgb, get_center(v)


def cornell_unit():
    """The Cornell room of the benchmark workloads: x and z negated (open side
    facing +z), each axis normalised to [-1,1].  Returns (xyz, faces, face_rgb)."""
    v, f, rgb = cornell_raw()
    v = v.copy()
    v[:, 0] = -v[:, 0]
    v[:, 2] = -v[:, 2]
    return normalize_per_axis(v), f, rgb


def icosphere(subdivisions: int, radius: float = 1.0, center=(0.0, 0.0, 0.0)):
    """Icosphere by repeated 4-way subdivision of an icosahedron (vertices
    projected to the sphere).  20 * 4**subdivisions triangles."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
         (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    xyz = np.asarray(verts) * radius + np.asarray(center, dtype=np.float64)
    return xyz.astype(np.float32), np.asarray(faces, dtype=np.uint32)


def coplanar_groups(xyz, faces, tol: float = 1e-5) -> np.ndarray:
    """Group id per face; faces lying in one plane share an id.  Hits on
    coplanar, overlapping faces (the Cornell light panel in the ceiling, the
    block footprints in the floor) are decided by rounding ties, so accuracy
    checks count a hit-id difference inside one group as a tie."""
    v = np.asarray(xyz, np.float64)[np.asarray(faces, np.int64)]
    n = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    n = np.where(ln > 0, n / np.where(ln > 0, ln, 1), 0)
    # canonical orientation: first non-zero component positive
    sign = np.sign(n[np.arange(len(n)), np.argmax(np.abs(n) > tol, axis=1)])
    n = n * np.where(sign == 0, 1, sign)[:, None]
    d = np.einsum("ij,ij->i", n, v[:, 0])
    key = np.round(np.concatenate([n, d[:, None]], axis=1) / tol).astype(np.int64)
    _, ids = np.unique(key, axis=0, return_inverse=True)
    return ids.ravel()


def merge(*meshes):
    """Concatenates (xyz, faces[, rgb]) meshes; faces are re-indexed."""
    xs, fs, cs = [], [], []
    base = 0
    for m in meshes:
        x, f = m[0], m[1]
        rgb = m[2] if len(m) > 2 and m[2] is not None else np.full((len(f), 3), 0.8, np.float32)
        xs.append(x)
        fs.append(f.astype(np.int64) + base)
        cs.append(rgb)
        base += len(x)
    return (np.concatenate(xs).astype(np.float32), np.concatenate(fs).astype(np.uint32),
            np.concatenate(cs).astype(np.float32))


def cornell_with_spheres(seed: int = 0, n: int = 4, subdivisions: int = 5, radius: float = 0.3):
    """Cornell room plus n icospheres (20*4**subdivisions triangles each) with
    centres drawn uniformly inside the room's box shrunk by the radius."""
    rng = np.random.default_rng(seed)
    room = cornell_unit()
    lo, hi = room[0].min(axis=0) + radius, room[0].max(axis=0) - radius
    meshes = [room]
    for _ in range(n):
        c = rng.uniform(lo, hi)
        x, f = icosphere(subdivisions, radius, c)
        meshes.append((x, f, np.full((len(f), 3), (0.9, 0.9, 0.95), np.float32)))
    return merge(*meshes)


# ---- OBJ ingestion (src/main.rs:139-156, src/application.rs:199-226) ----

class ObjMesh:
    """One model of an OBJ file as the native loader returns it: positions
    (float32 [n,3]) in first-reference order, triangles (uint32 [m,3]), the
    number of models in the file and the bounding-box centre."""

    def __init__(self, xyz, faces, center, n_models):
        self.xyz, self.faces, self.center, self.n_models = xyz, faces, center, n_models


def _mesh_from_handle(lib, h) -> ObjMesh:
    import ctypes as C
    try:
        nv, nf, nm = C.c_uint32(), C.c_uint32(), C.c_uint32()
        c = (C.c_float * 3)()
        lib.linon_mesh_info(h, C.byref(nv), C.byref(nf), C.byref(nm), c)
        xyz = np.ctypeslib.as_array(lib.linon_mesh_positions(h), (nv.value * 3,)).copy() if nv.value else \
            np.zeros(0, np.float32)
        faces = np.ctypeslib.as_array(lib.linon_mesh_faces(h), (nf.value * 3,)).copy() if nf.value else \
            np.zeros(0, np.uint32)
        return ObjMesh(xyz.reshape(-1, 3), faces.reshape(-1, 3), np.array(c[:], np.float32), nm.value)
    finally:
        lib.linon_mesh_free(h)


def load_obj(path, model: int = 0, normalize: bool = True) -> ObjMesh:
    """The reference's dropped-file path: tobj's load_obj with triangulation,
    models[model].mesh, then (normalize=True) load_model's normalize_vertices
    and get_center.  Raises LinonError on unreadable or malformed files."""
    import ctypes as C
    from . import _abi
    lib = _abi.load()
    h = C.c_void_p()
    _abi.check(lib.linon_obj_load(str(path).encode(), model, _abi.LINON_OBJ_NORMALIZE if normalize else 0,
                                  C.byref(h)))
    return _mesh_from_handle(lib, h)


def parse_obj(text, model: int = 0, normalize: bool = True, mtl_dir=None) -> ObjMesh:
    """load_obj on OBJ text in memory ("mtllib" files are read from mtl_dir)."""
    import ctypes as C
    from . import _abi
    lib = _abi.load()
    data = text.encode() if isinstance(text, str) else bytes(text)
    h = C.c_void_p()
    _abi.check(lib.linon_obj_parse(data, len(data), None if mtl_dir is None else str(mtl_dir).encode(), model,
                                   _abi.LINON_OBJ_NORMALIZE if normalize else 0, C.byref(h)))
    return _mesh_from_handle(lib, h)


def normalize_vertices_native(xyz) -> tuple[np.ndarray, np.ndarray]:
    """normalize_vertices + get_center through the C ABI (float32, in place on a copy)."""
    import ctypes as C
    from . import _abi
    v = np.ascontiguousarray(xyz, dtype=np.float32).copy()
    c = (C.c_float * 3)()
    _abi.check(_abi.load().linon_normalize_vertices(v.ctypes.data, v.size, c if v.size >= 3 else None))
    return v, np.array(c[:], np.float32)


def to_obj(xyz, faces, polygons=None) -> str:
    """OBJ text of a triangle mesh ("v" and 1-based "f" records); extra
    polygons (lists of 0-based vertex indices) are appended as faces."""
    xyz = np.asarray(xyz, np.float32).reshape(-1, 3)
    lines = [f"v {float(a)!r} {float(b)!r} {float(c)!r}" for a, b, c in xyz.tolist()]
    lines += [f"f {a + 1} {b + 1} {c + 1}" for a, b, c in np.asarray(faces).reshape(-1, 3).tolist()]
    for poly in polygons or []:
        lines.append("f " + " ".join(str(i + 1) for i in poly))
    return "\n".join(lines) + "\n"


def torus(n_major: int = 48, n_minor: int = 24, R: float = 0.35, r: float = 0.12, center=(0.0, 0.0, 0.0),
          tilt: float = 0.6):
    """Torus as quads (for OBJ files with non-triangle faces): vertices
    float32 [n_major*n_minor, 3] and quads int [n_major*n_minor, 4], tilted
    about the x axis by `tilt` radians."""
    i, j = np.meshgrid(np.arange(n_major), np.arange(n_minor), indexing="ij")
    u, v = 2 * np.pi * i / n_major, 2 * np.pi * j / n_minor
    x = (R + r * np.cos(v)) * np.cos(u)
    y = (R + r * np.cos(v)) * np.sin(u)
    z = r * np.sin(v)
    ct, st = np.cos(tilt), np.sin(tilt)
    y, z = y * ct - z * st, y * st + z * ct
    xyz = np.stack([x, y, z], -1).reshape(-1, 3) + np.asarray(center)
    idx = lambda a, b: (a % n_major) * n_minor + (b % n_minor)
    quads = np.stack([idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)], -1).reshape(-1, 4)
    return xyz.astype(np.float32), quads
