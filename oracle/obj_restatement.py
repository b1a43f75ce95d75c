"""Restatement of the reference's OBJ scene ingestion — TEST INFRASTRUCTURE.

This module is the oracle for the native OBJ loader (linon_obj_load /
linon_obj_parse).  Only tests import it; nothing in the product calls it.

The reference's path (src/main.rs:139-156): a dropped ``.obj`` file goes
through ``tobj::load_obj(path, &LoadOptions { triangulate: true,
..Default::default() })``; ``models[0].mesh.positions`` / ``.indices`` go
to ``Application::load_model`` (src/application.rs:199-226), which calls
``normalize_vertices`` (src/vertices.rs:3-17) and ``get_center``
(src/vertices.rs:19-57).

tobj 4.0.2 (Cargo.lock:2898-2900) is a third-party crate that the reference
does not vendor; what follows restates its published behaviour for those
load options (``load_obj_buf``, ``parse_floatn``, ``parse_face``,
``VertexIndices::parse``, the multi-index export used when ``single_index``
is false, and the triangulation of points, lines, quads and polygons):

* one record per line, words split on whitespace, first word = keyword;
* ``v``: three floats required (Rust ``f32::from_str``: correctly rounded,
  ``[+-]`` then ``inf|infinity|nan`` or a decimal with optional exponent);
* ``vt``: two floats; ``vn``: three floats;
* ``f`` / ``l``: vertex references ``v[/vt[/vn]]`` (empty parts allowed),
  ``isize`` indices, ``n > 0 -> n-1``, ``n < 0 -> count + n``; -1 is the
  "missing" marker;
* ``o`` / ``g``: the current model ends if it has faces;
* ``usemtl``: the current model ends if it has faces and the material id
  changes (ids from the ``newmtl`` names of ``mtllib`` files);
* the model left at the end is always emitted;
* export: positions keyed by position index in first-reference order; point
  -> (a,a,a), line -> (a,b,b), quad -> (a,b,c)(a,c,d), n-gon -> fan;
  position references must exist; texture/normal references must exist
  when their list is not empty.

Parity status against tobj itself: unpinned (the crate is not present and
the reference ships no OBJ fixtures); tests pin the native loader to this
restatement on generated files.
"""
from __future__ import annotations

import re
from fractions import Fraction
from pathlib import Path

import numpy as np

_FLOAT_RE = re.compile(r"[+-]?(?:inf|infinity|nan|(?:[0-9]+(?:\.[0-9]*)?|\.[0-9]+)(?:[eE][+-]?[0-9]+)?)\Z",
                       re.IGNORECASE)
_INT_RE = re.compile(r"[+-]?[0-9]+\Z")
_F32_MAX = Fraction(float(np.finfo(np.float32).max))
_OVERFLOW = _F32_MAX + Fraction(2) ** 103  # max + half an ulp: ties round to infinity (even)
_I64 = 2 ** 63


class ObjError(ValueError):
    pass


def f32_from_str(tok: str) -> np.float32:
    """Rust's f32::from_str: exact decimal value rounded once to f32 (ties to even)."""
    if not _FLOAT_RE.match(tok):
        raise ObjError(f"bad number {tok!r}")
    neg = tok[0] == "-"
    body = tok.lstrip("+-").lower()
    if body in ("inf", "infinity"):
        return np.float32(-np.inf if neg else np.inf)
    if body == "nan":
        return np.float32(np.nan)
    q = Fraction(body)
    if q == 0:
        return np.float32(-0.0 if neg else 0.0)
    if q >= _OVERFLOW:
        r = np.float32(np.inf)
    else:
        c = np.float32(min(float(q), float(_F32_MAX)))
        best = None
        with np.errstate(over="ignore"):
            cands = (np.nextafter(c, np.float32(-np.inf)), c, np.nextafter(c, np.float32(np.inf)))
        for cand in cands:
            if not np.isfinite(cand) or cand < 0:
                continue
            err = abs(Fraction(float(cand)) - q)
            even = int(np.array(cand, np.float32).view(np.uint32)) % 2 == 0
            key = (err, not even)
            if best is None or key < best[0]:
                best = (key, cand)
        r = best[1]
    return np.float32(-r if neg else r)


def _isize(tok: str) -> int:
    if not _INT_RE.match(tok):
        raise ObjError(f"bad index {tok!r}")
    x = int(tok)
    if not -_I64 <= x < _I64:
        raise ObjError(f"index overflow {tok!r}")
    return x


def _materials(text: str, mtl_dir) -> dict:
    ids: dict = {}
    if mtl_dir is None:
        return ids
    n = 0
    for line in text.split("\n"):
        words = line.split()
        if not words or words[0] != "mtllib":
            continue
        name = line.strip()[len("mtllib"):].strip()
        path = Path(name) if name.startswith("/") else Path(mtl_dir) / name
        try:
            body = path.read_text()
        except OSError:
            continue
        for ml in body.split("\n"):
            w = ml.split()
            if w and w[0] == "newmtl":
                nm = ml.strip()[len("newmtl"):].strip()
                if nm:
                    ids[nm] = n
                    n += 1
    return ids


def load(text: str, model: int = 0, mtl_dir=None):
    """Returns (positions float32 [n,3], triangles uint32 [m,3], n_models).
    Raises ObjError where the native loader must fail."""
    mats = _materials(text, mtl_dir)
    pos: list = []
    n_vt = n_vn = 0
    faces: list = []          # list of lists of (v, vt, vn)
    models: list = []         # (faces, n_pos, n_vt, n_vn) snapshots at close
    material = None

    def close():
        models.append(_export(faces[:], pos, n_vt, n_vn))
        faces.clear()

    for raw in text.split("\n"):
        w = raw.split()
        if not w or w[0] == "#":
            continue
        key = w[0]
        if key in ("v", "vt", "vn"):
            need = 2 if key == "vt" else 3
            if len(w) < need + 1:
                raise ObjError(f"short {key}")
            vals = [f32_from_str(t) for t in w[1:need + 1]]
            if key == "v":
                pos.extend(vals)
            elif key == "vt":
                n_vt += 1
            else:
                n_vn += 1
        elif key in ("f", "l"):
            refs = []
            for t in w[1:]:
                parts = t.split("/")
                if len(parts) > 3:
                    raise ObjError("too many parts")
                sizes = (len(pos) // 3, n_vt, n_vn)
                r = [-1, -1, -1]
                for i, s in enumerate(parts):
                    if s:
                        x = _isize(s)
                        r[i] = sizes[i] + x if x < 0 else x - 1
                refs.append(tuple(r))
            if not refs:
                raise ObjError("empty face")
            faces.append(refs)
        elif key in ("o", "g"):
            if faces:
                close()
        elif key == "usemtl":
            name = raw.strip()[len("usemtl"):].strip()
            if not name:
                raise ObjError("usemtl without name")
            new = mats.get(name)
            if new != material and faces:
                close()
            material = new
    close()
    if model >= len(models):
        raise ObjError("no such model")
    out = [m for m in models]
    for m in out:
        if isinstance(m, ObjError):
            raise m
    p, t = out[model]
    return p, t, len(models)


def _export(faces, pos, n_vt, n_vn):
    n_pos = len(pos) // 3
    for f in faces:
        for v, vt, vn in f:
            if not 0 <= v < n_pos:
                return ObjError("position out of range")
            if n_vt and vt != -1 and not 0 <= vt < n_vt:
                return ObjError("texcoord out of range")
            if n_vn and vn != -1 and not 0 <= vn < n_vn:
                return ObjError("normal out of range")
    local: dict = {}
    xyz: list = []
    tris: list = []

    def idx(v):
        if v not in local:
            local[v] = len(local)
            xyz.extend(pos[3 * v:3 * v + 3])
        return local[v]

    for f in faces:
        vs = [r[0] for r in f]
        if len(vs) == 1:
            corners = [(vs[0], vs[0], vs[0])]
        elif len(vs) == 2:
            corners = [(vs[0], vs[1], vs[1])]
        else:
            corners = [(vs[0], vs[j], vs[j + 1]) for j in range(1, len(vs) - 1)]
        for a, b, c in corners:
            tris.append((idx(a), idx(b), idx(c)))
    return (np.array(xyz, np.float32).reshape(-1, 3), np.array(tris, np.uint32).reshape(-1, 3))


def normalize_vertices(v) -> np.ndarray:
    """src/vertices.rs:3-17 with its comparisons (NaN never replaces the
    running min/max, which start at f32::MAX / f32::MIN)."""
    flat = np.asarray(v, np.float32).ravel().copy()
    lo, hi = np.float32(np.finfo(np.float32).max), np.float32(np.finfo(np.float32).min)
    finite = flat[~np.isnan(flat)]
    if finite.size:
        lo, hi = min(lo, finite.min()), max(hi, finite.max())
    with np.errstate(all="ignore"):
        out = (flat - lo) / (hi - lo) * np.float32(2.0) - np.float32(1.0)
    return out.astype(np.float32).reshape(np.shape(v))


def get_center(v) -> np.ndarray:
    """src/vertices.rs:19-57: running min/max started at the first vertex."""
    a = np.asarray(v, np.float32).reshape(-1, 3)
    lo, hi = a[0].copy(), a[0].copy()
    for row in a[1:]:
        for k in range(3):
            if row[k] < lo[k]:
                lo[k] = row[k]
            if row[k] > hi[k]:
                hi[k] = row[k]
    with np.errstate(all="ignore"):
        return ((lo + hi) / np.float32(2.0)).astype(np.float32)
