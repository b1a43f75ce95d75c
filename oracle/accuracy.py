"""Accuracy of engine results against the FP64 oracle, per workload.

TEST INFRASTRUCTURE ONLY: used by tests/ and by bench.py's accuracy leg
(outside every timed region) as the checker; never as the thing measured or
shipped.  The engine's planes are sampled on seeded pixel sets; the oracle
(oracle/linon_oracle.hpp through pyoracle) renders the same pixels in FP64
and in FP32, so every figure comes with the FP32 restatement's own error
beside it.

Per frame (the outputs of main_view.wgsl:373-374 -- colour, endpoint
"mapping" -- plus the first-hit face of ray_color, main_view.wgsl:182-198):
  * endpoint error: Euclidean distance |p_engine - p_fp64| in scene units;
  * hit-id mismatch, split into ties that rounding decides: coplanar faces
    (the Cornell light panel in the ceiling, block footprints in the floor)
    and faces sharing a vertex (a path grazing the edge between two facets);
    everything else is "other";
  * RGBA8 difference in 1/255 steps on the pixels whose hit ids agree;
  * equal accuracy: where the path is chaotic (the point-lens field) FP32
    and FP64 trajectories separate whatever the implementation, so the
    engine's error quantiles are compared with the FP32 oracle's own.
Lyapunov (overlay.wgsl:99-135 and the finite-time exponent): exponents at
sampled pixels from FP64 endpoints of the pixel and its four neighbours,
against the engine's FP64-differenced maps.
"""
from __future__ import annotations

import numpy as np

from . import pyoracle

QUANTILES = (50, 90, 99)


def sample_pixels(width, height, n, seed, border=0):
    """n distinct pixel indices row*W+x (sorted), at least `border` pixels
    from every image edge."""
    rng = np.random.default_rng(seed)
    w, h = width - 2 * border, height - 2 * border
    n = min(n, w * h)
    k = rng.choice(w * h, size=n, replace=False)
    x, y = k % w + border, k // w + border
    return np.sort((y * width + x).astype(np.int32))


def stats(err):
    err = np.asarray(err, np.float64)
    if err.size == 0:
        return {"n": 0}
    out = {"n": int(err.size), "max": float(err.max())}
    for q in QUANTILES:
        out[f"p{q}"] = float(np.percentile(err, q))
    return out


class FaceInfo:
    """Per-face data for classifying hit-id mismatches."""

    def __init__(self, xyz, faces):
        from linon_gb300 import scene  # coplanar grouping of the scene module
        self.groups = scene.coplanar_groups(xyz, faces)
        v = np.asarray(xyz, np.float32)[np.asarray(faces, np.int64)]  # [nf, 3, 3]
        self.keys = [frozenset(map(tuple, f.tolist())) for f in v]

    def classify(self, a, b):
        """Counts of (coplanar, shared_vertex, other) over mismatching pairs."""
        cop = edge = other = 0
        for fa, fb in zip(np.asarray(a).tolist(), np.asarray(b).tolist()):
            if fa >= 0 and fb >= 0 and self.groups[fa] == self.groups[fb]:
                cop += 1
            elif fa >= 0 and fb >= 0 and self.keys[fa] & self.keys[fb]:
                edge += 1
            else:
                other += 1
        return cop, edge, other


def hit_mismatch(h_test, h_ref, info: FaceInfo):
    h_test, h_ref = np.asarray(h_test), np.asarray(h_ref)
    diff = h_test != h_ref
    n = max(1, h_test.size)
    cop, edge, other = info.classify(h_test[diff], h_ref[diff])
    return {"total": float(diff.sum() / n), "coplanar_tie": cop / n, "edge_graze": edge / n, "other": other / n}


def rgba8_diff(c_test, c_ref, same):
    d = np.abs(np.asarray(c_test, np.int32)[:, :3] - np.asarray(c_ref, np.int32)[:, :3]).max(axis=1)[same]
    if d.size == 0:
        return {"max_lsb": 0, "frac_gt_1_lsb": 0.0}
    return {"max_lsb": int(d.max()), "frac_gt_1_lsb": float(np.mean(d > 1))}


def endpoint_err(m_test, m64):
    return np.linalg.norm(np.asarray(m_test, np.float64)[:, :3] - np.asarray(m64, np.float64)[:, :3], axis=1)


ENDPOINT_TOL = 1e-4  # scene units: the endpoint tolerance against FP64
FTLE_TOL = 1e-4      # finite-time exponent, absolute (1/T units)


def equal_accuracy(err_engine, err_fp32, slack=1.25, floor=ENDPOINT_TOL):
    """The engine's error distribution against the FP32 oracle's on the same
    pixels: every reported quantile of the engine's error is within the
    tolerance `floor`, or at most `slack` times the FP32 oracle's (where FP32
    itself cannot meet the tolerance, e.g. on chaotic paths)."""
    ratios = {}
    ok = True
    for q in QUANTILES:
        a = float(np.percentile(err_engine, q))
        b = float(np.percentile(err_fp32, q))
        ratios[f"p{q}"] = a / b if b > 0 else (0.0 if a == 0 else float("inf"))
        ok = ok and (a <= slack * b or a <= floor)
    return {"ok": bool(ok), "slack": slack, "ratio_engine_over_fp32": ratios}


def oracle_pixels(w, field_id, width, height, camera, params, pix, accel=False, settings=None):
    """FP64 and FP32 oracle results at pixels `pix`."""
    st = settings or w.settings
    o64 = pyoracle.render(w.xyz, w.faces, w.face_rgb, camera, st, params, field_id, width, height, pixels=pix,
                          precision=64, want=("color", "mapping64", "hit_id", "steps"), accel=accel)
    o32 = pyoracle.render(w.xyz, w.faces, w.face_rgb, camera, st, params, field_id, width, height, pixels=pix,
                          precision=32, want=("color", "mapping", "hit_id", "steps"), accel=accel)
    return o64, o32


def frame_report(engine_px, o64, o32, info: FaceInfo):
    """engine_px: dict of the engine's planes at the sampled pixels
    (mapping [n,4] float32, hit_id [n], color [n,4] uint8, steps [n])."""
    e_eng = endpoint_err(engine_px["mapping"], o64["mapping64"])
    e_32 = endpoint_err(o32["mapping"], o64["mapping64"])
    same = np.asarray(engine_px["hit_id"]) == o64["hit_id"]
    rep = {"pixels": int(len(e_eng)),
           "endpoint_err": stats(e_eng), "endpoint_err_fp32_oracle": stats(e_32),
           "hit_mismatch": hit_mismatch(engine_px["hit_id"], o64["hit_id"], info),
           "hit_mismatch_fp32_oracle": hit_mismatch(o32["hit_id"], o64["hit_id"], info),
           "rgba8_vs_fp64": rgba8_diff(engine_px["color"], o64["color"], same),
           "rgba8_fp32_oracle_vs_fp64": rgba8_diff(o32["color"], o64["color"], o32["hit_id"] == o64["hit_id"]),
           "equal_accuracy": equal_accuracy(e_eng, e_32)}
    if "steps" in engine_px:
        rep["steps_equal_fp64"] = float(np.mean(np.asarray(engine_px["steps"]) == o64["steps"]))
    rep["_err"] = e_eng
    rep["_err32"] = e_32
    return rep


def public(rep):
    """The report without its raw arrays (for JSON)."""
    if isinstance(rep, dict):
        return {k: public(v) for k, v in rep.items() if not k.startswith("_")}
    if isinstance(rep, list):
        return [public(v) for v in rep]
    return rep


# ---------------------------------------------------------------------------
# Lyapunov: overlay exponent (overlay.wgsl:99-135, delta = 1) and finite-time
# exponent ln(max_nb |e(nb) - e(c)| / |d0(nb) - d0(c)|) / T from FP64 data
# ---------------------------------------------------------------------------
_NB = ((1, 0), (-1, 0), (0, 1), (0, -1))  # x+1, x-1, row+1, row-1


def stencil_pixels(width, centres, height=None):
    """The centres and their four neighbours as one sorted pixel list, and
    per direction the neighbour pixel (-1 outside the image when `height` is
    given; interior centres otherwise)."""
    c = np.asarray(centres, np.int64)
    x, y = c % width, c // width
    nb = []
    for dx, dy in _NB:
        n = c + dx + dy * width
        if height is not None:
            ok = (x + dx >= 0) & (x + dx < width) & (y + dy >= 0) & (y + dy < height)
            n = np.where(ok, n, -1)
        nb.append(n)
    allp = np.unique(np.concatenate([c] + [n[n >= 0] for n in nb])).astype(np.int32)
    return allp, nb


def overlay_scaled(m, c, nb_idx, scaling=50.0):
    """Scaled exponent exp(scaling * lambda - 5) in FP64 from endpoint map
    rows m[...] (lookup by position in the stencil pixel list)."""
    xn, xp, yn, yp = (m[i] for i in nb_idx)
    g0 = 0.5 * (xn - xp)
    g1 = 0.5 * (yn - yp)
    m00 = np.einsum("ij,ij->i", g0, g0)
    m01 = np.einsum("ij,ij->i", g0, g1)
    m11 = np.einsum("ij,ij->i", g1, g1)
    a0 = m00 * m11 - m01 * m01
    a1 = -(m00 + m11)
    disc = a1 * a1 - 4.0 * a0
    root = np.sqrt(np.abs(disc))
    e_hi = np.where(disc >= 0, np.maximum((-a1 - root) / 2.0, (-a1 + root) / 2.0),
                    np.maximum(-a1 / 2.0, root / 2.0))
    lam = np.sqrt(e_hi)
    with np.errstate(over="ignore"):
        return np.exp(scaling * lam - 5.0)


def ftle(m, d, c_idx, nb_idx, T):
    """ln(max over the neighbours inside the image of |e(nb) - e(c)| /
    |d0(nb) - d0(c)|) / T; nb_idx entries < 0 are outside the image."""
    best = np.full(len(c_idx), -1.0)
    for i in nb_idx:
        ok = i >= 0
        j = np.where(ok, i, c_idx)
        de = np.linalg.norm(m[j] - m[c_idx], axis=1)
        dd = np.linalg.norm(d[j] - d[c_idx], axis=1)
        with np.errstate(invalid="ignore", divide="ignore"):
            best = np.where(ok, np.maximum(best, de / dd), best)
    with np.errstate(divide="ignore"):
        return np.where(best > 0, np.log(np.where(best > 0, best, 1.0)) / T, -np.inf)


def lyapunov_report(w, field_id, centres, engine_ftle, engine_expo, engine_thr_full, outline_pixels, T,
                    quantile=0.95, scaling=50.0, engine_px=None, info=None):
    """engine_ftle / engine_expo: the engine's finite-time and scaled overlay
    exponents at `centres`; outline_pixels: the engine's 8 (x, y) outline
    pixels; engine_thr_full: its quantile threshold over the whole image."""
    W, H = w.width, w.height
    allp, nb = stencil_pixels(W, centres)
    pos = {int(p): i for i, p in enumerate(allp.tolist())}
    c_idx = np.array([pos[int(p)] for p in centres])
    nb_idx = [np.array([pos[int(p)] for p in n]) for n in nb]
    o64, o32 = oracle_pixels(w, field_id, W, H, w.camera, w.params, allp)
    m64 = o64["mapping64"][:, :3]
    m32 = o32["mapping"][:, :3].astype(np.float64)
    d64 = pyoracle.primary_dirs(w.camera, w.params, W, H, allp, precision=64)
    d32 = pyoracle.primary_dirs(w.camera, w.params, W, H, allp).astype(np.float64)
    f64 = ftle(m64, d64, c_idx, nb_idx, T)
    f32 = ftle(m32, d32, c_idx, nb_idx, T)
    s64 = overlay_scaled(m64, c_idx, nb_idx, scaling)
    eng_f = np.asarray(engine_ftle, np.float64)
    fin = np.isfinite(f64) & np.isfinite(eng_f)
    fin32 = fin & np.isfinite(f32)
    rep = {"centres": int(len(centres)), "rays": int(len(allp)),
           "ftle_abs_err": stats(np.abs(eng_f - f64)[fin]),
           "ftle_abs_err_fp32_oracle": stats(np.abs(f32 - f64)[fin32]),
           "ftle_equal_accuracy": equal_accuracy(np.abs(eng_f - f64)[fin32], np.abs(f32 - f64)[fin32],
                                                 floor=FTLE_TOL)}
    eng_s = np.asarray(engine_expo, np.float64)
    ok = np.isfinite(s64) & (s64 > 0)
    rep["overlay_exponent_rel_err"] = stats(np.abs(eng_s[ok] - s64[ok]) / s64[ok])
    rep["overlay_blend_decision_agree"] = float(np.mean((eng_s >= 0.8) == (s64 >= 0.8)))
    # quantile threshold on the same sample, and the classification it makes
    q_eng = float(np.quantile(eng_f[fin], quantile))
    q_64 = float(np.quantile(f64[fin], quantile))
    rep["p95_on_sample"] = {"engine": q_eng, "fp64": q_64, "abs_diff": abs(q_eng - q_64),
                            "engine_full_image": float(engine_thr_full)}
    rep["above_p95_agree"] = float(np.mean((eng_f[fin] > q_eng) == (f64[fin] > q_64)))
    # the engine's outline pixels under the FP64 exponent
    if outline_pixels is not None:
        op = np.unique(np.array([int(y) * W + int(x) for x, y in np.asarray(outline_pixels).tolist()], np.int32))
        if len(op):
            allo, nbo = stencil_pixels(W, op, H)
            poso = {int(p): i for i, p in enumerate(allo.tolist())}
            ci = np.array([poso[int(p)] for p in op])
            ni = [np.array([poso[int(p)] if p >= 0 else -1 for p in n]) for n in nbo]
            oo = pyoracle.render(w.xyz, w.faces, w.face_rgb, w.camera, w.settings, w.params, field_id, W, H,
                                 pixels=allo, precision=64, want=("mapping64",))
            fo = ftle(oo["mapping64"][:, :3], pyoracle.primary_dirs(w.camera, w.params, W, H, allo, precision=64),
                      ci, ni, T)
            rep["outline_pixels_above_engine_threshold_in_fp64"] = int(np.sum(fo >= engine_thr_full))
            rep["outline_pixels_checked"] = int(len(op))
    if engine_px is not None and info is not None:
        ci_pix = np.asarray(centres)
        sel = np.searchsorted(allp, ci_pix)
        o64c = {k: v[sel] for k, v in o64.items()}
        o32c = {k: v[sel] for k, v in o32.items()}
        rep["frame"] = frame_report(engine_px, o64c, o32c, info)
    return rep


def frame_pixels_report(w, field_id, engine_px, pix, info=None, accel=False):
    """One frame of workload `w` (its camera and march parameters)."""
    o64, o32 = oracle_pixels(w, field_id, w.width, w.height, w.camera, w.params, pix, accel=accel)
    return frame_report(engine_px, o64, o32, info or FaceInfo(w.xyz, w.faces))


def batch_report(w, views, engine_px_views, pix_views, field_names, info=None):
    """The uneven-view batch: each view's sampled pixels against the oracle
    (its camera, step, budget and field; the candidate grid over the large
    scene), pooled per field."""
    info = info or FaceInfo(w.xyz, w.faces)
    pooled = {}
    for (W, H, camera, params, fidx), eng, pix in zip(views, engine_px_views, pix_views):
        o64, o32 = oracle_pixels(w, w.fields[fidx], W, H, camera, params, pix, accel=True)
        d = pooled.setdefault(fidx, {"eng": [], "o64": [], "o32": [], "views": 0})
        d["eng"].append(eng)
        d["o64"].append(o64)
        d["o32"].append(o32)
        d["views"] += 1
    out = {}
    for fidx, d in sorted(pooled.items()):
        cat = lambda lst: {k: np.concatenate([x[k] for x in lst]) for k in lst[0]}
        rep = frame_report(cat(d["eng"]), cat(d["o64"]), cat(d["o32"]), info)
        rep["views"] = d["views"]
        out[field_names[fidx]] = rep
    return out
