"""Writes tests/golden/rays.npz from the numpy float32 restatement.

Run from the repository root:  python tests/golden/make_golden.py

Cases: the reference's own first frame setting (Cornell box prepared as the
application does, arcball default camera, t <= 5 loop with h = 0.1 and
adaptive refinement) and fixed-step cases on the benchmark room, over the
transcendental-free fields (identity, linear, Lorenz, Roessler, translation,
the two non-sigmoid mirages: their arithmetic is +,-,*,/,sqrt only, so the
C++ oracle must match these fixtures bit for bit).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))

import np_restatement as R  # noqa: E402
from linon_gb300 import scene  # noqa: E402

FIELDS = ["identity", "linear", "lorenz", "roessler", "translation_x", "mirage_spherical", "mirage_plane"]


def cases():
    ref_xyz, ref_faces, _, center = scene.cornell_reference()
    eye = (center + np.float32([0.0, 0.0, 2.0])).astype(np.float32)
    unit_xyz, unit_faces, unit_rgb = scene.cornell_unit()
    vh45 = float(np.float32(2.0 * np.tan(np.radians(22.5))))
    out = []
    for fname in FIELDS:
        out.append(dict(name=f"reference_{fname}", xyz=ref_xyz, faces=ref_faces, rgb=None, W=48, H=40,
                        origin=eye, vd=(0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0), focal=0.035, vh=0.025,
                        h=0.1, t_max=5.0, steps=0, adaptive=True, kahan=False, fw=1.0, field=fname))
        out.append(dict(name=f"steps_{fname}", xyz=unit_xyz, faces=unit_faces, rgb=unit_rgb, W=40, H=32,
                        origin=(0.0, 0.0, 3.0), vd=(0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0), focal=1.0, vh=vh45,
                        h=0.05, t_max=0.0, steps=80, adaptive=False, kahan=True, fw=0.75, field=fname))
    return out


def main():
    rng = np.random.default_rng(1234)
    data = {}
    for c in cases():
        sc = R.Scene(c["xyz"], c["faces"], c["rgb"])
        b = R.camera_basis(c["origin"], c["vd"], c["up"], c["W"], c["H"], c["focal"], c["vh"])
        pix = rng.choice(c["W"] * c["H"], size=12, replace=False).astype(np.int32)
        color = np.zeros((len(pix), 4), np.uint8)
        mapping = np.zeros((len(pix), 4), np.float32)
        hit = np.zeros(len(pix), np.int32)
        steps = np.zeros(len(pix), np.int32)
        for i, p in enumerate(pix):
            row, x = divmod(int(p), c["W"])
            d = R.primary_dir(b, x, c["H"] - 1 - row)
            col, face, endp, n = R.march(sc, c["field"], b["origin"], d, c["h"], c["t_max"], c["steps"],
                                         c["adaptive"], c["fw"], kahan=c["kahan"])
            if col is None:
                color[i] = (0, 0, 0, 255)
            else:
                color[i] = (R.unorm8(col[0]), R.unorm8(col[1]), R.unorm8(col[2]), 255)
            mapping[i] = (endp[0], endp[1], endp[2], 1.0)
            hit[i] = face
            steps[i] = n
        k = c["name"]
        data[f"{k}/pixels"] = pix
        data[f"{k}/color"] = color
        data[f"{k}/mapping"] = mapping
        data[f"{k}/hit_id"] = hit
        data[f"{k}/steps"] = steps
        print(k, "steps", steps.min(), steps.max(), "hits", int((hit >= 0).sum()))
    np.savez_compressed(Path(__file__).resolve().parent / "rays.npz", **data)


if __name__ == "__main__":
    main()
