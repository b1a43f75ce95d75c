"""Second, independent restatement of the shader path in numpy float32.

Written from src/main_view.wgsl (:78-146 helpers, :150-175 hit_triangle,
:177-220 ray_color, :229-279 nonlinear_ray_color, :347-366 primary rays) with
one numpy float32 operation per WGSL operation (numpy element-wise float32
arithmetic rounds every operation and never fuses a*b+c), so for fields without
transcendental calls it must agree bit for bit with the C++ oracle.  Used by
make_golden.py to write the golden fixtures the oracle is checked against;
small cases only (a Python loop per ray step).
"""
from __future__ import annotations

import numpy as np

f32 = np.float32
EPS = f32(0.0000001)


def dot(a, b):
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]


def cross(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def add(a, b):
    return (a[0] + b[0], a[1] + b[1], a[2] + b[2])


def sub(a, b):
    return (a[0] - b[0], a[1] - b[1], a[2] - b[2])


def scale(s, a):
    return (s * a[0], s * a[1], s * a[2])


def div(a, s):
    return (a[0] / s, a[1] / s, a[2] / s)


def length(a):
    return np.sqrt(dot(a, a))


def normalize(a):
    return div(a, np.sqrt(dot(a, a)))


def vec(x, y, z):
    return (f32(x), f32(y), f32(z))


def refraction_index(t):
    P, c1, c2 = f32(101325.0), f32(0.0000104), f32(0.00366)
    return c1 * P * (f32(1.0) + P * (f32(60.1) - f32(0.972) * t) * f32(1e-10)) / (f32(1.0) + c2 * t)


def refraction(t_in, t_out, v_in, n):
    eta_in, eta_out = refraction_index(t_in), refraction_index(t_out)
    cosi = np.fmin(np.fmax(f32(-1.0), f32(1.0)), dot(v_in, n))  # clamp(-1.0, 1.0, x)
    n_ref = n
    if cosi < f32(0.0):
        cosi = -cosi
    else:
        n_ref = (-n[0], -n[1], -n[2])
    eta = eta_in / eta_out
    k = f32(1.0) - eta * eta * (f32(1.0) - cosi * cosi)
    if k < f32(0.0):
        d = f32(2.0) * dot(n_ref, v_in)
        return sub(v_in, scale(d, n_ref))
    return add(scale(eta, v_in), scale(eta * cosi - np.sqrt(k), n_ref))


def point_plane_distance(p, n, p0):
    d = dot(p0, n)
    return np.abs(dot(p, n) - d)


def translate(v, dx, dy, dz):
    return (v[0] + dx, v[1] + dy, v[2] + dz)


def field(name, p_prev, p, v0, v, t):
    if name == "identity":
        return v
    if name == "linear":
        return v0
    if name == "lorenz":
        rho, sigma, beta = f32(28.0), f32(10.0), f32(8.0 / 3.0)
        return (sigma * (p[1] - p[0]), p[0] * (rho - p[2]) - p[1], p[0] * p[1] - beta * p[2])
    if name == "roessler":
        a, b, c = f32(0.1), f32(0.1), f32(14.0)
        return (-p[1] - p[2], p[0] + a * p[1], b + p[2] * (p[0] - c))
    if name == "translation_x":
        return translate(v0, f32(0.5) * t, f32(0.0), f32(0.0))
    if name in ("mirage_spherical", "mirage_plane"):
        t_env = f32(15.0)
        if name == "mirage_spherical":
            t_src, max_dist = f32(200.0), f32(0.25)
            center = vec(-0.5, 0.5, -0.5)
            center_dest = sub(p, center)
            normal = normalize(center_dest)
            dist_in = length(sub(p_prev, center))
            dist_out = length(center_dest)
        else:
            t_src, max_dist = f32(30.0), f32(0.01)
            plane_p0, normal = vec(0.0, 0.1, 0.0), vec(0.0, 1.0, 0.0)
            dist_in = point_plane_distance(p_prev, normal, plane_p0)
            dist_out = point_plane_distance(p, normal, plane_p0)
        part_in = np.fmin(np.fmax(f32(0.0), f32(1.0)), dist_in / max_dist)
        part_out = np.fmin(np.fmax(f32(0.0), f32(1.0)), dist_out / max_dist)
        t_in = part_in * t_env + (f32(1.0) - part_in) * t_src
        t_out = part_out * t_env + (f32(1.0) - part_out) * t_src
        return refraction(t_in, t_out, v, normal)
    raise KeyError(name)


class Scene:
    def __init__(self, xyz, faces, face_rgb=None):
        xyz = np.asarray(xyz, np.float32)
        faces = np.asarray(faces, np.int64)
        a, b, c = xyz[faces[:, 0]], xyz[faces[:, 1]], xyz[faces[:, 2]]
        self.v0 = tuple(a[:, k] for k in range(3))
        self.e1 = tuple(b[:, k] - a[:, k] for k in range(3))
        self.e2 = tuple(c[:, k] - a[:, k] for k in range(3))
        self.rgb = None if face_rgb is None else np.asarray(face_rgb, np.float32)


def ray_color(sc, origin, direction, max_dist):
    """Closest hit over all faces (vectorised over faces, first index on ties)."""
    with np.errstate(all="ignore"):
        d = tuple(np.full_like(sc.v0[0], direction[k]) for k in range(3))
        h = cross(d, sc.e2)
        a = dot(sc.e1, h)
        ok = ~((a > -EPS) & (a < EPS))
        f = f32(1.0) / a
        s = tuple(f32(origin[k]) - sc.v0[k] for k in range(3))
        u = f * dot(s, h)
        ok &= ~((u < f32(0.0)) | (u > f32(1.0)))
        q = cross(s, sc.e1)
        v = f * dot(d, q)
        ok &= ~((v < f32(0.0)) | (u + v > f32(1.0)))
        t = f * dot(sc.e2, q)
        ok &= t > EPS
        valid = ok & (t > f32(0.0)) & (t < max_dist)
    if not valid.any():
        return None
    tv = np.where(valid, t, np.float32(np.inf))
    i = int(np.argmin(tv))
    tt = tv[i]
    normal = normalize(cross((sc.e1[0][i], sc.e1[1][i], sc.e1[2][i]), (sc.e2[0][i], sc.e2[1][i], sc.e2[2][i])))
    nd = (-direction[0], -direction[1], -direction[2])
    intensity = np.fmax(dot(normal, nd), f32(0.0))
    if intensity == f32(0.0):
        intensity = np.fmax(dot((-normal[0], -normal[1], -normal[2]), nd), f32(0.0))
    spec = np.power(intensity, f32(64.0), dtype=np.float32)
    shade = (f32(0.01) + intensity) + spec
    base = (np.abs(normal[0]), np.abs(normal[1]), np.abs(normal[2])) if sc.rgb is None else tuple(sc.rgb[i])
    return (shade * base[0], shade * base[1], shade * base[2], tt), i


def march(sc, fname, start_point, start_dir, h_initial, t_max, max_steps, adaptive, field_weight,
          h_fine=0.001, h_fine_above=0.002, kahan=False):
    fw = f32(field_weight)
    h_initial, h_fine, h_fine_above, t_max = f32(h_initial), f32(h_fine), f32(h_fine_above), f32(t_max)
    cur_point, cur_dir = start_point, start_dir
    t = f32(0.0)
    last_v = vec(0, 0, 0)
    last_diff = f32(-1.0)
    h = h_initial
    color, face, has_color = None, -1, False
    cp, ct = [f32(0.0)] * 3, f32(0.0)
    steps = 0
    half, two, six, ten = f32(0.5), f32(2.0), f32(6.0), f32(10.0)
    while True:
        if max_steps > 0:
            if steps >= max_steps:
                break
        elif not (t <= t_max):
            break
        hh = half * h
        k1 = field(fname, cur_point, cur_point, start_dir, cur_dir, t)
        k2 = field(fname, cur_point, add(cur_point, scale(hh, k1)), start_dir, k1, t + hh)
        k3 = field(fname, cur_point, add(cur_point, scale(hh, k2)), start_dir, k2, t + hh)
        k4 = field(fname, cur_point, add(cur_point, scale(h, k3)), start_dir, k3, t + h)
        v = div(add(add(add(k1, scale(two, k2)), scale(two, k3)), k4), six)
        diff = length(sub(v, last_v))
        if adaptive and last_diff >= f32(0.0) and diff > ten * last_diff and h > h_fine_above:
            h = h_fine
            continue
        cur_dir = add(scale(f32(1.0) - fw, cur_dir), scale(fw, v))
        step_dir = scale(h, cur_dir)
        if not has_color:
            r = ray_color(sc, cur_point, normalize(step_dir), length(step_dir))
            if r is not None:
                color, face, has_color = r[0], r[1], True
        if kahan:
            np_ = []
            for k in range(3):
                y = step_dir[k] - cp[k]
                s = cur_point[k] + y
                cp[k] = (s - cur_point[k]) - y
                np_.append(s)
            cur_point = tuple(np_)
            y = h - ct
            s = t + y
            ct = (s - t) - y
            t = s
        else:
            cur_point = add(cur_point, step_dir)
            t = t + h
        last_v = v
        if two * diff < last_diff and h < h_initial:
            h = h_initial
        last_diff = diff
        steps += 1
    return color, face, cur_point, steps


def camera_basis(origin, view_direction, up, W, H, focal, vh):
    width, height = f32(W), f32(H)
    aspect = width / height
    vh = f32(vh)
    vw = aspect * vh
    vd = tuple(f32(x) for x in view_direction)
    w = (-vd[0], -vd[1], -vd[2])
    horizontal = cross(tuple(f32(x) for x in up), w)
    vertical = cross(w, horizontal)
    return dict(origin=tuple(f32(x) for x in origin), vd=vd, nh=normalize(horizontal), nv=normalize(vertical),
                width=width, height=height, vw=vw, vh=vh, focal=f32(focal))


def primary_dir(b, gx, gy):
    u = f32(gx) / (b["width"] - f32(1.0)) * b["vw"] - f32(0.5) * b["vw"]
    v = f32(gy) / (b["height"] - f32(1.0)) * b["vh"] - f32(0.5) * b["vh"]
    s = add(add(scale(u, b["nh"]), scale(v, b["nv"])), scale(b["focal"], b["vd"]))
    return normalize(s)


def unorm8(x):
    c = np.fmin(np.fmax(f32(x), f32(0.0)), f32(1.0))
    return int(np.rint(c * f32(255.0)))
