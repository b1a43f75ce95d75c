// oracle_capi.cpp — C entry points over linon_oracle.hpp for the test suite,
// smoke() and bench.py's CPU-baseline leg (ctypes).  TEST INFRASTRUCTURE ONLY.
//
// Build: oracle/Makefile (g++ -O2 -ffp-contract=off -fopenmp, no -ffast-math).
// Every entry point follows the shader routine named in linon_oracle.hpp.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/linon.h"
#include "linon_oracle.hpp"

using namespace linon_oracle;

namespace {

Scene make_scene(const float* xyz, int nv, const uint32_t* abc, int nf, const float* face_rgb) {
  Scene s;
  s.xyz.assign(xyz, xyz + size_t(nv) * 3);
  s.abc.assign(abc, abc + size_t(nf) * 3);
  if (face_rgb) s.face_rgb.assign(face_rgb, face_rgb + size_t(nf) * 3);
  return s;
}

March make_march(const linon_settings* st, const linon_march_params* mp) {
  March m;
  m.h_initial = mp->h_initial;
  m.t_max = mp->t_max;
  m.max_steps = mp->max_steps;
  m.adaptive = mp->adaptive != 0;
  m.h_fine = mp->h_fine;
  m.h_fine_above = mp->h_fine_above;
  m.stop_on_hit = mp->stop_on_hit != 0;
  m.kahan = mp->kahan != 0;
  m.focal_length = mp->focal_length;
  m.viewport_height = mp->viewport_height;
  m.linear_mode = mp->linear_mode != 0;
  m.field_weight = st ? st->field_weight : 1.0f;
  return m;
}

Camera make_camera(const linon_camera* c) {
  Camera k;
  for (int i = 0; i < 3; ++i) {
    k.origin[i] = c->origin[i];
    k.view_direction[i] = c->view_direction[i];
    k.up[i] = c->up[i];
  }
  return k;
}

template <class T>
void render_impl(const Scene& sc, int field, const Camera& cam, const March& m, int W, int H,
                 const int32_t* pixels, int64_t npix, uint8_t* color, float* mapping,
                 double* mapping64, int32_t* hit, int32_t* steps, int nthreads) {
  CameraBasis<T> b = camera_basis<T>(cam, W, H, m);
  const int64_t n = pixels ? npix : int64_t(W) * H;
#pragma omp parallel for schedule(dynamic, 8) num_threads(nthreads)
  for (int64_t i = 0; i < n; ++i) {
    int64_t pix = pixels ? pixels[i] : i;
    int row = int(pix / W), x = int(pix % W);
    RayResult<T> r = render_pixel<T>(sc, field, b, W, H, x, row, m);
    if (color) {
      color[4 * i + 0] = unorm8(float(r.color.x));
      color[4 * i + 1] = unorm8(float(r.color.y));
      color[4 * i + 2] = unorm8(float(r.color.z));
      color[4 * i + 3] = unorm8(float(r.color.w));
    }
    if (mapping) {
      mapping[4 * i + 0] = float(r.mapping.x);
      mapping[4 * i + 1] = float(r.mapping.y);
      mapping[4 * i + 2] = float(r.mapping.z);
      mapping[4 * i + 3] = float(r.mapping.w);
    }
    if (mapping64) {
      mapping64[4 * i + 0] = double(r.mapping.x);
      mapping64[4 * i + 1] = double(r.mapping.y);
      mapping64[4 * i + 2] = double(r.mapping.z);
      mapping64[4 * i + 3] = double(r.mapping.w);
    }
    if (hit) hit[i] = r.face;
    if (steps) steps[i] = r.steps;
  }
}

}  // namespace

extern "C" {

// Renders a frame (pixels == NULL) or the listed pixels (indices row*W+x,
// outputs compacted in list order).  precision: 32 or 64.
// accel != 0 tests each segment against the faces the oracle's candidate
// grid lists (the same result as the loop over all faces, faster on large
// scenes); accel == 0 is the shader's loop.
int oracle_render(int precision, const float* xyz, int nv, const uint32_t* abc, int nf,
                  const float* face_rgb, const linon_camera* cam, const linon_settings* st,
                  const linon_march_params* mp, int field, int W, int H, const int32_t* pixels,
                  int64_t npix, uint8_t* color, float* mapping, double* mapping64, int32_t* hit,
                  int32_t* steps, int nthreads, int accel) {
  if (!xyz || !abc || !cam || !mp || W <= 0 || H <= 0) return LINON_EINVAL;
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  Scene sc = make_scene(xyz, nv, abc, nf, face_rgb);
  Accel grid;
  if (accel) {
    build_accel(sc, grid);
    sc.accel = &grid;
  }
  March m = make_march(st, mp);
  Camera c = make_camera(cam);
  if (precision == 64)
    render_impl<double>(sc, field, c, m, W, H, pixels, npix, color, mapping, mapping64, hit, steps,
                        nthreads);
  else
    render_impl<float>(sc, field, c, m, W, H, pixels, npix, color, mapping, mapping64, hit, steps,
                       nthreads);
  return LINON_OK;
}

// FP32 operation counts of one ray (summed over its steps) for the listed
// pixels: out[i*6 + {0..5}] = add, mul, div, sqrt, cmp, transcendental;
// steps_out[i] = accepted steps.
int oracle_count_ops(const float* xyz, int nv, const uint32_t* abc, int nf,
                     const linon_camera* cam, const linon_settings* st,
                     const linon_march_params* mp, int field, int W, int H,
                     const int32_t* pixels, int npix, int64_t* out, int32_t* steps_out) {
  Scene sc = make_scene(xyz, nv, abc, nf, nullptr);
  March m = make_march(st, mp);
  Camera c = make_camera(cam);
  CameraBasis<CountingFloat> b = camera_basis<CountingFloat>(c, W, H, m);
  for (int i = 0; i < npix; ++i) {
    int row = pixels[i] / W, x = pixels[i] % W;
    counts() = OpCounts();
    RayResult<CountingFloat> r = render_pixel<CountingFloat>(sc, field, b, W, H, x, row, m);
    const OpCounts& k = counts();
    out[6 * i + 0] = k.add; out[6 * i + 1] = k.mul; out[6 * i + 2] = k.div;
    out[6 * i + 3] = k.sqrt; out[6 * i + 4] = k.cmp; out[6 * i + 5] = k.transc;
    steps_out[i] = r.steps;
  }
  return LINON_OK;
}

// Algorithmic FP32 operations per accepted step (TraceFloat): the operations
// the ray's endpoint depends on, loop-invariant work and launch-constant
// products excluded.  Per listed pixel, the live loop-variant operations of
// a march of `steps_a` and of `steps_b` (> steps_a) fixed steps on the given
// scene are taken and their difference divided by steps_b - steps_a, so the
// work before the first and after the last step cancels.  out[i*8 + k],
// k = add, mul, div, sqrt, transcendental, free, cmp (TraceKind order from 1).
int oracle_count_live_ops(const float* xyz, int nv, const uint32_t* abc, int nf,
                          const linon_camera* cam, const linon_settings* st,
                          const linon_march_params* mp, int field, int W, int H,
                          const int32_t* pixels, int npix, int steps_a, int steps_b, double* out) {
  if (steps_b <= steps_a || steps_a <= 0 || mp->adaptive) return LINON_EINVAL;
  Scene sc = make_scene(xyz, nv, abc, nf, nullptr);
  Camera c = make_camera(cam);
  for (int i = 0; i < npix; ++i) {
    int row = pixels[i] / W, x = pixels[i] % W;
    long long cnt[2][8];
    for (int pass = 0; pass < 2; ++pass) {
      March m = make_march(st, mp);
      m.max_steps = pass == 0 ? steps_a : steps_b;
      m.stop_on_hit = false;
      tape().clear();
      CameraBasis<TraceFloat> b = camera_basis<TraceFloat>(c, W, H, m);
      RayResult<TraceFloat> r = render_pixel<TraceFloat>(sc, field, b, W, H, x, row, m);
      tape().roots.push_back(r.mapping.x.id);
      tape().roots.push_back(r.mapping.y.id);
      tape().roots.push_back(r.mapping.z.id);
      tape().count(cnt[pass]);
    }
    for (int k = 0; k < 7; ++k)
      out[8 * i + k] = double(cnt[1][k + 1] - cnt[0][k + 1]) / double(steps_b - steps_a);
    out[8 * i + 7] = 0.0;
  }
  tape().clear();
  return LINON_OK;
}

// Counts of one field evaluation at the given inputs (13 floats).
int oracle_count_field(int field, const float* in, int64_t* out6) {
  counts() = OpCounts();
  V3<CountingFloat> pp(in[0], in[1], in[2]), p(in[3], in[4], in[5]), v0(in[6], in[7], in[8]),
      v(in[9], in[10], in[11]);
  (void)field_eval<CountingFloat>(field, pp, p, v0, v, CountingFloat(in[12]));
  const OpCounts& k = counts();
  out6[0] = k.add; out6[1] = k.mul; out6[2] = k.div; out6[3] = k.sqrt; out6[4] = k.cmp;
  out6[5] = k.transc;
  return LINON_OK;
}

// Field evaluation at n points: in is n*13 (p_prev, p, v0, v, t), out n*3.
int oracle_field_eval(int precision, int field, const float* in, int64_t n, float* out,
                      double* out64) {
  for (int64_t i = 0; i < n; ++i) {
    const float* q = in + 13 * i;
    if (precision == 64) {
      V3<double> r = field_eval<double>(field, V3<double>(q[0], q[1], q[2]),
                                        V3<double>(q[3], q[4], q[5]), V3<double>(q[6], q[7], q[8]),
                                        V3<double>(q[9], q[10], q[11]), double(q[12]));
      if (out) { out[3 * i] = float(r.x); out[3 * i + 1] = float(r.y); out[3 * i + 2] = float(r.z); }
      if (out64) { out64[3 * i] = r.x; out64[3 * i + 1] = r.y; out64[3 * i + 2] = r.z; }
    } else {
      V3<float> r = field_eval<float>(field, V3<float>(q[0], q[1], q[2]),
                                      V3<float>(q[3], q[4], q[5]), V3<float>(q[6], q[7], q[8]),
                                      V3<float>(q[9], q[10], q[11]), q[12]);
      out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
    }
  }
  return LINON_OK;
}

// hit_triangle known-answer interface: tri 9 floats, ray 6 floats -> t.
float oracle_hit_triangle(const float* tri, const float* ray) {
  V3<float> a(tri[0], tri[1], tri[2]), b(tri[3], tri[4], tri[5]), c(tri[6], tri[7], tri[8]);
  return hit_triangle<float>(a, b, c, V3<float>(ray[0], ray[1], ray[2]),
                             V3<float>(ray[3], ray[4], ray[5]));
}

// Primary ray directions of the listed pixels (precision 32 -> float out).
int oracle_primary_dirs(const linon_camera* cam, const linon_march_params* mp, int W, int H,
                        const int32_t* pixels, int npix, float* out) {
  March m = make_march(nullptr, mp);
  Camera c = make_camera(cam);
  CameraBasis<float> b = camera_basis<float>(c, W, H, m);
  for (int i = 0; i < npix; ++i) {
    int row = pixels[i] / W, x = pixels[i] % W;
    V3<float> d = primary_dir(b, x, H - 1 - row);
    out[3 * i] = d.x; out[3 * i + 1] = d.y; out[3 * i + 2] = d.z;
  }
  return LINON_OK;
}

// The same directions in FP64 (the camera basis and the normalisation in
// double), for the FP64 finite-time exponent.
int oracle_primary_dirs64(const linon_camera* cam, const linon_march_params* mp, int W, int H,
                          const int32_t* pixels, int npix, double* out) {
  March m = make_march(nullptr, mp);
  Camera c = make_camera(cam);
  CameraBasis<double> b = camera_basis<double>(c, W, H, m);
  for (int i = 0; i < npix; ++i) {
    int row = pixels[i] / W, x = pixels[i] % W;
    V3<double> d = primary_dir(b, x, H - 1 - row);
    out[3 * i] = d.x; out[3 * i + 1] = d.y; out[3 * i + 2] = d.z;
  }
  return LINON_OK;
}

// Lyapunov overlay over a whole frame.  out_rgba8 gets the stored colour;
// exponents (W*H) is written where the shader writes it.
int oracle_overlay(int precision, const uint8_t* rgba, const float* mapping, int W, int H,
                   const linon_settings* st, int srgb, uint8_t* out_rgba8, float* exponents,
                   int nthreads) {
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int y = 0; y < H; ++y) {
    for (int x = 0; x < W; ++x) {
      float c[4];
      bool wrote;
      if (precision == 64)
        overlay_pixel<double>(rgba, mapping, W, H, x, y, st->overlay_mode,
                              st->central_difference_delta, st->lyapunov_scaling, c, exponents,
                              &wrote);
      else
        overlay_pixel<float>(rgba, mapping, W, H, x, y, st->overlay_mode,
                             st->central_difference_delta, st->lyapunov_scaling, c, exponents,
                             &wrote);
      if (srgb) {
        for (int i = 0; i < 3; ++i) c[i] = srgb_from_linear(c[i]);
      }
      for (int i = 0; i < 4; ++i) out_rgba8[4 * (size_t(y) * W + x) + i] = unorm8(c[i]);
    }
  }
  return LINON_OK;
}

// Finite-time exponent in FP64: ln(max_nb |e(nb) - e(c)| / |d0(nb) - d0(c)|) / T
// over the 4-neighbourhood inside the image.  d0 = FP32 primary directions.
int oracle_ftle(const linon_camera* cam, const linon_march_params* mp, int W, int H,
                const float* mapping, double T, float* out) {
  March m = make_march(nullptr, mp);
  Camera c = make_camera(cam);
  CameraBasis<float> b = camera_basis<float>(c, W, H, m);
  std::vector<float> dirs(size_t(W) * H * 3);
  for (int row = 0; row < H; ++row)
    for (int x = 0; x < W; ++x) {
      V3<float> d = primary_dir(b, x, H - 1 - row);
      float* o = &dirs[3 * (size_t(row) * W + x)];
      o[0] = d.x; o[1] = d.y; o[2] = d.z;
    }
  const int dx[4] = {1, -1, 0, 0}, dy[4] = {0, 0, 1, -1};
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      size_t ci = size_t(y) * W + x;
      double best = -1.0;
      for (int k = 0; k < 4; ++k) {
        int nx = x + dx[k], ny = y + dy[k];
        if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
        size_t ni = size_t(ny) * W + nx;
        double de = 0, dd = 0;
        for (int j = 0; j < 3; ++j) {
          double a = double(mapping[4 * ni + j]) - double(mapping[4 * ci + j]);
          double q = double(dirs[3 * ni + j]) - double(dirs[3 * ci + j]);
          de += a * a;
          dd += q * q;
        }
        double r = std::sqrt(de) / std::sqrt(dd);
        if (r > best) best = r;
      }
      out[ci] = best > 0.0 ? float(std::log(best) / T) : -INFINITY;
    }
  return LINON_OK;
}

// Path capture: n_rays rays at normalised positions, positions recorded
// before every `every`-th step (+ the final one when record_final).
int oracle_capture(int precision, int field, const linon_camera* cam, const linon_settings* st,
                   const linon_march_params* mp, int W, int H, const float* pos_xy, int n_rays,
                   float h, int n_steps, int every, int record_final, float* out) {
  March m = make_march(st, mp);
  Camera c = make_camera(cam);
  int npts = n_steps / every + (record_final ? 1 : 0);
  if (n_steps % every) npts = (n_steps + every - 1) / every + (record_final ? 1 : 0);
#pragma omp parallel for schedule(dynamic, 1)
  for (int r = 0; r < n_rays; ++r) {
    float* o = out + size_t(r) * npts * 4;
    if (precision == 64) {
      CameraBasis<double> b = camera_basis<double>(c, W, H, m);
      V3<double> d = position_dir<double>(b, pos_xy[2 * r], pos_xy[2 * r + 1]);
      sample_ray<double>(field, b.origin, d, double(m.field_weight), double(h), n_steps, every,
                         record_final != 0, o);
    } else {
      CameraBasis<float> b = camera_basis<float>(c, W, H, m);
      V3<float> d = position_dir<float>(b, pos_xy[2 * r], pos_xy[2 * r + 1]);
      sample_ray<float>(field, b.origin, d, m.field_weight, h, n_steps, every, record_final != 0,
                        o);
    }
  }
  return LINON_OK;
}

int oracle_outline_select(const float* e, int W, int H, int stride, float min_exp, int* px,
                          int* py) {
  outline_select(e, W, H, stride, min_exp, px, py);
  return LINON_OK;
}

int oracle_max_threads(void) { return omp_get_max_threads(); }

}  // extern "C"
