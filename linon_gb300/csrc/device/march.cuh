// march.cuh — nonlinear ray-casting kernels (device code compiled by NVRTC
// together with the CUDA C that the WGSL front end generated for the field
// functions).
//
// Reference: src/main_view.wgsl
//   :339-376 main_view  (primary ray per pixel, stores)
//   :229-279 nonlinear_ray_color (RK4, adaptive step, first-hit colour,
//            endpoint "mapping")
//   :177-220 ray_color, :150-175 hit_triangle (Moeller-Trumbore)
//   :281-314 sample_rays, :470-479 capture seeds
// Every arithmetic expression keeps the shader's evaluation order, so a
// module compiled with LINON_PRECISE and --fmad=false is op-for-op the FP32
// restatement.  Fast modules let the compiler contract a*b+c into FMA, issue
// the march's float3 arithmetic as packed FP32 pairs (wgsl_rt.cuh vmadd &c.)
// and use the hardware reciprocal square root.
#pragma once

#include "wgsl_rt.cuh"
#include "march_types.h"

namespace linon {

using wgsl::vec3f;

// --------------------------------------------------------------------------
// Scene access.  Triangles are four float4 each: (v0, face id bits),
// (e1 = v1 - v0, 0), (e2 = v2 - v0, 0), (unit normal n, d = n . v0); e1/e2
// are the differences hit_triangle computes (IEEE subtraction, so
// precomputing them changes nothing); the plane (zero for a degenerate
// triangle) only serves conservative culling.  BVH nodes are two float4: (lo.xyz, first), (hi.xyz, count);
// count > 0 is a leaf over triangles [first, first+count), otherwise the
// children are nodes first and first+1.  Node boxes are inflated on the host
// so that culling never drops a triangle the brute-force loop would hit.
// --------------------------------------------------------------------------
struct SceneView {
  const float4* tris;
  const float4* nodes;
  const float4* face_rgb;
  int n_tris;
  int n_nodes;
  float margin;
  const float* grid;  // distance grid (see DevScene), NULL: none
  const int2* cells;  // per-cell candidate lists (see DevScene), NULL: none
  const int* cell_tris;
  float reach;
  int gx, gy, gz;
  float gox, goy, goz, gcell, ginv;
};

__device__ __forceinline__ vec3f xyz(const float4& a) { return vec3f(a.x, a.y, a.z); }

// hit_triangle, main_view.wgsl:150-175 (eps 1e-7, no back-face culling)
__device__ __forceinline__ float hit_triangle(const vec3f& v0, const vec3f& edge1,
                                              const vec3f& edge2, const vec3f& origin,
                                              const vec3f& direction) {
  const float eps = 1e-7f;
  vec3f h = wgsl::cross(direction, edge2);
  float a = wgsl::dot(edge1, h);
  if (a > -eps && a < eps) return -1.0f;
  float f = 1.0f / a;
  vec3f s = origin - v0;
  float u = f * wgsl::dot(s, h);
  if (u < 0.0f || u > 1.0f) return -1.0f;
  vec3f q = wgsl::cross(s, edge1);
  float v = f * wgsl::dot(direction, q);
  if (v < 0.0f || u + v > 1.0f) return -1.0f;
  float t = f * wgsl::dot(edge2, q);
  if (t > eps) return t;
  return -1.0f;
}

struct HitRec {
  float t;   // -1: none
  int id;    // original face index
  int slot;  // position in the triangle array
};

// Closest hit of the segment origin + [0, max_dist) * direction, ties to the
// lower face index (the brute-force loop's strict `<`, main_view.wgsl:193).
__device__ __forceinline__ void test_tri(const SceneView& sc, int slot, const vec3f& origin,
                                         const vec3f& direction, float max_dist, HitRec& best) {
  // A segment whose two ends lie on the same side of the triangle's plane,
  // both farther than the culling margin, cannot produce a hit inside the
  // segment (the rounding of the plane distances and of hit_triangle is
  // orders of magnitude below the margin): skip the full test.
  const float4 P = sc.tris[4 * slot + 3];
  const vec3f n = xyz(P);
  const float s0 = wgsl::dot(origin, n) - P.w;
  const float s1 = fmaf(max_dist, wgsl::dot(direction, n), s0);
  if ((s0 > sc.margin && s1 > sc.margin) || (s0 < -sc.margin && s1 < -sc.margin)) return;
  const float4 A = sc.tris[4 * slot];
  const float4 B = sc.tris[4 * slot + 1];
  const float4 C = sc.tris[4 * slot + 2];
  float t_new = hit_triangle(xyz(A), xyz(B), xyz(C), origin, direction);
  if (t_new > 0.0f && t_new < max_dist) {
    int id = __float_as_int(A.w);
    if (best.t < 0.0f || t_new < best.t || (t_new == best.t && id < best.id)) {
      best.t = t_new;
      best.id = id;
      best.slot = slot;
    }
  }
}

__device__ __forceinline__ bool box_overlap(const float4& lo, const float4& hi, const vec3f& smin,
                                            const vec3f& smax) {
  return !(smax.x < lo.x || smin.x > hi.x || smax.y < lo.y || smin.y > hi.y || smax.z < lo.z ||
           smin.z > hi.z);
}

#ifndef LINON_BVH_STACK
#define LINON_BVH_STACK 48
#endif

// Launch bounds of the persistent batched kernels: up to 256-thread CTAs,
// at least LINON_BATCH_MIN_CTAS (default 4) of them resident per SM, which
// caps the kernels at 64 registers (64 uneven views, warps taking whole
// tiles: 11.55 ms at 4, 11.73 ms at 3 (80 registers), 14.1 ms at 5).
#ifndef LINON_BATCH_MIN_CTAS
#define LINON_BATCH_MIN_CTAS 4
#endif
#define LINON_BATCH_BOUNDS __launch_bounds__(256, LINON_BATCH_MIN_CTAS)

// Launch bounds of the one-CTA-per-tile batched kernels: 128-thread CTAs,
// at least LINON_MULTI_MIN_CTAS (default 8) resident per SM, which caps them
// at 64 registers (64 uneven views: 16.5 ms uncapped at 72 registers, 14.8
// ms at 8 or 9 CTAs per SM, 15.6 ms at 10, 16.2 ms at 12).
#ifndef LINON_MULTI_MIN_CTAS
#define LINON_MULTI_MIN_CTAS 8
#endif
#define LINON_MULTI_BOUNDS __launch_bounds__(128, LINON_MULTI_MIN_CTAS)

// Launch bounds of the plain march kernels (128-thread CTAs).  Defining
// LINON_MARCH_MIN_CTAS adds the minimum resident CTAs per SM, which caps the
// registers per thread (and may spill).
#ifdef LINON_MARCH_MIN_CTAS
#define LINON_MARCH_BOUNDS __launch_bounds__(128, LINON_MARCH_MIN_CTAS)
#else
#define LINON_MARCH_BOUNDS __launch_bounds__(128)
#endif


// Segment query; seg_end is origin + step (the unnormalised step vector).
// PAIR selects the walk: false visits one node per iteration (the smallest
// code, best for the small scenes staged in shared memory); true tests both
// children of an inner node when it is reached, descends only into the
// overlapping ones and loads each node record once (fewer iterations and
// loads on deep trees read through L1).  Both test the triangles of the
// leaves whose boxes and all ancestors' boxes overlap the segment's box.
template <bool PAIR = false>
__device__ __forceinline__ HitRec intersect_segment(const SceneView& sc, const vec3f& origin,
                                                    const vec3f& direction, float max_dist,
                                                    const vec3f& seg_end, int* err) {
  HitRec best;
  best.t = -1.0f;
  best.id = 0x7fffffff;
  best.slot = -1;
  if (sc.n_nodes == 0) {
    for (int i = 0; i < sc.n_tris; ++i) test_tri(sc, i, origin, direction, max_dist, best);
    return best;
  }
  vec3f smin = wgsl::min(origin, seg_end), smax = wgsl::max(origin, seg_end);
  int stack[LINON_BVH_STACK];
  int sp = 0;
  if (!PAIR) {
    int node = 0;
    for (;;) {
      const float4 lo = sc.nodes[2 * node];
      const float4 hi = sc.nodes[2 * node + 1];
      if (box_overlap(lo, hi, smin, smax)) {
        const int first = __float_as_int(lo.w);
        const int count = __float_as_int(hi.w);
        if (count > 0) {
          for (int i = 0; i < count; ++i) test_tri(sc, first + i, origin, direction, max_dist, best);
        } else {
          if (sp < LINON_BVH_STACK) {
            stack[sp++] = first + 1;
          } else {
            // The host caps the tree depth below the stack size, so this is
            // unreachable; if it ever were reached the flag reports it.
            atomicOr(err, 2);
          }
          node = first;
          continue;
        }
      }
      if (sp == 0) break;
      node = stack[--sp];
    }
    return best;
  }
  float4 lo = sc.nodes[0], hi = sc.nodes[1];
  if (!box_overlap(lo, hi, smin, smax)) return best;
  for (;;) {
    const int first = __float_as_int(lo.w);
    const int count = __float_as_int(hi.w);
    if (count > 0) {
      for (int i = 0; i < count; ++i) test_tri(sc, first + i, origin, direction, max_dist, best);
    } else {
      const float4 lo0 = sc.nodes[2 * first], hi0 = sc.nodes[2 * first + 1];
      const float4 lo1 = sc.nodes[2 * first + 2], hi1 = sc.nodes[2 * first + 3];
      const bool o0 = box_overlap(lo0, hi0, smin, smax);
      const bool o1 = box_overlap(lo1, hi1, smin, smax);
      if (o0) {
        if (o1) {
          if (sp < LINON_BVH_STACK) stack[sp++] = first + 1;
          else atomicOr(err, 2);  // unreachable: the host caps the depth
        }
        lo = lo0;
        hi = hi0;
        continue;
      }
      if (o1) {
        lo = lo1;
        hi = hi1;
        continue;
      }
    }
    if (sp == 0) break;
    const int node = stack[--sp];
    lo = sc.nodes[2 * node];
    hi = sc.nodes[2 * node + 1];
  }
  return best;
}

// Lower bound on the distance from q to any triangle of the scene: the
// distance to the nearest (inflated) leaf box, found by a pruned traversal
// that visits the nearer child first.  A segment starting at q and shorter
// than this bound cannot reach any inflated box, so it cannot hit anything
// the brute-force loop would hit (the same margin argument as the culling).
__device__ __forceinline__ float box_dist2(const float4& lo, const float4& hi, const vec3f& q) {
  const float dx = fmaxf(fmaxf(lo.x - q.x, q.x - hi.x), 0.0f);
  const float dy = fmaxf(fmaxf(lo.y - q.y, q.y - hi.y), 0.0f);
  const float dz = fmaxf(fmaxf(lo.z - q.z, q.z - hi.z), 0.0f);
  return dx * dx + dy * dy + dz * dz;
}

// Lower bound on the distance from q to the triangles of one leaf: the
// leaf box distance, raised to the smallest distance from q to the leaf's
// triangle planes minus the culling margin (a triangle lies in its plane).
__device__ __forceinline__ float leaf_bound2(const SceneView& sc, int first, int count, float box_d2,
                                             const vec3f& q, float margin) {
  float pmin = 3.0e38f;
  for (int i = 0; i < count; ++i) {
    // a degenerate triangle has a zero plane: distance 0, bound 0
    const float4 P = sc.tris[4 * (first + i) + 3];
    const float pd = fabsf(wgsl::dot(q, xyz(P)) - P.w) - margin;
    pmin = fminf(pmin, fmaxf(pd, 0.0f));
  }
  return fmaxf(box_d2, pmin * pmin);
}

__device__ __forceinline__ float nearest_leaf_bound(const SceneView& sc, const vec3f& q, float margin) {
  float best = 3.0e38f;  // squared distance
  int stack[LINON_BVH_STACK];
  int sp = 0;
  int node = 0;
  float nd = box_dist2(sc.nodes[0], sc.nodes[1], q);
  for (;;) {
    if (nd < best) {
      const float4 lo = sc.nodes[2 * node];
      const float4 hi = sc.nodes[2 * node + 1];
      const int count = __float_as_int(hi.w);
      if (count > 0) {
        best = fminf(best, leaf_bound2(sc, __float_as_int(lo.w), count, nd, q, margin));
      } else {
        const int first = __float_as_int(lo.w);
        const float d0 = box_dist2(sc.nodes[2 * first], sc.nodes[2 * first + 1], q);
        const float d1 = box_dist2(sc.nodes[2 * first + 2], sc.nodes[2 * first + 3], q);
        const int near = d0 <= d1 ? first : first + 1;
        const float dnear = fminf(d0, d1), dfar = fmaxf(d0, d1);
        if (dfar < best) {
          // the far child is revisited with its distance re-derived on pop;
          // the tree depth is capped below the stack size, and a full stack
          // would end the query with the trivial bound 0 (no skipping)
          if (sp >= LINON_BVH_STACK) return 0.0f;
          stack[sp++] = near == first ? first + 1 : first;
        }
        node = near;
        nd = dnear;
        continue;
      }
    }
    if (sp == 0) break;
    node = stack[--sp];
    nd = box_dist2(sc.nodes[2 * node], sc.nodes[2 * node + 1], q);
  }
  // shrink by a relative 1e-5 against rounding of the distance itself
  return best >= 3.0e38f ? 3.0e38f : sqrtf(best) * 0.99999f;
}

// Centre of grid cell (ix, iy, iz); the grid build and the queries use this
// same expression.
__device__ __forceinline__ vec3f grid_centre(const SceneView& sc, int ix, int iy, int iz) {
  return vec3f(fmaf(float(ix) + 0.5f, sc.gcell, sc.gox), fmaf(float(iy) + 0.5f, sc.gcell, sc.goy),
               fmaf(float(iz) + 0.5f, sc.gcell, sc.goz));
}

// Segment test through the candidate list of the cell holding the segment's
// start when the lists apply (a segment no longer than `reach` that starts in
// a listed cell can only meet the listed triangles: every leaf box within
// the cell's half diagonal plus `reach` of its centre is listed), otherwise
// the BVH walk.  The same triangles' Moeller-Trumbore results decide, so the
// hit is the BVH's (and the brute-force loop's).
template <bool PAIR>
__device__ __forceinline__ HitRec intersect_segment_cells(const SceneView& sc, const vec3f& origin,
                                                          const vec3f& direction, float max_dist,
                                                          const vec3f& seg_end, int* err) {
  if (sc.cells && max_dist <= sc.reach) {
    const float fx = (origin.x - sc.gox) * sc.ginv, fy = (origin.y - sc.goy) * sc.ginv,
                fz = (origin.z - sc.goz) * sc.ginv;
    if (fx >= 0.0f && fy >= 0.0f && fz >= 0.0f && fx < float(sc.gx) && fy < float(sc.gy) && fz < float(sc.gz)) {
      const int2 l = sc.cells[(size_t(int(fz)) * sc.gy + int(fy)) * sc.gx + int(fx)];
      if (l.y >= 0) {
        HitRec best;
        best.t = -1.0f;
        best.id = 0x7fffffff;
        best.slot = -1;
        for (int k = 0; k < l.y; ++k) test_tri(sc, sc.cell_tris[l.x + k], origin, direction, max_dist, best);
        return best;
      }
    }
  }
  return intersect_segment<PAIR>(sc, origin, direction, max_dist, seg_end, err);
}

// Radius of a safe ball around q: every point closer to q than the result is
// outside every margin-inflated leaf box (hence farther than the culling
// margin from every triangle).  With a distance grid: the bound stored at
// the centre c of q's cell minus |q - c| (triangle inequality); outside the
// grid: the distance to the root box, which holds every leaf box.  Without
// a grid: the BVH query.  The result is shrunk by a relative 1e-5 and 1e-6
// absolute against the rounding of the differences.
__device__ __forceinline__ float safe_radius(const SceneView& sc, const vec3f& q) {
  if (sc.grid) {
    const float fx = (q.x - sc.gox) * sc.ginv, fy = (q.y - sc.goy) * sc.ginv, fz = (q.z - sc.goz) * sc.ginv;
    if (fx >= 0.0f && fy >= 0.0f && fz >= 0.0f && fx < float(sc.gx) && fy < float(sc.gy) && fz < float(sc.gz)) {
      const int ix = int(fx), iy = int(fy), iz = int(fz);
      const float c = sc.grid[(size_t(iz) * sc.gy + iy) * sc.gx + ix];
      const float b = c - wgsl::length(q - grid_centre(sc, ix, iy, iz));
      return fmaxf(b * 0.99999f - 1e-6f, 0.0f);
    }
    if (!(q.x == q.x && q.y == q.y && q.z == q.z)) return 0.0f;
    return fmaxf(sqrtf(box_dist2(sc.nodes[0], sc.nodes[1], q)) * 0.99999f - 1e-6f, 0.0f);
  }
  return nearest_leaf_bound(sc, q, sc.margin);
}

// Shading of ray_color, main_view.wgsl:199-217 (camera is the light source).
__device__ __forceinline__ wgsl::vec4f shade_hit(const SceneView& sc, const HitRec& hit,
                                                 const vec3f& direction) {
  const vec3f d1 = xyz(sc.tris[4 * hit.slot + 1]);
  const vec3f d2 = xyz(sc.tris[4 * hit.slot + 2]);
  vec3f normal = wgsl::normalize(wgsl::cross(d1, d2));
  float intensity = wgsl::max(wgsl::dot(normal, -direction), 0.0f);
  if (intensity == 0.0f) intensity = wgsl::max(wgsl::dot(-normal, -direction), 0.0f);
#if defined(LINON_PRECISE)
  float spec = powf(intensity, 64.0f);
#else
  // x^64 by six squarings (fast modules): a few ulp from powf, and far less
  // code in the march loop than the library pow
  float spec = intensity * intensity;
  spec *= spec;
  spec *= spec;
  spec *= spec;
  spec *= spec;
  spec *= spec;
#endif
  float shade = (0.01f + intensity) + spec;
  vec3f base = wgsl::abs(normal);
  if (sc.face_rgb) {
    const float4 c = sc.face_rgb[hit.id];
    base = vec3f(c.x, c.y, c.z);
  }
  return wgsl::vec4f(shade * base.x, shade * base.y, shade * base.z, hit.t);
}

// --------------------------------------------------------------------------
// Camera, main_view.wgsl:347-366
// --------------------------------------------------------------------------
struct Basis {
  vec3f origin, view_direction, nh, nv;
  float width, height, vw, vh, focal;
};

__device__ __forceinline__ Basis make_basis(const DevCamera& c, int W, int H, float focal,
                                            float viewport_height) {
  Basis b;
  b.width = float(W);
  b.height = float(H);
  float aspect = b.width / b.height;
  b.origin = vec3f(c.o[0], c.o[1], c.o[2]);
  b.view_direction = vec3f(c.d[0], c.d[1], c.d[2]);
  vec3f up(c.u[0], c.u[1], c.u[2]);
  b.focal = focal;
  b.vh = viewport_height;
  b.vw = aspect * b.vh;
  vec3f w = -b.view_direction;
  vec3f horizontal = wgsl::cross(up, w);
  vec3f vertical = wgsl::cross(w, horizontal);
  b.nh = wgsl::normalize(horizontal);
  b.nv = wgsl::normalize(vertical);
  return b;
}

__device__ __forceinline__ vec3f primary_dir(const Basis& b, int gx, int gy) {
  float u = float(gx) / (b.width - 1.0f) * b.vw - 0.5f * b.vw;
  float v = float(gy) / (b.height - 1.0f) * b.vh - 0.5f * b.vh;
  vec3f s = (u * b.nh + v * b.nv) + b.focal * b.view_direction;
  return wgsl::normalize(s);
}

__device__ __forceinline__ vec3f position_dir(const Basis& b, float px, float py) {
  float u2 = px * b.vw - 0.5f * b.vw;
  float v2 = py * b.vh - 0.5f * b.vh;
  vec3f s2 = (u2 * b.nh + v2 * b.nv) + b.focal * b.view_direction;
  return wgsl::normalize(s2);
}

__device__ __forceinline__ unsigned char unorm8(float x) {
  float c = fminf(fmaxf(x, 0.0f), 1.0f);
  return (unsigned char)__float2uint_rn(c * 255.0f);
}

// --------------------------------------------------------------------------
// Ray state and the RK4 march
// --------------------------------------------------------------------------
struct RayState {
  vec3f p, dir, v0;     // position, direction, start direction
  vec3f last_v;
  vec3f cp;             // Kahan carry of p
  float t, ct;          // time and its Kahan carry
  float h, last_diff;
  wgsl::vec4f color;
  vec3f q0;             // centre of the current safe ball
  float safe2;          // its squared radius (< 0: no ball)
  int face;
  int steps;
  int cool;             // steps left before the next safe-distance query
  bool has_color;
};

__device__ __forceinline__ void ray_init(RayState& r, const vec3f& origin, const vec3f& dir,
                                         float h_initial) {
  r.p = origin;
  r.dir = dir;
  r.v0 = dir;
  r.last_v = vec3f(0.0f, 0.0f, 0.0f);
  r.cp = vec3f(0.0f, 0.0f, 0.0f);
  r.t = 0.0f;
  r.ct = 0.0f;
  r.h = h_initial;
  r.last_diff = -1.0f;
  r.color = wgsl::vec4f(0.0f, 0.0f, 0.0f, 0.0f);
  r.face = -1;
  r.steps = 0;
  r.q0 = origin;
  r.safe2 = -1.0f;
  r.cool = 0;
  r.has_color = false;
}

__device__ __forceinline__ void kahan_add(float& sum, float& c, float x) {
  float y = x - c;
  float t = sum + y;
  c = (t - sum) - y;
  sum = t;
}
// kahan_add on each component (packed x/y pairs in fast modules)
__device__ __forceinline__ void kahan_add3(vec3f& sum, vec3f& c, const vec3f& x) {
  const vec3f y = wgsl::vsub(x, c);
  const vec3f t = wgsl::vadd(sum, y);
  c = wgsl::vsub(wgsl::vsub(t, sum), y);
  sum = t;
}

// (((k1 + 2 k2) + 2 k3) + k4) / 6, the RK4 average in the shader's order
__device__ __forceinline__ vec3f rk4_combine(const vec3f& k1, const vec3f& k2, const vec3f& k3,
                                             const vec3f& k4) {
  const vec3f s = wgsl::vadd(wgsl::vmadd(k3, 2.0f, wgsl::vmadd(k2, 2.0f, k1)), k4);
#if defined(LINON_PRECISE)
  return s / 6.0f;
#else
  return wgsl::vscale(s, 1.0f / 6.0f);
#endif
}

// Is the ray still marching?  (loop condition of main_view.wgsl:244, or the
// fixed step budget, or the first hit with stop_on_hit)
// LOOP: 0 decided at run time, 1 fixed step budget, 2 the t-loop.
template <int LOOP = 0>
__device__ __forceinline__ bool ray_active(const RayState& r, const DevMarch& m) {
  if (m.stop_on_hit && r.has_color) return false;
  if (LOOP == 1) return r.steps < m.max_steps;
  if (LOOP == 2) return r.t <= m.t_max;
  if (m.max_steps > 0) return r.steps < m.max_steps;
  return r.t <= m.t_max;
}

// Variant bits of the specialised march kernels (one NVRTC kernel per used
// combination): adaptive refinement, Kahan sums, fixed step budget (with it
// the compiler drops the time accumulator when the field ignores t), and
// field_weight == 1 in fast modules (the blend is then dir = v, identical
// for finite directions).  V_PAIRS: two rays per thread (march_pair_kernel).
enum { V_ADAPTIVE = 1, V_KAHAN = 2, V_STEPS = 4, V_W1 = 8, V_PAIRS = 16 };

// The segment [p, p + step_dir) of a ray that has not hit yet and whose end
// left its safe ball: the intersection test (ray_color, main_view.wgsl:
// 177-220, through the candidate lists or the BVH), the shading of a hit, and
// a new safe ball around the segment's end (or, close to geometry, plain
// tests for the next 8 segments).
template <bool PAIR>
__device__ __forceinline__ void segment_test(const SceneView& sc, const vec3f& p, const vec3f& step_dir,
                                             const vec3f& seg_end, bool& has_color, wgsl::vec4f& color,
                                             int& face, vec3f& q0, float& safe2, int& cool, int* err) {
  const float len = wgsl::length(step_dir);
#if defined(LINON_PRECISE)
  const vec3f dirn = step_dir / len;
#else
  const vec3f dirn = wgsl::normalize(step_dir);
#endif
  HitRec hit = intersect_segment_cells<PAIR>(sc, p, dirn, len, seg_end, err);
  if (hit.t > 0.0f && hit.t < len) {
    color = shade_hit(sc, hit, dirn);
    has_color = color.w > 0.0f;
    if (has_color) face = hit.id;
  }
  safe2 = -1.0f;
  if (!has_color && sc.n_nodes > 0) {
    if (cool > 0) {
      cool--;
    } else {
      // a new ball around the segment's end, where the next one starts
      const float b = safe_radius(sc, seg_end);
      q0 = seg_end;
      safe2 = b * b;
      // close to geometry the ball buys little: test plainly for a while
      if (b < 4.0f * len) cool = 8;
    }
  }
}

// One attempted RK4 step (main_view.wgsl:245-270).  Returns false when the
// step was rejected by the adaptive rule (h refined, nothing advanced).
// PAIR: the BVH walk of intersect_segment (child-pair for the batched
// kernels, which read large scenes through L1).
template <bool ADAPTIVE, bool KAHAN, bool W1 = false, bool PAIR = false, class F>
__device__ __forceinline__ bool ray_step(RayState& r, const F& field, const DevMarch& m,
                                         const SceneView& sc, int* err) {
  const float h = r.h;
  const float hh = 0.5f * h;
  const vec3f k1 = field(r.p, r.p, r.v0, r.dir, r.t);
  // The stage positions stay scalar (FMA-contracted) so that the compiler
  // drops the components a field never reads (the three 1080p frames: 62.2
  // ms scalar, 62.9 ms packed).
  const vec3f k2 = field(r.p, r.p + hh * k1, r.v0, k1, r.t + hh);
  const vec3f k3 = field(r.p, r.p + hh * k2, r.v0, k2, r.t + hh);
  const vec3f k4 = field(r.p, r.p + h * k3, r.v0, k3, r.t + h);
  const vec3f v = rk4_combine(k1, k2, k3, k4);
  float diff = 0.0f;
  if (ADAPTIVE) {
    diff = wgsl::length(v - r.last_v);
    if (r.last_diff >= 0.0f && diff > 10.0f * r.last_diff && h > m.h_fine_above) {
      r.h = m.h_fine;
      return false;
    }
  }
  if (W1) {
    r.dir = v;
  } else {
    const float w = m.field_weight;
    r.dir = wgsl::vmadd(v, w, (1.0f - w) * r.dir);
  }
  const vec3f step_dir = wgsl::vscale(r.dir, h);
  // Safe-ball skip: every point within the ball of radius sqrt(safe2) around
  // q0 is farther than the culling margin from every triangle, and a
  // segment whose ends both lie in the ball lies in it (the ball is convex;
  // the start was checked by the previous step), so such a segment cannot
  // hit anything the brute-force loop would hit.  After the first hit
  // nothing is tested; before it, safe2 = -1 on scenes without a BVH makes
  // every segment fail the one test (no scene constant is read on this
  // path), and a NaN distance fails it too, as a segment leaving the ball
  // does.
  if (!r.has_color) {
    const vec3f seg_end = wgsl::vadd(r.p, step_dir);
    const vec3f dq = wgsl::vsub(seg_end, r.q0);
    if (!(wgsl::dot(dq, dq) <= r.safe2))
      segment_test<PAIR>(sc, r.p, step_dir, seg_end, r.has_color, r.color, r.face, r.q0, r.safe2, r.cool, err);
  }
  if (KAHAN) {
    kahan_add3(r.p, r.cp, step_dir);
    kahan_add(r.t, r.ct, h);
  } else {
    r.p = wgsl::vadd(r.p, step_dir);
    r.t = r.t + h;
  }
  if (ADAPTIVE) {
    r.last_v = v;
    if (2.0f * diff < r.last_diff && h < m.h_initial) r.h = m.h_initial;
    r.last_diff = diff;
  }
  r.steps++;
  return true;
}

// Final stores of main_view.wgsl:373-374 (alpha forced to 1, wgsl:274-277).
__device__ __forceinline__ void ray_store(const RayState& r, const DevFrame& f, size_t idx) {
  if (f.color) {
    uchar4 c;
    if (r.has_color) {
      c.x = unorm8(r.color.x);
      c.y = unorm8(r.color.y);
      c.z = unorm8(r.color.z);
    } else {
      c.x = c.y = c.z = 0;
    }
    c.w = 255;
    f.color[idx] = c;
  }
  if (f.mapping) f.mapping[idx] = make_float4(r.p.x, r.p.y, r.p.z, 1.0f);
  if (f.hit) f.hit[idx] = r.has_color ? r.face : -1;
  if (f.steps) f.steps[idx] = r.steps;
}

// --------------------------------------------------------------------------
// Shared-memory staging of small scenes with one TMA bulk copy
// (cp.async.bulk global -> shared, completion on an mbarrier).  The wait is
// bounded: after the budget the kernel flags LINON error bit 1, waits once
// more (bounded) for its own copy, and falls back to global memory.
// --------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned phase) {
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(phase)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned phase, int budget) {
  for (int i = 0; i < budget; ++i)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}

// Copies `bytes` (multiple of 16, both pointers 16-byte aligned) into smem.
// All threads of the CTA call it; returns true when the copy is usable.
__device__ __forceinline__ bool stage_to_smem(void* smem, const void* gmem, unsigned bytes,
                                              unsigned long long* mbar, int* err) {
  const unsigned bar = smem_addr(mbar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(smem)),
        "l"(gmem), "r"(bytes), "r"(bar)
        : "memory");
  }
  bool ok = mbar_wait_bounded(bar, 0, 1 << 20);
  if (!ok) {
    atomicOr(err, 1);
    ok = mbar_wait_bounded(bar, 0, 1 << 22);
  }
  // every thread must agree before the smem copy is used
  ok = __syncthreads_and(ok ? 1 : 0) != 0;
  return ok;
}

// Sets up the scene view of a CTA: small scenes come from shared memory.
__device__ __forceinline__ SceneView cta_scene(const DevScene& s, float4* smem,
                                               unsigned long long* mbar, int* err) {
  SceneView v;
  v.tris = s.tris;
  v.nodes = s.nodes;
  v.face_rgb = s.face_rgb;
  v.n_tris = s.n_tris;
  v.n_nodes = s.n_nodes;
  v.margin = s.margin;
  v.grid = s.grid;
  v.cells = s.cells;
  v.cell_tris = s.cell_tris;
  v.reach = s.reach;
  v.gx = s.gx;
  v.gy = s.gy;
  v.gz = s.gz;
  v.gox = s.gox;
  v.goy = s.goy;
  v.goz = s.goz;
  v.gcell = s.gcell;
  v.ginv = s.ginv;
  if (s.staged_bytes > 0) {
    // staged block = [nodes | tris] contiguous in global memory
    if (stage_to_smem(smem, s.staged, (unsigned)s.staged_bytes, mbar, err)) {
      v.nodes = smem;
      v.tris = smem + 2 * s.n_nodes;
    }
  }
  return v;
}

// --------------------------------------------------------------------------
// Kernels (instantiated per field by the generated module)
// --------------------------------------------------------------------------

// One thread per pixel; the CTA covers a tile_w x tile_h pixel tile.
// V: variant bits (V_ADAPTIVE | V_KAHAN | V_STEPS | V_W1).
template <int V, class F>
__device__ __forceinline__ void march_plain_kernel(const F& field, const MarchArgs& a) {
  constexpr bool ADAPTIVE = (V & V_ADAPTIVE) != 0;
  constexpr bool KAHAN = (V & V_KAHAN) != 0;
  constexpr int LOOP = (V & V_STEPS) ? 1 : 2;
#if defined(LINON_PRECISE)
  constexpr bool W1 = false;  // op-for-op modules keep the shader's blend
#else
  constexpr bool W1 = (V & V_W1) != 0;
#endif
  extern __shared__ float4 linon_smem[];
  __shared__ unsigned long long mbar;
  const SceneView sc = cta_scene(a.scene, linon_smem, &mbar, a.err);
  const int W = a.frame.W, H = a.frame.H;
  const int lx = threadIdx.x % a.tile_w, ly = threadIdx.x / a.tile_w;
  const int x = blockIdx.x * a.tile_w + lx;
  const int row = a.row0 + blockIdx.y * a.tile_h + ly;
  // Threads outside the image stay in the warp as idle lanes (no early
  // exit) so that the per-step warp vote below always names all 32 lanes.
  const bool in_image = x < W && row < a.row1;
  const int gy = H - 1 - row;
  const Basis b = make_basis(a.cam, W, H, a.m.focal_length, a.m.viewport_height);
  const vec3f dir = primary_dir(b, in_image ? x : 0, in_image ? gy : 0);
  const size_t idx = in_image ? size_t(row) * W + x : 0;
  RayState r;
  ray_init(r, b.origin, dir, a.m.h_initial);
  if (a.m.linear_mode) {  // main_view.wgsl:368-370
    if (!in_image) return;
    HitRec hit = intersect_segment(sc, b.origin, dir, 100.0f, b.origin + 100.0f * dir, a.err);
    wgsl::vec4f c(0.0f, 0.0f, 0.0f, 0.0f);
    if (hit.t > 0.0f && hit.t < 100.0f) c = shade_hit(sc, hit, dir);
    if (a.frame.color) {
      uchar4 o;
      o.x = unorm8(c.x); o.y = unorm8(c.y); o.z = unorm8(c.z); o.w = unorm8(c.w);
      a.frame.color[idx] = o;
    }
    if (a.frame.hit) a.frame.hit[idx] = hit.t > 0.0f && hit.t < 100.0f ? hit.id : -1;
    if (a.frame.mapping) a.frame.mapping[idx] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (a.frame.steps) a.frame.steps[idx] = 0;
    return;
  }
#if !defined(LINON_VOTE_LOOP)
  if ((V & V_STEPS) && !ADAPTIVE && !a.m.stop_on_hit) {
    // Fixed step budget without adaptive retries or early stop: every lane
    // takes exactly max_steps steps (lanes outside the image march pixel
    // (0, 0)'s ray and store nothing), so the trip count is the same for the
    // whole warp and no vote is needed; __syncwarp after each step
    // reconverges lanes that diverged at an intersection test.
    // One copy of the step in the loop: the step inlines the BVH traversal,
    // and a second copy (unrolling, a remainder loop) costs more in
    // instruction-cache misses than it saves.
    for (int s = 0; s < a.m.max_steps; ++s) {
      ray_step<ADAPTIVE, KAHAN, W1>(r, field, a.m, sc, a.err);
      __syncwarp();
    }
    if (in_image) ray_store(r, a.frame, idx);
    return;
  }
#endif
  // The vote at the top of every step reconverges the warp: without it the
  // lanes that diverged at a (rare) intersection test would walk the rest of
  // the march separately, a few lanes per issued instruction.
  bool active = in_image && ray_active<LOOP>(r, a.m);
  while (__any_sync(0xffffffffu, active)) {
    if (active) {
      ray_step<ADAPTIVE, KAHAN, W1>(r, field, a.m, sc, a.err);
      active = ray_active<LOOP>(r, a.m);
    }
  }
  if (in_image) ray_store(r, a.frame, idx);
}

#if defined(LINON_PAIRS) && defined(LINON_F32X2)
// --------------------------------------------------------------------------
// Two rays per thread: the fixed-step march (no adaptive retries, no stop at
// the first hit) of two horizontally adjacent pixels, their arithmetic
// issued as packed FP32 pairs (wgsl::f2) with the field function emitted in
// pair form.  Per pair of rays the thread issues the field evaluations, the
// RK4 average, the step, the safe-ball test and the Kahan sums once instead
// of twice, and the loop and reconvergence bookkeeping once; the march is
// issue-bound in one-ray form (twist, linear) or close to it (lens).  Each
// operation rounds like the one-ray fast kernel's, whose multiply-adds the
// compiler contracts where these are written as packed FMAs.  The segment
// test of a ray that left its safe ball runs on that ray's values alone
// (segment_test, as in ray_step); a hit's colour and face are stored at
// once, so no shading state is carried through the loop.  The CTA covers
// tile_w x tile_h pixels with tile_w / 2 x tile_h threads.
// --------------------------------------------------------------------------
using wgsl::f2;
using wgsl::vec3p;

__device__ __forceinline__ vec3p pack_pair(const vec3f& a, const vec3f& b) {
  return vec3p(f2(a.x, b.x), f2(a.y, b.y), f2(a.z, b.z));
}
__device__ __forceinline__ vec3f pair_lane(const vec3p& v, int k) {
  return k ? vec3f(v.x.v.y, v.y.v.y, v.z.v.y) : vec3f(v.x.v.x, v.y.v.x, v.z.v.x);
}
__device__ __forceinline__ void kahan_add_pair(f2& sum, f2& c, f2 x) {
  const f2 y = x - c;
  const f2 t = sum + y;
  c = (t - sum) - y;
  sum = t;
}

template <int V, class F>
__device__ __forceinline__ void march_pair_kernel(const F& field, const MarchArgs& a) {
  constexpr bool KAHAN = (V & V_KAHAN) != 0;
  constexpr bool W1 = (V & V_W1) != 0;
  extern __shared__ float4 linon_smem[];
  __shared__ unsigned long long mbar;
  // The scene view lives in shared memory: only the (rare) segment test
  // reads it, and the march keeps its registers for the two rays (96
  // registers without spills, 5 CTAs per SM: the 1080p lens frame 28.02 ->
  // 27.63 ms against the view in registers, 80 registers with spills).
  __shared__ SceneView scene_sh;
  {
    const SceneView v = cta_scene(a.scene, linon_smem, &mbar, a.err);
    if (threadIdx.x == 0) scene_sh = v;
    __syncthreads();
  }
  const SceneView& sc = scene_sh;
  const int W = a.frame.W, H = a.frame.H;
  const int pairs_w = a.tile_w / 2;
  const int lx = threadIdx.x % pairs_w, ly = threadIdx.x / pairs_w;
  const int x0 = blockIdx.x * a.tile_w + 2 * lx;
  const int row = a.row0 + blockIdx.y * a.tile_h + ly;
  // lanes outside the image march pixel (0, 0)'s ray and store nothing
  const bool in0 = x0 < W && row < a.row1, in1 = x0 + 1 < W && row < a.row1;
  const int gy = H - 1 - row;
  const Basis b = make_basis(a.cam, W, H, a.m.focal_length, a.m.viewport_height);
  const vec3f d0 = primary_dir(b, in0 ? x0 : 0, in0 ? gy : 0);
  const vec3f d1 = primary_dir(b, in1 ? x0 + 1 : 0, in1 ? gy : 0);
  const size_t idx0 = in0 ? size_t(row) * W + x0 : 0, idx1 = idx0 + 1;
  vec3p p = pack_pair(b.origin, b.origin), dir = pack_pair(d0, d1);
  const vec3p v0 = dir;
  vec3p cp(f2(0.0f), f2(0.0f), f2(0.0f));
  f2 t(0.0f), ct(0.0f);
  const f2 h(a.m.h_initial), hh(0.5f * a.m.h_initial);
  vec3p q0 = p;
  f2 safe2(-1.0f);
  bool has0 = false, has1 = false;
  int cool0 = 0, cool1 = 0;
  for (int s = 0; s < a.m.max_steps; ++s) {
    const vec3p k1 = field(p, p, v0, dir, t);
    const vec3p k2 = field(p, vec3p(p + hh * k1), v0, k1, t + hh);
    const vec3p k3 = field(p, vec3p(p + hh * k2), v0, k2, t + hh);
    const vec3p k4 = field(p, vec3p(p + h * k3), v0, k3, t + h);
    // (((k1 + 2 k2) + 2 k3) + k4) / 6, as rk4_combine
    const vec3p sum = (vec3p(k1 + f2(2.0f) * k2) + f2(2.0f) * k3) + k4;
    const vec3p v = sum * f2(1.0f / 6.0f);
    if (W1) {
      dir = v;
    } else {
      const f2 w(a.m.field_weight);
      dir = vec3p((f2(1.0f) - w) * dir) + v * w;
    }
    const vec3p step_dir = dir * h;
    // The new position first (with Kahan sums: the compensated sum, which
    // lies within rounding of p + step_dir); the safe-ball test reads it, so
    // the segment end is formed only for a lane that is tested.
    vec3p ky, pn;
    if (KAHAN) {
      ky = step_dir - cp;
      pn = p + ky;
    } else {
      pn = p + step_dir;
    }
    if (!(has0 && has1)) {
      const vec3p dq = pn - q0;
      const f2 d2 = wgsl::dot(dq, dq);
      const bool need0 = !has0 && !(d2.v.x <= safe2.v.x);
      const bool need1 = !has1 && !(d2.v.y <= safe2.v.y);
      if (need0 || need1) {
#pragma unroll 1
        for (int k = 0; k < 2; ++k) {
          if (!(k ? need1 : need0)) continue;
          bool has = false;
          wgsl::vec4f color(0.0f, 0.0f, 0.0f, 0.0f);
          int face = -1;
          vec3f q = pair_lane(q0, k);
          float sf = k ? safe2.v.y : safe2.v.x;
          int cool = k ? cool1 : cool0;
          const vec3f pk = pair_lane(p, k), sk = pair_lane(step_dir, k);
          segment_test<false>(sc, pk, sk, wgsl::vadd(pk, sk), has, color, face, q, sf, cool, a.err);
          if (has && (k ? in1 : in0)) {  // the first hit decides the pixel's colour and face
            const size_t idx = k ? idx1 : idx0;
            if (a.frame.color) {
              uchar4 c;
              c.x = unorm8(color.x);
              c.y = unorm8(color.y);
              c.z = unorm8(color.z);
              c.w = 255;
              a.frame.color[idx] = c;
            }
            if (a.frame.hit) a.frame.hit[idx] = face;
          }
          if (k) {
            has1 = has;
            cool1 = cool;
            q0.x.v.y = q.x; q0.y.v.y = q.y; q0.z.v.y = q.z;
            safe2.v.y = sf;
          } else {
            has0 = has;
            cool0 = cool;
            q0.x.v.x = q.x; q0.y.v.x = q.y; q0.z.v.x = q.z;
            safe2.v.x = sf;
          }
        }
      }
    }
    if (KAHAN) {
      cp = vec3p(pn - p) - ky;
      p = pn;
      kahan_add_pair(t, ct, h);
    } else {
      p = pn;
      t = t + h;
    }
    __syncwarp();
  }
  // final stores of main_view.wgsl:373-374 (a hit's colour was stored above)
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    if (!(k ? in1 : in0)) continue;
    const size_t idx = k ? idx1 : idx0;
    const bool has = k ? has1 : has0;
    if (!has) {
      if (a.frame.color) a.frame.color[idx] = make_uchar4(0, 0, 0, 255);
      if (a.frame.hit) a.frame.hit[idx] = -1;
    }
    const vec3f e = pair_lane(p, k);
    if (a.frame.mapping) a.frame.mapping[idx] = make_float4(e.x, e.y, e.z, 1.0f);
    if (a.frame.steps) a.frame.steps[idx] = a.m.max_steps;
  }
}
#endif  // LINON_PAIRS

// --------------------------------------------------------------------------
// Persistent batched march: many views of uneven size, camera, step size and
// field in one launch, fed by a device work queue (persistent "while-while"
// ray scheduling, Aila & Laine 2009).  Each warp is bound to one view at a
// time, so the view's march parameters, camera and field are uniform across
// the warp: the field is chosen once per quantum, the camera basis is set up
// once per binding (in shared memory) and no lane carries per-view state.
// The queue is one counter per view (BatchView::next) over its rays in
// tile_w x tile_h tiles of 32 (consecutive rays are image neighbours).  A
// warp marches `quantum` RK4 steps at a time, retires finished rays (storing
// their pixels) and refills its free lanes from its view when fewer than
// refill_below lanes are still marching (or when it is empty); once the view
// has no rays left the warp finishes its lanes and binds to the next view
// that has some (views are queued with the largest step budget first, and
// counter[0] holds the first view that may still have rays).  Warps exit
// when every view is drained and their lanes are done.
// --------------------------------------------------------------------------
// linear_mode's one straight segment per pixel (main_view.wgsl:368-370).
__device__ __forceinline__ void linear_shot(const SceneView& sc, const vec3f& origin, const vec3f& dir,
                                            const DevFrame& out, size_t idx, int* err) {
  HitRec hit = intersect_segment<true>(sc, origin, dir, 100.0f, origin + 100.0f * dir, err);
  wgsl::vec4f c(0.0f, 0.0f, 0.0f, 0.0f);
  if (hit.t > 0.0f && hit.t < 100.0f) c = shade_hit(sc, hit, dir);
  if (out.color) {
    uchar4 o;
    o.x = unorm8(c.x); o.y = unorm8(c.y); o.z = unorm8(c.z); o.w = unorm8(c.w);
    out.color[idx] = o;
  }
  if (out.hit) out.hit[idx] = hit.t > 0.0f && hit.t < 100.0f ? hit.id : -1;
  if (out.mapping) out.mapping[idx] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (out.steps) out.steps[idx] = 0;
}

template <class F>
__device__ __forceinline__ void ray_step_rt(RayState& r, const F& field, const DevMarch& m,
                                            const SceneView& sc, int* err) {
  if (m.adaptive) {
    if (m.kahan) ray_step<true, true, false, true>(r, field, m, sc, err);
    else ray_step<true, false, false, true>(r, field, m, sc, err);
  } else {
    if (m.kahan) ray_step<false, true, false, true>(r, field, m, sc, err);
    else ray_step<false, false, false, true>(r, field, m, sc, err);
  }
}

__device__ __forceinline__ long long view_rays(const BatchArgs& a, int v) {
  return (v + 1 < a.n_views ? a.views[v + 1].ray_begin : a.total_rays) - a.views[v].ray_begin;
}

// First view at or after counter[0] whose queue is not drained (-1: none);
// drained views at the front advance counter[0].
__device__ __forceinline__ int next_open_view(const BatchArgs& a) {
  volatile unsigned long long* cursor = a.counter;
  int v = int(*cursor);
  for (; v < a.n_views; ++v) {
    const volatile unsigned long long* nx = &a.views[v].next;
    if ((long long)*nx < view_rays(a, v)) break;
    atomicMax(a.counter, (unsigned long long)(v + 1));
  }
  return v < a.n_views ? v : -1;
}

// MODE: 0 any views (the step variant is chosen per view at run time); 1
// every view has a fixed step budget without Kahan sums; 2 the same with
// Kahan sums.  The specialised modes carry no adaptive-step or unused-sum
// state.
#ifndef LINON_BATCH_MAX_WARPS
#define LINON_BATCH_MAX_WARPS 8  // 256-thread CTAs at most (LINON_BATCH_BOUNDS)
#endif
template <int MODE = 0, class Fields>
__device__ __forceinline__ void march_batch_kernel(const Fields& fields, const BatchArgs& a) {
  extern __shared__ float4 linon_smem[];
  __shared__ unsigned long long mbar;
  // each warp's camera basis of its bound view (raw storage: Basis has
  // constructors, which a __shared__ variable may not run)
  __shared__ __align__(16) unsigned char warp_basis[LINON_BATCH_MAX_WARPS * sizeof(Basis)];
  const SceneView sc = cta_scene(a.scene, linon_smem, &mbar, a.err);
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  Basis& wb = reinterpret_cast<Basis*>(warp_basis)[threadIdx.x >> 5];
  RayState r;
  unsigned pix = 0;  // row * W + x (images hold at most 2^31 - 1 pixels)
  bool active = false;
  int view = -1;           // warp-uniform: the bound view
  bool view_open = false;  // warp-uniform: the bound view may still have rays
  for (;;) {
    unsigned act = __ballot_sync(FULL, active);
    // ---- bind the next view with rays when the warp is empty ----
    if (act == 0u && !view_open) {
      view = 0;
      if (lane == 0) view = next_open_view(a);
      view = __shfl_sync(FULL, view, 0);
      if (view < 0) break;
      view_open = true;
      __syncwarp();  // every lane is done with the previous view's basis
      if (lane == 0) {
        const BatchView& V = a.views[view];
        wb = make_basis(V.cam, V.frame.W, V.frame.H, V.m.focal_length, V.m.viewport_height);
      }
      __syncwarp();
    }
    const BatchView& V = a.views[view];
    const DevMarch m = V.m;
    // ---- refill free lanes from the bound view ----
    if (view_open && (act == 0u || __popc(act) < a.refill_below)) {
      const int nfree = 32 - __popc(act);
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(&a.views[view].next, (unsigned long long)nfree);
      base = __shfl_sync(FULL, base, 0);
      const long long n_rays = view_rays(a, view);
      if ((long long)(base + nfree) >= n_rays) view_open = false;
      if (!active) {
        const long long local = (long long)base + __popc(~act & ((1u << lane) - 1));
        if (local < n_rays) {
          const int tile = int(local / (a.tile_w * a.tile_h));
          const int within = int(local % (a.tile_w * a.tile_h));
          const int x = (tile % V.tiles_x) * a.tile_w + within % a.tile_w;
          const int row = (tile / V.tiles_x) * a.tile_h + within / a.tile_w;
          if (x < V.frame.W && row < V.frame.H) {
            pix = unsigned(row) * unsigned(V.frame.W) + unsigned(x);
            ray_init(r, wb.origin, primary_dir(wb, x, V.frame.H - 1 - row), m.h_initial);
            active = true;
            if (m.linear_mode) {
              linear_shot(sc, wb.origin, r.dir, V.frame, pix, a.err);
              active = false;
            }
          }
        }
      }
      act = __ballot_sync(FULL, active);
    }
    if (act == 0u) continue;  // nothing to march: refill again or bind the next view
    // ---- march a quantum with the view's field (uniform across the warp);
    //      a warp whose view still has rays leaves early to refill once
    //      fewer than refill_below lanes are marching ----
    fields.visit(V.field, [&](const auto& field) {
      for (int q = 0; q < a.quantum; ++q) {
        const bool go = active && ray_active(r, m);
        const unsigned g = __ballot_sync(FULL, go);
        if (g == 0u || (view_open && __popc(g) < a.refill_below)) break;
        if (go) {
          if (MODE == 0) ray_step_rt(r, field, m, sc, a.err);
          else ray_step<false, MODE == 2, false, true>(r, field, m, sc, a.err);
        }
      }
    });
    if (active && !ray_active(r, m)) {
      ray_store(r, V.frame, pix);
      active = false;
    }
  }
}

// Persistent queue of ray tiles, one tile per warp: a warp takes the next
// tile_w x tile_h tile of 32 rays from the first view that has tiles left
// (views with the largest step budget first), marches it to the end with the
// plain kernel's loop (per-step warp vote) and takes the next.  Unlike the
// lane-refilling queue above no lane carries queue state through the march,
// and unlike one CTA per tile a warp whose rays end early does not wait for
// the other warps of its CTA: it takes the next tile at once.
__device__ __forceinline__ int take_tile(const BatchArgs& a, unsigned long long& base) {
  int v = int(*(volatile unsigned long long*)a.counter);
  for (; v < a.n_views; ++v) {
    const long long n = view_rays(a, v);
    if ((long long)*(volatile unsigned long long*)&a.views[v].next < n) {
      const unsigned long long b = atomicAdd(&a.views[v].next, 32ull);
      if ((long long)b < n) {
        base = b;
        return v;
      }
    }
    atomicMax(a.counter, (unsigned long long)(v + 1));  // view v is drained
  }
  return -1;
}

template <int MODE = 0, class Fields>
__device__ __forceinline__ void march_queue_kernel(const Fields& fields, const BatchArgs& a) {
  extern __shared__ float4 linon_smem[];
  __shared__ unsigned long long mbar;
  const SceneView sc = cta_scene(a.scene, linon_smem, &mbar, a.err);
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long base = 0;
    int view = 0;
    if (lane == 0) view = take_tile(a, base);
    view = __shfl_sync(FULL, view, 0);
    if (view < 0) break;
    base = __shfl_sync(FULL, base, 0);
    const BatchView& V = a.views[view];
    const int tile = int(base >> 5);  // ray_begin and the queue advance in whole tiles of 32
    // tile_w divides 32, so it is a power of two
    const int x = (tile % V.tiles_x) * a.tile_w + (lane & (a.tile_w - 1));
    const int row = (tile / V.tiles_x) * a.tile_h + (lane >> (__ffs(a.tile_w) - 1));
    const int W = V.frame.W, H = V.frame.H;
    const bool in_image = x < W && row < H;
    const DevMarch m = V.m;
    const Basis b = make_basis(V.cam, W, H, m.focal_length, m.viewport_height);
    const vec3f dir = primary_dir(b, in_image ? x : 0, in_image ? H - 1 - row : 0);
    const size_t idx = in_image ? size_t(row) * W + x : 0;
    RayState r;
    ray_init(r, b.origin, dir, m.h_initial);
    if (m.linear_mode) {
      if (in_image) linear_shot(sc, b.origin, dir, V.frame, idx, a.err);
      continue;
    }
    fields.visit(V.field, [&](const auto& field) {
      bool active = in_image && ray_active(r, m);
      while (__any_sync(FULL, active)) {
        if (active) {
          if (MODE == 0) ray_step_rt(r, field, m, sc, a.err);
          else ray_step<false, MODE == 2, false, true>(r, field, m, sc, a.err);
          active = ray_active(r, m);
        }
      }
    });
    if (in_image) ray_store(r, V.frame, idx);
  }
}

// The other batched form: one launch, one 8 x 16-pixel CTA per tile of every
// view (views' tiles concatenated, views with the largest step budget
// first), the hardware's block scheduler balancing the load.  Each CTA's
// view, march parameters and field are uniform; the march is the plain
// kernel's (per-step warp vote, rays stop on their own budget or hit).
__device__ __forceinline__ int find_view_block(const BatchArgs& a, int block) {
  int lo = 0, hi = a.n_views - 1;  // last view with block_begin <= block
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (a.views[mid].block_begin <= block) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// One 8 x 16-pixel tile (tile number `block` of the concatenated views) by
// a 128-thread CTA.
template <int MODE, class Fields>
__device__ __forceinline__ void march_tile_block(const Fields& fields, const BatchArgs& a, const SceneView& sc,
                                                 int block) {
  const int view = find_view_block(a, block);
  const BatchView& V = a.views[view];
  const int local = block - V.block_begin;
  const int x = (local % V.blocks_x) * 8 + int(threadIdx.x % 8);
  const int row = (local / V.blocks_x) * 16 + int(threadIdx.x / 8);
  const int W = V.frame.W, H = V.frame.H;
  const bool in_image = x < W && row < H;
  const DevMarch m = V.m;
  const Basis b = make_basis(V.cam, W, H, m.focal_length, m.viewport_height);
  const vec3f dir = primary_dir(b, in_image ? x : 0, in_image ? H - 1 - row : 0);
  const size_t idx = in_image ? size_t(row) * W + x : 0;
  RayState r;
  ray_init(r, b.origin, dir, m.h_initial);
  if (m.linear_mode) {
    // (written out here rather than through linear_shot: the call changes
    // this kernel's register allocation, 64 uneven views 10.8 -> 11.2 ms)
    if (!in_image) return;
    HitRec hit = intersect_segment<true>(sc, b.origin, dir, 100.0f, b.origin + 100.0f * dir, a.err);
    wgsl::vec4f c(0.0f, 0.0f, 0.0f, 0.0f);
    if (hit.t > 0.0f && hit.t < 100.0f) c = shade_hit(sc, hit, dir);
    const DevFrame& out = V.frame;
    if (out.color) {
      uchar4 o;
      o.x = unorm8(c.x); o.y = unorm8(c.y); o.z = unorm8(c.z); o.w = unorm8(c.w);
      out.color[idx] = o;
    }
    if (out.hit) out.hit[idx] = hit.t > 0.0f && hit.t < 100.0f ? hit.id : -1;
    if (out.mapping) out.mapping[idx] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (out.steps) out.steps[idx] = 0;
    return;
  }
  // The CTA's field is chosen once: the march loop is instantiated per field
  // (no field switch in the four evaluations of every step; 64 uneven views
  // 14.3 -> 12.0 ms).
  fields.visit(V.field, [&](const auto& field) {
    bool active = in_image && ray_active(r, m);
    while (__any_sync(0xffffffffu, active)) {
      if (active) {
        if (MODE == 0) ray_step_rt(r, field, m, sc, a.err);
        else ray_step<false, MODE == 2, false, true>(r, field, m, sc, a.err);
        active = ray_active(r, m);
      }
    }
  });
  if (in_image) ray_store(r, V.frame, idx);
}

template <int MODE = 0, class Fields>
__device__ __forceinline__ void march_multi_kernel(const Fields& fields, const BatchArgs& a) {
  extern __shared__ float4 linon_smem[];
  __shared__ unsigned long long mbar;
  const SceneView sc = cta_scene(a.scene, linon_smem, &mbar, a.err);
  march_tile_block<MODE>(fields, a, sc, int(blockIdx.x));
}

// Persistent queue of CTA tiles: one CTA per resident slot marches the
// 8 x 16-pixel tile of its own index first (the one-CTA-per-tile schedule's
// tiles and order), then takes the next tile from a device counter (which
// starts past the grid's first tiles), until the counter passes the last
// tile.  Thread 0 takes the next tile when its own rays of the current one
// are done; two slots for the taken index leave one barrier per tile.
template <int MODE = 0, class Fields>
__device__ __forceinline__ void march_tileq_kernel(const Fields& fields, const BatchArgs& a) {
  extern __shared__ float4 linon_smem[];
  __shared__ unsigned long long mbar;
  __shared__ int next_tile[2];
  const SceneView sc = cta_scene(a.scene, linon_smem, &mbar, a.err);
  int block = int(blockIdx.x), slot = 0;
  while (block < a.n_blocks) {
    march_tile_block<MODE>(fields, a, sc, block);
    if (threadIdx.x == 0) next_tile[slot] = int(gridDim.x + atomicAdd(a.counter, 1ull));
    // the slot written here was last read before the previous barrier
    __syncthreads();
    block = next_tile[slot];
    slot ^= 1;
  }
}

// sample_rays generalised: one thread per ray; out[ray][point] float4.
template <class F>
__device__ __forceinline__ void capture_kernel(const F& field, const CaptureArgs& a) {
  const int ray = blockIdx.x * blockDim.x + threadIdx.x;
  if (ray >= a.n_rays) return;
  const Basis b = make_basis(a.cam, a.W, a.H, a.focal_length, a.viewport_height);
  const vec3f start_dir = position_dir(b, a.pos[2 * ray], a.pos[2 * ray + 1]);
  vec3f p = b.origin, dir = start_dir;
  float t = 0.0f;
  const float h = a.h, hh = 0.5f * a.h, w = a.field_weight;
  float4* out = a.out + size_t(ray) * a.n_points;
  int until = 0, slot = 0;  // steps before the next recorded point (every `every` steps from 0), its slot
  for (int i = 0; i < a.n_steps; ++i) {
    const vec3f k1 = field(p, p, start_dir, dir, t);
    const vec3f k2 = field(p, p + hh * k1, start_dir, k1, t + hh);
    const vec3f k3 = field(p, p + hh * k2, start_dir, k2, t + hh);
    const vec3f k4 = field(p, p + h * k3, start_dir, k3, t + h);
    const vec3f v = rk4_combine(k1, k2, k3, k4);
    dir = wgsl::vmadd(v, w, (1.0f - w) * dir);
    const vec3f step_dir = wgsl::vscale(dir, h);
    if (until == 0) {
      out[slot++] = make_float4(p.x, p.y, p.z, 1.0f);
      until = a.every;
    }
    --until;
    p = wgsl::vadd(p, step_dir);
    t = t + h;
  }
  if (a.record_final) out[a.n_points - 1] = make_float4(p.x, p.y, p.z, 1.0f);
}

// Field evaluation at listed inputs (13 floats each) for front-end tests.
template <class F>
__device__ __forceinline__ void field_eval_kernel(const F& field, const float* in, float* out,
                                                  int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* q = in + 13 * size_t(i);
  vec3f r = field(vec3f(q[0], q[1], q[2]), vec3f(q[3], q[4], q[5]), vec3f(q[6], q[7], q[8]),
                  vec3f(q[9], q[10], q[11]), q[12]);
  out[3 * size_t(i)] = r.x;
  out[3 * size_t(i) + 1] = r.y;
  out[3 * size_t(i) + 2] = r.z;
}

}  // namespace linon
