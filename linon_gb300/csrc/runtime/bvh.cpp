// bvh.cpp — triangle arrays and the BVH behind the segment test.
//
// The reference tests every march segment against every face
// (src/main_view.wgsl:182-198).  The BVH keeps that result: node boxes bound
// the triangles' vertices inflated by a margin far above the FP32 rounding of
// the Moeller-Trumbore arithmetic, so a culled triangle is one the brute-force
// loop cannot hit, and the traversal keeps the lexicographic minimum of
// (t, original face index), which is what the strict `<` of the loop keeps.
// Build: binned SAH (16 bins) on the triangle centroids, leaves of <= 4
// triangles, depth capped below the device traversal stack.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

#include "internal.hpp"

namespace linon {
namespace {

constexpr int kLeafSize = 4;
constexpr int kMaxDepth = 40;  // device stack holds 48 entries
constexpr int kBins = 16;

struct Prim {
  float lo[3], hi[3], c[3];
};

struct Box {
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
  float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  void grow(const float* l, const float* h) {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], l[k]);
      hi[k] = std::max(hi[k], h[k]);
    }
  }
  double area() const {
    double dx = std::max(0.0, double(hi[0]) - lo[0]), dy = std::max(0.0, double(hi[1]) - lo[1]),
           dz = std::max(0.0, double(hi[2]) - lo[2]);
    return 2.0 * (dx * dy + dy * dz + dz * dx);
  }
};

struct Builder {
  std::vector<Prim> prims;
  std::vector<uint32_t> idx;
  std::vector<float4> nodes;
  float margin = 0;
  uint32_t max_depth = 0;

  static float int_bits(int v) {
    float f;
    std::memcpy(&f, &v, 4);
    return f;
  }

  void set_node(size_t n, const Box& b, int first, int count) {
    nodes[2 * n] = make_float4(b.lo[0] - margin, b.lo[1] - margin, b.lo[2] - margin, int_bits(first));
    nodes[2 * n + 1] = make_float4(b.hi[0] + margin, b.hi[1] + margin, b.hi[2] + margin, int_bits(count));
  }

  void build(size_t node, uint32_t begin, uint32_t end, uint32_t depth) {
    max_depth = std::max(max_depth, depth);
    Box b, cb;
    for (uint32_t i = begin; i < end; ++i) {
      const Prim& p = prims[idx[i]];
      b.grow(p.lo, p.hi);
      cb.grow(p.c, p.c);
    }
    const uint32_t count = end - begin;
    if (count <= uint32_t(kLeafSize) || depth >= uint32_t(kMaxDepth)) {
      set_node(node, b, int(begin), int(count));
      return;
    }
    int axis = 0;
    float ext[3];
    for (int k = 0; k < 3; ++k) ext[k] = cb.hi[k] - cb.lo[k];
    if (ext[1] > ext[axis]) axis = 1;
    if (ext[2] > ext[axis]) axis = 2;
    uint32_t mid = begin + count / 2;
    if (ext[axis] > 0.0f) {
      Box bins[kBins];
      uint32_t cnt[kBins] = {0};
      const float scale = float(kBins) / ext[axis];
      auto bin_of = [&](const Prim& p) {
        int k = int((p.c[axis] - cb.lo[axis]) * scale);
        return std::min(kBins - 1, std::max(0, k));
      };
      for (uint32_t i = begin; i < end; ++i) {
        const Prim& p = prims[idx[i]];
        int k = bin_of(p);
        cnt[k]++;
        bins[k].grow(p.lo, p.hi);
      }
      double best = 1e300;
      int best_split = -1;
      for (int s = 1; s < kBins; ++s) {
        Box l, r;
        uint32_t nl = 0, nr = 0;
        for (int k = 0; k < s; ++k)
          if (cnt[k]) { l.grow(bins[k].lo, bins[k].hi); nl += cnt[k]; }
        for (int k = s; k < kBins; ++k)
          if (cnt[k]) { r.grow(bins[k].lo, bins[k].hi); nr += cnt[k]; }
        if (nl == 0 || nr == 0) continue;
        double cost = nl * l.area() + nr * r.area();
        if (cost < best) { best = cost; best_split = s; }
      }
      if (best_split > 0) {
        auto it = std::partition(idx.begin() + begin, idx.begin() + end,
                                 [&](uint32_t i) { return bin_of(prims[i]) < best_split; });
        mid = uint32_t(it - idx.begin());
      }
    }
    if (mid == begin || mid == end) {
      std::nth_element(idx.begin() + begin, idx.begin() + begin + count / 2, idx.begin() + end,
                       [&](uint32_t a, uint32_t c) { return prims[a].c[axis] < prims[c].c[axis]; });
      mid = begin + count / 2;
    }
    const size_t left = nodes.size() / 2;
    nodes.resize(nodes.size() + 4);
    set_node(node, b, int(left), 0);
    build(left, begin, mid, depth + 1);
    build(left + 1, mid, end, depth + 1);
  }
};

float int_bits(int v) {
  float f;
  std::memcpy(&f, &v, 4);
  return f;
}

void push_tri(std::vector<float4>& tris, const float* xyz, const uint32_t* abc, uint32_t f) {
  const float* a = xyz + 3 * size_t(abc[3 * f]);
  const float* b = xyz + 3 * size_t(abc[3 * f + 1]);
  const float* c = xyz + 3 * size_t(abc[3 * f + 2]);
  // edge1 = v1 - v0, edge2 = v2 - v0 exactly as hit_triangle computes them
  const float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
  const float e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
  tris.push_back(make_float4(a[0], a[1], a[2], int_bits(int(f))));
  tris.push_back(make_float4(e1[0], e1[1], e1[2], 0.0f));
  tris.push_back(make_float4(e2[0], e2[1], e2[2], 0.0f));
  // unit plane for conservative culling (double, rounded once); zero for a
  // degenerate or non-finite triangle
  const double n[3] = {double(e1[1]) * e2[2] - double(e1[2]) * e2[1], double(e1[2]) * e2[0] - double(e1[0]) * e2[2],
                       double(e1[0]) * e2[1] - double(e1[1]) * e2[0]};
  const double len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  if (len > 0.0 && std::isfinite(len)) {
    const float nx = float(n[0] / len), ny = float(n[1] / len), nz = float(n[2] / len);
    const double d = double(nx) * a[0] + double(ny) * a[1] + double(nz) * a[2];
    tris.push_back(make_float4(nx, ny, nz, float(d)));
  } else {
    tris.push_back(make_float4(0.0f, 0.0f, 0.0f, 0.0f));
  }
}

// Culling margin: 2e-4 of the scene extent plus a few ulps of the largest
// coordinate (far above the FP32 rounding of the plane distances and of the
// Moeller-Trumbore quantities for points near the scene).
float scene_margin(const float* xyz, const uint32_t* abc, uint32_t nf) {
  float smin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, smax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  float amax = 0.0f;
  for (uint32_t f = 0; f < nf; ++f)
    for (int j = 0; j < 3; ++j) {
      const float* v = xyz + 3 * size_t(abc[3 * f + j]);
      for (int k = 0; k < 3; ++k) {
        smin[k] = std::min(smin[k], v[k]);
        smax[k] = std::max(smax[k], v[k]);
        amax = std::max(amax, std::fabs(v[k]));
      }
    }
  if (nf == 0) return 1e-7f;
  const float extent = std::max(smax[0] - smin[0], std::max(smax[1] - smin[1], smax[2] - smin[2]));
  return 2e-4f * extent + 8.0f * FLT_EPSILON * amax + 1e-7f;
}

}  // namespace

void build_scene_arrays(const float* xyz, uint32_t nv, const uint32_t* abc, uint32_t nf, bool bvh,
                        BvhBuild& out) {
  (void)nv;
  out.nodes.clear();
  out.tris.clear();
  out.max_depth = 0;
  out.tris.reserve(size_t(nf) * 4);
  out.margin = scene_margin(xyz, abc, nf);
  if (!bvh || nf == 0) {
    for (uint32_t f = 0; f < nf; ++f) push_tri(out.tris, xyz, abc, f);
    return;
  }
  Builder B;
  B.prims.resize(nf);
  for (uint32_t f = 0; f < nf; ++f) {
    Prim& p = B.prims[f];
    for (int k = 0; k < 3; ++k) {
      p.lo[k] = FLT_MAX;
      p.hi[k] = -FLT_MAX;
    }
    for (int j = 0; j < 3; ++j) {
      const float* v = xyz + 3 * size_t(abc[3 * f + j]);
      for (int k = 0; k < 3; ++k) {
        p.lo[k] = std::min(p.lo[k], v[k]);
        p.hi[k] = std::max(p.hi[k], v[k]);
      }
    }
    for (int k = 0; k < 3; ++k) p.c[k] = 0.5f * (p.lo[k] + p.hi[k]);
  }
  B.margin = out.margin;
  B.idx.resize(nf);
  for (uint32_t i = 0; i < nf; ++i) B.idx[i] = i;
  B.nodes.resize(2);
  B.build(0, 0, nf, 0);
  out.nodes = std::move(B.nodes);
  out.max_depth = B.max_depth;
  out.margin = B.margin;
  for (uint32_t i = 0; i < nf; ++i) push_tri(out.tris, xyz, abc, B.idx[i]);
}

}  // namespace linon
