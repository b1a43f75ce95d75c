// grid.cu — the distance grid behind the safe-ball radius of the march.
//
// At each cell centre the grid holds nearest_leaf_bound (march.cuh): a lower
// bound on the distance to every margin-inflated BVH leaf box.  A ray that
// needs a new safe ball reads its cell instead of walking the BVH (the walk
// is a divergent loop of a few hundred instructions; the read is uniform).
#include "../device/march.cuh"
#include "kernels.hpp"

namespace linon {
namespace {

__global__ void __launch_bounds__(256) grid_build_kernel(DevScene s, float* grid) {
  const size_t n = size_t(s.gx) * s.gy * s.gz;
  const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  SceneView v;
  v.tris = s.tris;
  v.nodes = s.nodes;
  v.face_rgb = s.face_rgb;
  v.n_tris = s.n_tris;
  v.n_nodes = s.n_nodes;
  v.margin = s.margin;
  v.grid = nullptr;
  v.gx = s.gx;
  v.gy = s.gy;
  v.gz = s.gz;
  v.gox = s.gox;
  v.goy = s.goy;
  v.goz = s.goz;
  v.gcell = s.gcell;
  v.ginv = s.ginv;
  const int ix = int(i % size_t(s.gx));
  const int iy = int((i / size_t(s.gx)) % size_t(s.gy));
  const int iz = int(i / (size_t(s.gx) * s.gy));
  grid[i] = nearest_leaf_bound(v, grid_centre(v, ix, iy, iz), s.margin);
}

}  // namespace

cudaError_t launch_grid_build(const DevScene& s, float* grid, cudaStream_t stream) {
  const size_t n = size_t(s.gx) * s.gy * s.gz;
  if (n == 0) return cudaSuccess;
  grid_build_kernel<<<unsigned((n + 255) / 256), 256, 0, stream>>>(s, grid);
  return cudaGetLastError();
}

}  // namespace linon

namespace linon {
namespace {

// Leaves whose (margin-inflated) box is within distance `reach` of q: calls
// visit(first, count) for each; returns false if the stack overflowed.
template <class Visit>
__device__ bool leaves_within(const SceneView& v, const vec3f& q, float reach, Visit visit) {
  const float r2 = reach * reach;
  int stack[LINON_BVH_STACK];
  int sp = 0;
  int node = 0;
  for (;;) {
    const float4 lo = v.nodes[2 * node];
    const float4 hi = v.nodes[2 * node + 1];
    if (box_dist2(lo, hi, q) <= r2) {
      const int first = __float_as_int(lo.w);
      const int count = __float_as_int(hi.w);
      if (count > 0) {
        visit(first, count);
      } else {
        if (sp >= LINON_BVH_STACK) return false;
        stack[sp++] = first + 1;
        node = first;
        continue;
      }
    }
    if (sp == 0) return true;
    node = stack[--sp];
  }
}

__device__ SceneView view_of(const DevScene& s) {
  SceneView v;
  v.tris = s.tris;
  v.nodes = s.nodes;
  v.face_rgb = s.face_rgb;
  v.n_tris = s.n_tris;
  v.n_nodes = s.n_nodes;
  v.margin = s.margin;
  v.grid = nullptr;
  v.cells = nullptr;
  v.cell_tris = nullptr;
  v.reach = 0.0f;
  v.gx = s.gx;
  v.gy = s.gy;
  v.gz = s.gz;
  v.gox = s.gox;
  v.goy = s.goy;
  v.goz = s.goz;
  v.gcell = s.gcell;
  v.ginv = s.ginv;
  return v;
}

__device__ __forceinline__ void cell_of(const DevScene& s, size_t i, int& ix, int& iy, int& iz) {
  ix = int(i % size_t(s.gx));
  iy = int((i / size_t(s.gx)) % size_t(s.gy));
  iz = int(i / (size_t(s.gx) * s.gy));
}

// Candidate count per cell (-1: more than max_list, the cell uses the BVH).
__global__ void __launch_bounds__(256) cell_count_kernel(DevScene s, float reach, int max_list, int* counts) {
  const size_t n = size_t(s.gx) * s.gy * s.gz;
  const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const SceneView v = view_of(s);
  int ix, iy, iz;
  cell_of(s, i, ix, iy, iz);
  int c = 0;
  const bool ok = leaves_within(v, grid_centre(v, ix, iy, iz), reach, [&](int, int count) { c += count; });
  counts[i] = (!ok || c > max_list) ? -1 : c;
}

// Triangle slots of each listed cell, written at its start.
__global__ void __launch_bounds__(256) cell_fill_kernel(DevScene s, float reach, const int2* lists, int* slots) {
  const size_t n = size_t(s.gx) * s.gy * s.gz;
  const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int2 l = lists[i];
  if (l.y <= 0) return;
  const SceneView v = view_of(s);
  int ix, iy, iz;
  cell_of(s, i, ix, iy, iz);
  int k = 0;
  leaves_within(v, grid_centre(v, ix, iy, iz), reach, [&](int first, int count) {
    for (int j = 0; j < count && k < l.y; ++j) slots[l.x + k++] = first + j;
  });
}

}  // namespace

cudaError_t launch_cell_count(const DevScene& s, float reach, int max_list, int* counts, cudaStream_t stream) {
  const size_t n = size_t(s.gx) * s.gy * s.gz;
  if (n == 0) return cudaSuccess;
  cell_count_kernel<<<unsigned((n + 255) / 256), 256, 0, stream>>>(s, reach, max_list, counts);
  return cudaGetLastError();
}

cudaError_t launch_cell_fill(const DevScene& s, float reach, const int2* lists, int* slots, cudaStream_t stream) {
  const size_t n = size_t(s.gx) * s.gy * s.gz;
  if (n == 0) return cudaSuccess;
  cell_fill_kernel<<<unsigned((n + 255) / 256), 256, 0, stream>>>(s, reach, lists, slots);
  return cudaGetLastError();
}

}  // namespace linon
