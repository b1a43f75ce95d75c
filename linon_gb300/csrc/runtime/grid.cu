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
