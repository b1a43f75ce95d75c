// kernels.hpp — host launchers of the ahead-of-time kernels in kernels.cu.
#pragma once

#include <cuda_runtime.h>

#include "../../../include/linon.h"
#include "../device/march_types.h"

namespace linon {

struct OverlayArgs {
  const uchar4* in;       // ray-casting image (rgba8)
  const float4* mapping;  // endpoints
  uchar4* out;            // target image
  float* exponents;       // W*H, may be NULL
  int W, H;
  int mode, delta;
  float scaling;
  int srgb;
};

struct FtleArgs {
  DevCamera cam;
  const float4* mapping;
  float* out;
  int W, H;
  float focal_length, viewport_height;
  double half_over_T;  // 0.5 / T, in FP64 (a multiply per pixel instead of a divide)
};

cudaError_t launch_overlay(const OverlayArgs& a, bool fp64, cudaStream_t s);
// Fills the distance grid of s (s.gx * s.gy * s.gz floats) from its BVH.
cudaError_t launch_grid_build(const DevScene& s, float* grid, cudaStream_t stream);
// Candidate lists of the grid's cells: counts of the triangles in the leaves
// within `reach` of each cell centre (-1 above max_list), then their slots.
cudaError_t launch_cell_count(const DevScene& s, float reach, int max_list, int* counts, cudaStream_t stream);
cudaError_t launch_cell_fill(const DevScene& s, float reach, const int2* lists, int* slots, cudaStream_t stream);
cudaError_t launch_ftle(const FtleArgs& a, cudaStream_t s);
// slots: 9 u64 (8 selection keys + a found counter)
cudaError_t launch_outline(const float* e, int W, int H, float min_exp, unsigned long long* slots,
                           cudaStream_t s);
cudaError_t launch_quantile_hist(const float* e, int W, int H, int border, unsigned prefix,
                                 int high_shift, int shift, int bits, unsigned* hist,
                                 cudaStream_t s);
cudaError_t launch_pack_samples(const float4* pos, linon_ray_sample* out, int n_rays, int n_pts,
                                cudaStream_t s);
cudaError_t launch_fp32_probe(float* out, int blocks, int threads, int iters, cudaStream_t s);
// One CTA waiting (at most `polls` polls) on an mbarrier nothing completes:
// sets error bit 1 in *err (selfcheck.cu).
cudaError_t launch_bounded_wait_check(int* err, int polls, cudaStream_t stream);
cudaError_t launch_sum_steps(const int* steps, long long n, unsigned long long* out, cudaStream_t s);

}  // namespace linon
