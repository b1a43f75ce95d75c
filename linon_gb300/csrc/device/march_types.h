// march_types.h — POD argument blocks shared by the host runtime and the
// NVRTC-compiled march / capture kernels (passed by value as the single
// kernel parameter).  Plain C layout, no system headers on the device side.
#pragma once

#if !defined(__CUDACC_RTC__)
#include <vector_types.h>
#endif

namespace linon {

// linon_march_params + Settings.field_weight, in device form.
struct DevMarch {
  float h_initial;
  float t_max;
  int max_steps;
  int adaptive;
  float h_fine;
  float h_fine_above;
  int stop_on_hit;
  int kahan;
  float focal_length;
  float viewport_height;
  int linear_mode;
  float field_weight;
};

// Camera uniform fields read by the shader (origin, view_direction, up).
struct DevCamera {
  float o[3];
  float d[3];
  float u[3];
};

struct DevScene {
  const float4* tris;      // 4 float4 per triangle (see march.cuh)
  const float4* nodes;     // 2 float4 per BVH node, NULL = brute force
  const float4* face_rgb;  // optional per-face colour (by original face index)
  const float4* staged;    // contiguous [nodes | tris] block for smem staging
  int n_tris;
  int n_nodes;
  int staged_bytes;        // 0 = read the scene from global memory
  float margin;            // inflation of the BVH boxes (culling margin)
  // distance grid (NULL: none): at each cell centre a lower bound on the
  // distance to every margin-inflated BVH leaf box
  const float* grid;
  int gx, gy, gz;          // cells per axis
  float gox, goy, goz;     // corner of cell (0, 0, 0)
  float gcell, ginv;       // cell size and its inverse
  // per-cell candidate triangles (NULL: none): cells[i] = (start, count)
  // into cell_tris (triangle slots), count -1 = use the BVH; valid for
  // segments of length <= reach that start in the cell
  const int2* cells;
  const int* cell_tris;
  float reach;
};

struct DevFrame {
  int W, H;
  uchar4* color;
  float4* mapping;
  int* hit;
  int* steps;
};

struct MarchArgs {
  DevMarch m;
  DevCamera cam;
  DevScene scene;
  DevFrame frame;
  int tile_w, tile_h;
  int row0, row1;          // rows [row0, row1) of the frame this launch covers
  int* err;                // device error word (bit 0: smem staging timeout)
};

// One view of a batched launch (device table entry).
struct BatchView {
  DevMarch m;
  DevCamera cam;
  int field;           // index into the module's field table
  int tiles_x;         // tiles per image row
  long long ray_begin; // first ray of this view in the batch's ray space
  DevFrame frame;
  int block_begin;     // first CTA of this view in a one-CTA-per-tile launch
  int blocks_x;        // 8 x 16-pixel CTA tiles per image row
  // persistent queue: the view's next ray to hand out (the host uploads the
  // table with 0 before every launch; warps take rays with atomicAdd)
  unsigned long long next;
};

struct BatchArgs {
  BatchView* views;
  int n_views;
  int quantum;             // RK4 steps between retire/refill
  long long total_rays;
  unsigned long long* counter;  // persistent queue: [0] first view that may have rays (zeroed before the launch)
  DevScene scene;
  int tile_w, tile_h;      // tile_w * tile_h == 32
  int refill_below;        // leave the quantum early below this many marching lanes
  int n_blocks;            // CTAs of a one-CTA-per-tile launch
  int* err;
};

struct CaptureArgs {
  DevCamera cam;
  const float* pos;        // n_rays * 2 normalised positions (device)
  float4* out;             // n_rays * n_points
  int W, H;
  float focal_length, viewport_height;
  float field_weight;
  float h;
  int n_rays, n_steps, every, n_points, record_final;
  int pad;
};

}  // namespace linon
