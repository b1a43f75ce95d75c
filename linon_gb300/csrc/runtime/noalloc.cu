// noalloc.cu — ray-path capture for callers that cannot allocate device memory.
//
// linon_capture_paths stages the rays' start positions in the context's
// scratch buffer, which it grows with cudaMalloc when a call needs more.  Some
// callers must not trigger that: a click handler on an interactive UI thread
// with a frame budget (a device allocation or free can synchronise the whole
// device), or a host that has given the context a fixed memory budget.  This
// entry point stages the positions in a fixed array inside the library
// instead, so it allocates nothing.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "internal.hpp"

namespace linon {
namespace {

// The largest number of rays one call takes.
constexpr int kNoAllocMaxRays = LINON_NOALLOC_MAX_RAYS;

// Start positions (x, y per ray) staged for the capture kernel: 2 x 16384
// floats = 128 KB, held on every GPU that loads the library until the
// process exits.  Every call overwrites the first 2 * n_rays floats before
// its kernel reads them and reads nothing else, so no part needs clearing.
// In host code the name is only a host-side stand-in: kernels get the device
// address from cudaGetSymbolAddress.
static __device__ __align__(256) float g_noalloc_positions[2 * kNoAllocMaxRays];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
float* g_positions_dev[kMaxDevices] = {nullptr};

// Device address of the array on the current device, looked up once per
// device (the first call on a device does this set-up).  The address belongs
// to the device's primary context: a cudaDeviceReset ends that context, and
// with it every linon context on the device and this set-up, so the library
// must not be used across a device reset.
int positions_address(int device, float** out) {
  if (device < 0 || device >= kMaxDevices) return set_error(LINON_EINVAL, "device index out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_positions_dev[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_positions);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(g_noalloc_positions)");
    g_positions_dev[device] = static_cast<float*>(p);
  }
  *out = g_positions_dev[device];
  return LINON_OK;
}

}  // namespace
}  // namespace linon

using namespace linon;

extern "C" int linon_capture_paths_noalloc(linon_ctx* ctx, const linon_field* field,
                                           const linon_camera* camera, const linon_settings* settings,
                                           const linon_march_params* params, int32_t width,
                                           int32_t height, const float* pos_xy, int32_t n_rays, float h,
                                           int32_t n_steps, int32_t record_every, float* out) {
  try {
    // the same checks as linon_capture_paths, then the array's limit
    if (int st = check_context(ctx)) return st;
    if (int st = check_field(ctx, field)) return st;
    if (!camera || !params || !pos_xy || !out) return set_error(LINON_EINVAL, "null capture argument");
    if (int st = check_image_size(width, height)) return st;
    if (n_rays <= 0) return set_error(LINON_EINVAL, "n_rays must be positive");
    if (n_rays > kNoAllocMaxRays)
      return set_error(LINON_EINVAL, "n_rays " + std::to_string(n_rays) + " exceeds the " +
                                         std::to_string(kNoAllocMaxRays) +
                                         " rays the no-alloc staging array holds");
    if (n_steps < 0 || n_steps > 10000000) return set_error(LINON_EINVAL, "n_steps must be in 0..1e7");
    if (record_every <= 0) return set_error(LINON_EINVAL, "record_every must be positive");
    if (!(h > 0.0f) || !std::isfinite(h)) return set_error(LINON_EINVAL, "h must be positive");
    float* pos_dev = nullptr;
    if (int st = positions_address(ctx->device, &pos_dev)) return st;
    // pos_xy is pageable host memory: the copy has read it when this returns
    cudaError_t e = cudaMemcpyAsync(pos_dev, pos_xy, sizeof(float) * 2 * size_t(n_rays),
                                    cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_error(e, "cudaMemcpyAsync (positions)");
    CaptureArgs a;
    std::memset(&a, 0, sizeof a);
    for (int k = 0; k < 3; ++k) {
      a.cam.o[k] = camera->origin[k];
      a.cam.d[k] = camera->view_direction[k];
      a.cam.u[k] = camera->up[k];
    }
    a.pos = pos_dev;
    a.out = reinterpret_cast<float4*>(out);
    a.W = width;
    a.H = height;
    a.focal_length = params->focal_length;
    a.viewport_height = params->viewport_height;
    a.field_weight = settings ? settings->field_weight : 1.0f;
    a.h = h;
    a.n_rays = n_rays;
    a.n_steps = n_steps;
    a.every = record_every;
    a.n_points = (n_steps + record_every - 1) / record_every + 1;
    a.record_final = 1;
    void* args[] = {&a};
    cudaKernel_t k = field->mod->kernels.at("linon_capture");
    const int threads = 32;
    e = cudaLaunchKernel((const void*)k, dim3(unsigned((n_rays + threads - 1) / threads)), dim3(threads), args, 0,
                         ctx->stream);
    if (e != cudaSuccess) return cuda_error(e, "cudaLaunchKernel (capture)");
    return LINON_OK;
  } catch (const std::exception& ex) {
    return set_error(LINON_EINVAL, std::string("internal error: ") + ex.what());
  }
}
