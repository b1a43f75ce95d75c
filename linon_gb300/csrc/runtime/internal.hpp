// internal.hpp — shared declarations of the linon runtime (not part of the ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../../include/linon.h"
#include "../device/march_types.h"

namespace linon {

// ---- errors -------------------------------------------------------------
int set_error(int status, const std::string& msg);
int cuda_error(cudaError_t e, const char* what);
#define LINON_CUDA(call)                                      \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return ::linon::cuda_error(e_, #call); \
  } while (0)

// no exception crosses the C ABI: entry points wrap their bodies in these
#define LINON_TRY_BEGIN try {
#define LINON_TRY_END                                                                       \
  }                                                                                         \
  catch (const std::bad_alloc&) {                                                           \
    return ::linon::set_error(LINON_ENOMEM, "host allocation failed");                      \
  }                                                                                         \
  catch (const std::exception& ex) {                                                        \
    return ::linon::set_error(LINON_EINVAL, std::string("internal error: ") + ex.what());    \
  }

// ---- device memory owned by a context -----------------------------------
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

// ---- embedded device sources (generated at build time) -------------------
struct EmbeddedFile {
  const char* name;
  const char* text;
};
extern const EmbeddedFile kEmbeddedDeviceSources[];
extern const int kEmbeddedDeviceSourceCount;

// ---- NVRTC JIT ----------------------------------------------------------
// One compiled module: the march kernels of one or several fields.
struct JitModule {
  cudaLibrary_t lib = nullptr;
  std::map<std::string, cudaKernel_t> kernels;
  std::string key;
  double compile_ms = 0;
};
// Compiles `source` (which #includes the embedded headers) for sm_103a and
// loads it on the current device.  Results are cached per (source, options)
// in memory and, when LINON_CACHE_DIR is set, on disk.
int jit_compile(const std::string& source, bool precise, const std::vector<std::string>& kernel_names,
                std::shared_ptr<JitModule>& out, std::string& log);
// Compiles `source` to a cubin without loading it (no device needed); the
// log carries the compiler's and ptxas' messages (registers, spills).
int jit_check(const std::string& source, bool precise, std::string& log, size_t* cubin_bytes);
std::string batched_module_source(const std::vector<const linon_field*>& fields);
bool any_stateful(const linon_field* const* fields, int n_fields);

// ---- BVH ----------------------------------------------------------------
struct BvhBuild {
  std::vector<float4> nodes;   // 2 per node
  std::vector<float4> tris;    // 3 per triangle, leaf order
  uint32_t max_depth = 0;
  float margin = 0.0f;         // inflation of the node boxes
};
// Builds the triangle array (brute force when leaf_size == 0) and, when
// requested, a binned-SAH BVH whose node boxes are inflated by `margin`.
void build_scene_arrays(const float* xyz, uint32_t nv, const uint32_t* abc, uint32_t nf,
                        bool bvh, BvhBuild& out);

// Scene pointers and parameters of a context for the kernels (api.cpp).
DevScene dev_scene(const linon_ctx* ctx);

// Argument checks shared by the entry points (api.cpp): a non-null context
// whose device is made current; a live field of that context; an image of
// 1..65535 pixels per side and at most 2^31-1 pixels.
int check_context(linon_ctx* ctx);
int check_field(const linon_ctx* ctx, const linon_field* f);
int check_image_size(int32_t W, int32_t H);

// Frees the batch tables, graphs and modules of a context (batch.cpp).
void batch_release(linon_ctx* ctx);

// Pieces of the batched launch, shared with the serving loop (batch.cpp).
int batch_tuning(const linon_ctx* ctx, const linon_batch_tuning* in, linon_batch_tuning& t);
long long batch_table(const linon_view* views, int n_views, const linon_batch_tuning& t,
                      std::vector<BatchView>& tab, int* n_blocks = nullptr);
// The module of the tuning's launch form (its three step modes).
int batch_module(linon_ctx* ctx, const linon_field* const* fields, int32_t n_fields, const linon_batch_tuning& t,
                 std::shared_ptr<JitModule>& mod);
// The batched kernel for a set of views: linon_batch_f / linon_batch_fk when
// no view refines its step adaptively and all (or none) use Kahan sums,
// otherwise the generic linon_batch.
const char* batch_kernel_name(const linon_view* views, int n_views, const linon_batch_tuning& t);
int batch_launch(linon_ctx* ctx, const std::shared_ptr<JitModule>& mod, const linon_batch_tuning& t,
                 BatchView* views_dev, int n_views, long long total_rays, int n_blocks,
                 unsigned long long* counter, cudaStream_t stream, const char* kernel);

}  // namespace linon

// ---- context and field objects (opaque in the ABI) ----------------------
struct linon_field {
  linon_ctx* ctx = nullptr;
  std::string body, helpers, cuda;
  int flags = 0;
  int flops_arith = 0, flops_transc = 0;
  bool stateful = false;  // var<private> state: batches never refill lanes mid-ray
  std::string cuda_pair;  // the field in pair form (two rays per thread), "" if none
  mutable int pair_state = 0;  // pair kernels: 0 not tried, 1 compiled, -1 not available
  std::shared_ptr<linon::JitModule> mod;  // capture, field_eval, base march variant
  mutable std::mutex vmu;                  // guards `variants`
  mutable std::map<int, std::shared_ptr<linon::JitModule>> variants;  // other march variants
};

struct linon_ctx {
  int device = 0;
  size_t budget = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  size_t device_bytes = 0;
  // scene
  bool has_scene = false;
  linon::DevBuf scene_block;  // [nodes | tris]
  linon::DevBuf face_rgb;
  int n_tris = 0, n_nodes = 0;
  uint32_t max_depth = 0;
  float margin = 0.0f;
  int staged_bytes = 0;
  // distance grid of the safe-ball radius (empty: the BVH query is used)
  linon::DevBuf grid;
  int gx = 0, gy = 0, gz = 0;
  float gox = 0.0f, goy = 0.0f, goz = 0.0f, gcell = 0.0f;
  // per-cell candidate triangle lists of the segment test (empty: BVH only)
  linon::DevBuf cells, cell_tris;
  float reach = 0.0f;
  // device error word and scratch
  int* d_err = nullptr;
  linon::DevBuf scratch;       // grown on demand (capture positions, queues, ...)
  linon::DevBuf host_io;       // device planes for linon_render_host
  // linon_render_host's band pipeline: two render streams (consecutive bands
  // overlap at their tails) and one copy stream, created on first use
  cudaStream_t band_stream[2] = {nullptr, nullptr};
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t band_start = nullptr, band_done[8] = {}, copies_done = nullptr;
  // batch tuning cache
  linon_batch_tuning tuned{};
  bool has_tuned = false;
};
