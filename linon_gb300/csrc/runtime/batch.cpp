// batch.cpp — batched rendering of many views in one launch.
//
// The reference renders one view per dispatch (MainView::render,
// src/main_view.rs:831-849) and re-renders at h = 0.001 for Enhance
// (src/main_view.rs:778-802).  Here any number of views (different size,
// camera, step size and field) go into one launch: one CTA per tile of every
// view, or a persistent kernel fed by a device work queue (warps take whole
// 32-ray tiles, or refill finished lanes mid-ray); the launch (queue reset +
// kernel) is captured in a CUDA graph and replayed while the batch shape
// stays the same.  An autotuner sweeps schedule x block size x tile shape
// (x quantum for lane refills) on the caller's batch and caches the winner
// in the context.
#include <algorithm>
#include <cstdlib>
#include <chrono>
#include <cmath>
#include <cstring>
#include <sstream>

#include "internal.hpp"

namespace linon {
namespace {

struct BatchState {
  DevBuf views;    // BatchView table
  DevBuf counter;  // queue head
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<char> key;  // kernel params + launch shape of the captured graph
  std::map<std::string, std::shared_ptr<JitModule>> modules;
};

std::mutex g_bmu;
std::map<const linon_ctx*, BatchState> g_batch;

// The batched kernels: entry name, launch bounds, kernel template, mode
// (0 any views, 1 fixed steps, 2 fixed steps with Kahan sums).  A module
// holds the entries one launch form needs, so a first launch compiles three
// march loops per field instead of twelve.
struct BatchEntry {
  const char* name;
  const char* bounds;
  const char* body;
  int mode;
};
const BatchEntry kBatchEntries[] = {
    {"linon_batch", "LINON_BATCH_BOUNDS", "march_batch_kernel", 0},
    {"linon_batch_f", "LINON_BATCH_BOUNDS", "march_batch_kernel", 1},
    {"linon_batch_fk", "LINON_BATCH_BOUNDS", "march_batch_kernel", 2},
    {"linon_queue", "LINON_BATCH_BOUNDS", "march_queue_kernel", 0},
    {"linon_queue_f", "LINON_BATCH_BOUNDS", "march_queue_kernel", 1},
    {"linon_queue_fk", "LINON_BATCH_BOUNDS", "march_queue_kernel", 2},
    {"linon_multi", "LINON_MULTI_BOUNDS", "march_multi_kernel", 0},
    {"linon_multi_f", "LINON_MULTI_BOUNDS", "march_multi_kernel", 1},
    {"linon_multi_fk", "LINON_MULTI_BOUNDS", "march_multi_kernel", 2},
    {"linon_tileq", "LINON_MULTI_BOUNDS", "march_tileq_kernel", 0},
    {"linon_tileq_f", "LINON_MULTI_BOUNDS", "march_tileq_kernel", 1},
    {"linon_tileq_fk", "LINON_MULTI_BOUNDS", "march_tileq_kernel", 2},
};

const BatchEntry* batch_entry(const std::string& name) {
  for (const BatchEntry& e : kBatchEntries)
    if (name == e.name) return &e;
  return nullptr;
}

// The three modes of one launch form (the form of `kernel`).
std::vector<std::string> form_kernels(const std::string& kernel) {
  std::string base = kernel;
  for (const char* suffix : {"_fk", "_f"})
    if (base.size() > std::strlen(suffix) && base.compare(base.size() - std::strlen(suffix), std::string::npos,
                                                          suffix) == 0) {
      base.resize(base.size() - std::strlen(suffix));
      break;
    }
  return {base, base + "_f", base + "_fk"};
}

std::vector<std::string> all_batch_kernels() {
  std::vector<std::string> k;
  for (const BatchEntry& e : kBatchEntries) k.push_back(e.name);
  return k;
}

std::string batch_module_source(const std::vector<const linon_field*>& fields,
                                const std::vector<std::string>& kernels) {
  std::ostringstream s;
  s << "#include \"march.cuh\"\n";
  for (size_t i = 0; i < fields.size(); ++i) {
    std::string code = fields[i]->cuda;
    // rename the namespace of each field
    const std::string from = "namespace linon_user {";
    size_t p = code.find(from);
    if (p != std::string::npos) code.replace(p, from.size(), "namespace linon_user_" + std::to_string(i) + " {");
    s << code;
  }
  // one functor per field, and LinonFields: field i chosen per call (the
  // persistent kernels, whose warps mix views) or once per CTA by visit()
  // (the one-CTA-per-tile kernels, whose CTAs lie in one view)
  for (size_t i = 0; i < fields.size(); ++i)
    s << "struct LinonField" << i << " {\n"
         "  mutable linon_user_" << i << "::Private pv;\n"
         "  __device__ __forceinline__ wgsl::vec3f operator()(const wgsl::vec3f& pp, const wgsl::vec3f& p,\n"
         "      const wgsl::vec3f& v0, const wgsl::vec3f& v, float t) const {\n"
         "    return linon_user_" << i << "::field_function(pv, pp, p, v0, v, t);\n  }\n};\n";
  s << "struct LinonFields {\n"
       "  __device__ __forceinline__ wgsl::vec3f operator()(int i, const wgsl::vec3f& pp, const wgsl::vec3f& p,\n"
       "      const wgsl::vec3f& v0, const wgsl::vec3f& v, float t) const {\n"
       "    switch (i) {\n";
  for (size_t i = 1; i < fields.size(); ++i)
    s << "      case " << i << ": return LinonField" << i << "()(pp, p, v0, v, t);\n";
  s << "      default: return LinonField0()(pp, p, v0, v, t);\n"
       "    }\n  }\n"
       "  template <class Fn> __device__ __forceinline__ void visit(int i, const Fn& fn) const {\n"
       "    switch (i) {\n";
  for (size_t i = 1; i < fields.size(); ++i) s << "      case " << i << ": fn(LinonField" << i << "()); return;\n";
  s << "      default: fn(LinonField0()); return;\n"
       "    }\n  }\n};\n";
  for (const std::string& k : kernels) {
    const BatchEntry* e = batch_entry(k);
    if (!e) continue;
    s << "extern \"C\" __global__ void " << e->bounds << " " << e->name << "(linon::BatchArgs a) {\n  linon::"
      << e->body << "<" << e->mode << ">(LinonFields(), a);\n}\n";
  }
  return s.str();
}

int dev_grow(linon_ctx* ctx, DevBuf& b, size_t bytes) {
  if (b.bytes >= bytes && b.p) return LINON_OK;
  if (ctx->budget && ctx->device_bytes + (bytes - b.bytes) > ctx->budget)
    return set_error(LINON_ENOMEM, "HBM budget exceeded by the batch tables");
  if (b.p) {
    cudaFree(b.p);
    ctx->device_bytes -= b.bytes;
  }
  b.p = nullptr;
  b.bytes = 0;
  cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e != cudaSuccess) return cuda_error(e, "cudaMalloc");
  b.bytes = bytes;
  ctx->device_bytes += bytes;
  return LINON_OK;
}

int get_module(linon_ctx* ctx, BatchState& bs, const linon_field* const* fields, int32_t n_fields,
               const std::vector<std::string>& kernels, std::shared_ptr<JitModule>& mod) {
  std::vector<const linon_field*> fv(fields, fields + n_fields);
  std::string key;
  for (auto* f : fv) key += f->cuda + "\x01" + std::to_string(f->flags) + "\x02";
  for (auto& k : kernels) key += k + "\x03";
  // the extra compiler options are part of what the module is
  if (const char* extra = std::getenv("LINON_JIT_OPTIONS")) key += extra;
  auto it = bs.modules.find(key);
  if (it != bs.modules.end()) {
    mod = it->second;
    return LINON_OK;
  }
  std::string log;
  const bool precise = (fv[0]->flags & LINON_COMPILE_PRECISE) != 0;
  int st = jit_compile(batch_module_source(fv, kernels), precise, kernels, mod, log);
  if (st != LINON_OK) return set_error(st, st == LINON_ECOMPILE ? log : std::string(linon_last_error()));
  bs.modules[key] = mod;
  (void)ctx;
  return LINON_OK;
}

DevMarch to_dev(const linon_settings& st, const linon_march_params& mp) {
  DevMarch m;
  m.h_initial = mp.h_initial;
  m.t_max = mp.t_max;
  m.max_steps = mp.max_steps;
  m.adaptive = mp.adaptive;
  m.h_fine = mp.h_fine;
  m.h_fine_above = mp.h_fine_above;
  m.stop_on_hit = mp.stop_on_hit;
  m.kahan = mp.kahan;
  m.focal_length = mp.focal_length;
  m.viewport_height = mp.viewport_height;
  m.linear_mode = mp.linear_mode;
  m.field_weight = st.field_weight;
  return m;
}

int validate_batch(const linon_ctx* ctx, const linon_field* const* fields, int32_t n_fields,
                   const linon_view* views, int32_t n_views) {
  if (!ctx) return set_error(LINON_EINVAL, "null context");
  if (!fields || n_fields <= 0 || n_fields > LINON_MAX_BATCH_FIELDS)
    return set_error(LINON_EINVAL, "batch needs 1..8 fields");
  for (int i = 0; i < n_fields; ++i) {
    if (!fields[i] || !fields[i]->mod) return set_error(LINON_EINVAL, "null field in batch");
    if (fields[i]->ctx != ctx) return set_error(LINON_EINVAL, "field belongs to another context");
    if ((fields[i]->flags & LINON_COMPILE_PRECISE) != (fields[0]->flags & LINON_COMPILE_PRECISE))
      return set_error(LINON_EINVAL, "all fields of a batch must share the precision flag");
  }
  if (!views || n_views <= 0) return set_error(LINON_EINVAL, "batch needs at least one view");
  if (!ctx->has_scene) return set_error(LINON_ENOSCENE, "render before linon_scene_upload");
  for (int i = 0; i < n_views; ++i) {
    const linon_view& v = views[i];
    if (v.field_index < 0 || v.field_index >= n_fields)
      return set_error(LINON_EINVAL, "view " + std::to_string(i) + ": field_index out of range");
    if (v.width <= 0 || v.height <= 0 || v.width > 65535 || v.height > 65535)
      return set_error(LINON_EINVAL, "view " + std::to_string(i) + ": bad image size");
    const linon_march_params& p = v.params;
    if (!(p.h_initial > 0.0f)) return set_error(LINON_EINVAL, "view " + std::to_string(i) + ": h_initial must be positive");
    if (p.max_steps < 0 || p.max_steps > 50000000)
      return set_error(LINON_EINVAL, "view " + std::to_string(i) + ": max_steps out of range");
    if (p.max_steps == 0) {
      float hmin = p.adaptive ? std::min(p.h_initial, p.h_fine) : p.h_initial;
      if (!(hmin > 0.0f) || double(p.t_max) / hmin > 5e7 || std::fabs(p.t_max) + hmin == std::fabs(p.t_max))
        return set_error(LINON_EINVAL, "view " + std::to_string(i) + ": t-loop would not terminate");
    }
  }
  return LINON_OK;
}

}  // namespace

// The batched module (persistent and one-CTA-per-tile kernels) for a list of
// fields, for compile checks without a context.
std::string batched_module_source(const std::vector<const linon_field*>& fields) {
  return batch_module_source(fields, all_batch_kernels());
}

// Fields with var<private> state need one field functor per ray for the
// whole march: one CTA per tile and the queue of whole-warp tiles have it,
// the lane-refilling queue (a functor per quantum) does not.
bool any_stateful(const linon_field* const* fields, int n_fields) {
  for (int i = 0; i < n_fields; ++i)
    if (fields[i] && fields[i]->stateful) return true;
  return false;
}

int batch_tuning(const linon_ctx* ctx, const linon_batch_tuning* in, linon_batch_tuning& t) {
  t = linon_batch_tuning{};
  if (in) t = *in;
  else if (ctx->has_tuned) t = ctx->tuned;
  if (t.quantum <= 0) t.quantum = 1024;
  if (t.schedule < 0 || t.schedule > 3) return set_error(LINON_EINVAL, "schedule must be 0, 1, 2 or 3");
  // auto: one CTA per tile (64 uneven views: 11.2 ms against 11.5 ms for
  // the queue of warp tiles and 12.5 ms for lane refills below 8)
  if (t.schedule == 0) t.schedule = 2;
  // 0: the queue of whole-warp tiles; > 0: refill lanes mid-ray
  if (t.refill_below < 0) t.refill_below = 0;
  if (t.refill_below > 32) t.refill_below = 32;
  if (t.block_threads <= 0) t.block_threads = 128;
  if (t.block_threads % 32 || t.block_threads > 256)
    return set_error(LINON_EINVAL, "block_threads must be a multiple of 32, <= 256");
  if (t.tile_w <= 0 || t.tile_h <= 0) {
    t.tile_w = 4;
    t.tile_h = 8;
  }
  if (t.tile_w * t.tile_h != 32) return set_error(LINON_EINVAL, "tile_w * tile_h must be 32");
  return LINON_OK;
}

long long batch_table(const linon_view* views, int n_views, const linon_batch_tuning& t,
                      std::vector<BatchView>& tab, int* n_blocks) {
  tab.assign(static_cast<size_t>(n_views), BatchView());
  // Queue order: views with the largest step budget per ray first, so that
  // when the queue drains the SMs finish on short rays (longest-first list
  // scheduling); each table entry carries its own outputs, so the order is
  // free.  Budget: max_steps, or t_max / h for the t-loop.
  std::vector<int> order(static_cast<size_t>(n_views));
  std::vector<double> budget(static_cast<size_t>(n_views));
  for (int i = 0; i < n_views; ++i) {
    const linon_march_params& p = views[i].params;
    order[size_t(i)] = i;
    budget[size_t(i)] = p.max_steps > 0 ? double(p.max_steps) : double(p.t_max) / double(p.h_initial);
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return budget[size_t(a)] > budget[size_t(b)]; });
  long long begin = 0;
  int blocks = 0;
  for (int k = 0; k < n_views; ++k) {
    const int i = order[size_t(k)];
    const linon_view& v = views[i];
    BatchView& b = tab[size_t(k)];
    b.block_begin = blocks;
    b.blocks_x = (v.width + 7) / 8;
    blocks += b.blocks_x * ((v.height + 15) / 16);
    b.m = to_dev(v.settings, v.params);
    for (int c = 0; c < 3; ++c) {
      b.cam.o[c] = v.camera.origin[c];
      b.cam.d[c] = v.camera.view_direction[c];
      b.cam.u[c] = v.camera.up[c];
    }
    b.field = v.field_index;
    b.tiles_x = (v.width + t.tile_w - 1) / t.tile_w;
    const int tiles_y = (v.height + t.tile_h - 1) / t.tile_h;
    b.ray_begin = begin;
    b.frame.W = v.width;
    b.frame.H = v.height;
    b.frame.color = reinterpret_cast<uchar4*>(v.out.color);
    b.frame.mapping = reinterpret_cast<float4*>(v.out.mapping);
    b.frame.hit = v.out.hit_id;
    b.frame.steps = v.out.steps;
    begin += (long long)b.tiles_x * tiles_y * 32;
  }
  if (n_blocks) *n_blocks = blocks;
  return begin;
}

int batch_module(linon_ctx* ctx, const linon_field* const* fields, int32_t n_fields, const linon_batch_tuning& t,
                 std::shared_ptr<JitModule>& mod) {
  // the three modes of the tuning's launch form (a wave's views decide which)
  linon_view v{};
  v.params.kahan = 1;
  std::lock_guard<std::mutex> lock(g_bmu);
  return get_module(ctx, g_batch[ctx], fields, n_fields, form_kernels(batch_kernel_name(&v, 1, t)), mod);
}

// schedule 1 with refill_below 0: the queue of whole-warp tiles
// (linon_queue*); with refill_below > 0: the lane-refilling queue
// (linon_batch*); schedule 2: one CTA per tile (linon_multi*); schedule 3:
// the queue of CTA tiles (linon_tileq*).
const char* batch_kernel_name(const linon_view* views, int n_views, const linon_batch_tuning& t) {
  static const char* names[4][3] = {{"linon_batch", "linon_batch_f", "linon_batch_fk"},
                                    {"linon_queue", "linon_queue_f", "linon_queue_fk"},
                                    {"linon_multi", "linon_multi_f", "linon_multi_fk"},
                                    {"linon_tileq", "linon_tileq_f", "linon_tileq_fk"}};
  const int form = t.schedule >= 2 ? t.schedule : t.refill_below > 0 ? 0 : 1;
  bool kahan = false, plain = false;
  for (int i = 0; i < n_views; ++i) {
    if (views[i].params.adaptive) return names[form][0];
    (views[i].params.kahan ? kahan : plain) = true;
  }
  if (kahan && plain) return names[form][0];
  return names[form][kahan ? 2 : 1];
}

int batch_launch(linon_ctx* ctx, const std::shared_ptr<JitModule>& mod, const linon_batch_tuning& t,
                 BatchView* views_dev, int n_views, long long total_rays, int n_blocks,
                 unsigned long long* counter, cudaStream_t stream, const char* kernel) {
  BatchArgs a;
  std::memset(&a, 0, sizeof a);
  a.views = views_dev;
  a.n_views = n_views;
  a.quantum = t.quantum;
  a.total_rays = total_rays;
  a.counter = counter;
  a.scene = dev_scene(ctx);
  a.tile_w = t.tile_w;
  a.tile_h = t.tile_h;
  a.refill_below = t.refill_below;
  a.n_blocks = n_blocks;
  a.err = ctx->d_err;
  cudaKernel_t k = mod->kernels.at(kernel);
  if (t.schedule == 2) {
    if (n_blocks <= 0) return LINON_OK;
    void* args[] = {&a};
    LINON_CUDA(cudaLaunchKernel((const void*)k, dim3(unsigned(n_blocks)), dim3(128), args,
                                size_t(a.scene.staged_bytes), stream));
    return LINON_OK;
  }
  int sms = 0;
  LINON_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  const int threads = t.schedule == 3 ? 128 : t.block_threads;
  int per_sm = t.ctas_per_sm;
  if (per_sm <= 0) {
    int occ = 0;
    LINON_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void*)k, threads,
                                                             size_t(a.scene.staged_bytes)));
    per_sm = std::max(1, occ);
  }
  LINON_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), stream));
  void* args[] = {&a};
  LINON_CUDA(cudaLaunchKernel((const void*)k, dim3(unsigned(sms * per_sm)), dim3(unsigned(threads)), args,
                              size_t(a.scene.staged_bytes), stream));
  return LINON_OK;
}

void batch_release(linon_ctx* ctx) {
  std::lock_guard<std::mutex> lock(g_bmu);
  auto it = g_batch.find(ctx);
  if (it == g_batch.end()) return;
  BatchState& bs = it->second;
  if (bs.exec) cudaGraphExecDestroy(bs.exec);
  if (bs.graph) cudaGraphDestroy(bs.graph);
  if (bs.views.p) cudaFree(bs.views.p);
  if (bs.counter.p) cudaFree(bs.counter.p);
  g_batch.erase(it);
}

}  // namespace linon

using namespace linon;

extern "C" {

int linon_render_batch(linon_ctx* ctx, const linon_field* const* fields, int32_t n_fields,
                       const linon_view* views, int32_t n_views, const linon_batch_tuning* tuning) {
  try {
    if (int st = validate_batch(ctx, fields, n_fields, views, n_views)) return st;
    LINON_CUDA(cudaSetDevice(ctx->device));
    std::lock_guard<std::mutex> lock(g_bmu);
    BatchState& bs = g_batch[ctx];
    linon_batch_tuning t;
    if (int st = batch_tuning(ctx, tuning, t)) return st;
    if (any_stateful(fields, n_fields)) t.refill_below = 0;  // the queue of warp tiles instead
    const char* kname = batch_kernel_name(views, n_views, t);
    std::shared_ptr<JitModule> mod;
    if (int st = get_module(ctx, bs, fields, n_fields, {kname}, mod)) return st;
    std::vector<BatchView> tab;
    int n_blocks = 0;
    const long long begin = batch_table(views, n_views, t, tab, &n_blocks);
    if (int st = dev_grow(ctx, bs.views, sizeof(BatchView) * tab.size())) return st;
    if (int st = dev_grow(ctx, bs.counter, 256)) return st;
    LINON_CUDA(cudaMemcpyAsync(bs.views.p, tab.data(), sizeof(BatchView) * tab.size(),
                               cudaMemcpyHostToDevice, ctx->stream));
    BatchArgs a;
    std::memset(&a, 0, sizeof a);
    a.views = static_cast<BatchView*>(bs.views.p);
    a.n_views = n_views;
    a.quantum = t.quantum;
    a.total_rays = begin;
    a.counter = static_cast<unsigned long long*>(bs.counter.p);
    a.scene = dev_scene(ctx);
    a.tile_w = t.tile_w;
    a.tile_h = t.tile_h;
    a.refill_below = t.refill_below;
    a.n_blocks = n_blocks;
    a.err = ctx->d_err;
    cudaKernel_t k = mod->kernels.at(kname);
    dim3 grid, block;
    if (t.schedule == 2) {
      grid = dim3(unsigned(std::max(n_blocks, 1)));
      block = dim3(128);
    } else {
      int sms = 0;
      LINON_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
      const int threads = t.schedule == 3 ? 128 : t.block_threads;  // CTA tiles: 128 threads
      int per_sm = t.ctas_per_sm;
      if (per_sm <= 0) {
        int occ = 0;
        LINON_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void*)k, threads,
                                                                 size_t(a.scene.staged_bytes)));
        per_sm = std::max(1, occ);
      }
      grid = dim3(unsigned(sms * per_sm));
      block = dim3(unsigned(threads));
    }
    // graph key: the kernel parameters and the launch shape
    std::vector<char> key(sizeof a + sizeof(k) + 2 * sizeof(unsigned));
    std::memcpy(key.data(), &a, sizeof a);
    std::memcpy(key.data() + sizeof a, &k, sizeof k);
    std::memcpy(key.data() + sizeof a + sizeof k, &grid.x, sizeof(unsigned));
    std::memcpy(key.data() + sizeof a + sizeof k + sizeof(unsigned), &block.x, sizeof(unsigned));
    if (!bs.exec || key != bs.key) {
      if (bs.exec) { cudaGraphExecDestroy(bs.exec); bs.exec = nullptr; }
      if (bs.graph) { cudaGraphDestroy(bs.graph); bs.graph = nullptr; }
      cudaStream_t cs;
      LINON_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      LINON_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      cudaMemsetAsync(bs.counter.p, 0, sizeof(unsigned long long), cs);
      void* args[] = {&a};
      cudaError_t le = cudaLaunchKernel((const void*)k, grid, block, args, size_t(a.scene.staged_bytes), cs);
      cudaError_t ce = cudaStreamEndCapture(cs, &bs.graph);
      cudaStreamDestroy(cs);
      if (le != cudaSuccess) return cuda_error(le, "cudaLaunchKernel (capture)");
      if (ce != cudaSuccess) return cuda_error(ce, "cudaStreamEndCapture");
      LINON_CUDA(cudaGraphInstantiate(&bs.exec, bs.graph, 0));
      bs.key = key;
    }
    LINON_CUDA(cudaGraphLaunch(bs.exec, ctx->stream));
    return LINON_OK;
  } catch (const std::exception& e) {
    return set_error(LINON_EINVAL, std::string("internal error: ") + e.what());
  }
}

int linon_render_views_plain(linon_ctx* ctx, const linon_field* const* fields, int32_t n_fields,
                             const linon_view* views, int32_t n_views) {
  if (int st = validate_batch(ctx, fields, n_fields, views, n_views)) return st;
  for (int i = 0; i < n_views; ++i) {
    const linon_view& v = views[i];
    linon_frame f = v.out;
    f.width = v.width;
    f.height = v.height;
    if (int st = linon_render(ctx, fields[v.field_index], &v.camera, &v.settings, &v.params, &f)) return st;
  }
  return LINON_OK;
}

int linon_autotune_batch(linon_ctx* ctx, const linon_field* const* fields, int32_t n_fields,
                         const linon_view* views, int32_t n_views, linon_batch_tuning* best,
                         double* best_ms) {
  if (int st = validate_batch(ctx, fields, n_fields, views, n_views)) return st;
  // Persistent queue: whole-warp tiles (refill_below 0; quantum unused),
  // or lanes refilled once fewer than 8 march, every quantum steps.
  const int quanta[] = {256, 1024, 4096};
  const int blocks[] = {128, 256};
  const int tiles[][2] = {{8, 4}, {4, 8}};
  const int refills[] = {0, 8};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best_t = 1e300;
  linon_batch_tuning bt{};
  const bool stateful = any_stateful(fields, n_fields);
  for (int rf : refills)
    for (int q : quanta)
      for (int b : blocks)
        for (auto& tl : tiles) {
        if (stateful && rf > 0) continue;  // lane refills: not for fields with var<private> state
        if (rf == 0 && q != quanta[0]) continue;  // the quantum plays no part
        linon_batch_tuning t{};
        t.schedule = 1;
        t.quantum = q;
        t.block_threads = b;
        t.tile_w = tl[0];
        t.tile_h = tl[1];
        t.refill_below = rf;
        if (int st = linon_render_batch(ctx, fields, n_fields, views, n_views, &t)) {
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
          return st;
        }
        cudaEventRecord(e0, ctx->stream);
        int st = linon_render_batch(ctx, fields, n_fields, views, n_views, &t);
        cudaEventRecord(e1, ctx->stream);
        if (st) {
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
          return st;
        }
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_t) {
          best_t = ms;
          bt = t;
        }
      }
  for (int sched : {2, 3}) {
    // one CTA per tile, and the queue of CTA tiles
    linon_batch_tuning t{};
    t.schedule = sched;
    int st = linon_render_batch(ctx, fields, n_fields, views, n_views, &t);
    if (!st) {
      cudaEventRecord(e0, ctx->stream);
      st = linon_render_batch(ctx, fields, n_fields, views, n_views, &t);
      cudaEventRecord(e1, ctx->stream);
    }
    if (st) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return st;
    }
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_t) {
      best_t = ms;
      bt = t;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->tuned = bt;
  ctx->has_tuned = true;
  if (best) *best = bt;
  if (best_ms) *best_ms = best_t;
  return LINON_OK;
}

}  // extern "C"
