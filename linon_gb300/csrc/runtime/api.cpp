// api.cpp — the C ABI of include/linon.h.
//
// Each entry point names the part of the reference's MainView
// (src/main_view.rs) or shader it replaces.  No exception leaves this file:
// every failure becomes a status code plus linon_last_error().
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "../wgsl/frontend.hpp"
#include "internal.hpp"
#include "kernels.hpp"

namespace linon {

namespace {
thread_local std::string g_last_error;
}

int set_error(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

int cuda_error(cudaError_t e, const char* what) {
  cudaGetLastError();  // clear a sticky-free error so the next call starts clean
  return set_error(e == cudaErrorMemoryAllocation ? LINON_ENOMEM : LINON_ECUDA,
                   std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {

int dev_alloc(linon_ctx* ctx, DevBuf& b, size_t bytes) {
  if (b.bytes >= bytes && b.p) return LINON_OK;
  size_t grow = bytes - b.bytes;
  if (ctx->budget && ctx->device_bytes + grow > ctx->budget)
    return set_error(LINON_ENOMEM, "HBM budget exceeded: " + std::to_string(ctx->device_bytes + grow) +
                                       " > " + std::to_string(ctx->budget) + " bytes");
  if (b.p) {
    cudaFree(b.p);
    ctx->device_bytes -= b.bytes;
    b.p = nullptr;
    b.bytes = 0;
  }
  cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e != cudaSuccess) return cuda_error(e, "cudaMalloc");
  b.bytes = bytes;
  ctx->device_bytes += bytes;
  return LINON_OK;
}

void dev_free(linon_ctx* ctx, DevBuf& b) {
  if (b.p) {
    cudaFree(b.p);
    ctx->device_bytes -= b.bytes;
  }
  b.p = nullptr;
  b.bytes = 0;
}

// Candidate triangle lists of the distance grid's cells (segment test
// without a BVH walk): a segment of length <= reach = 2 cells starting in a
// cell can only meet triangles of the leaves within the cell's half
// diagonal plus reach of its centre.  Cells with more than 64 candidates
// keep the BVH.  Skipped (BVH only) when the HBM budget cannot hold them.
int build_cell_lists(linon_ctx* ctx) {
  const size_t n = size_t(ctx->gx) * ctx->gy * ctx->gz;
  if (n == 0) return LINON_OK;
  const float reach = 2.0f * ctx->gcell;
  const float build_reach = (0.5f * std::sqrt(3.0f) * ctx->gcell + reach) * 1.0001f;
  const int max_list = 64;
  if (ctx->budget && ctx->device_bytes + n * (sizeof(int2) + sizeof(int)) > ctx->budget) return LINON_OK;
  DevBuf counts;
  if (int st = dev_alloc(ctx, counts, n * sizeof(int))) return st;
  DevScene s = dev_scene(ctx);
  cudaError_t e = launch_cell_count(s, build_reach, max_list, static_cast<int*>(counts.p), ctx->stream);
  std::vector<int> hc(n);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hc.data(), counts.p, n * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  dev_free(ctx, counts);
  if (e != cudaSuccess) return cuda_error(e, "cell list count");
  std::vector<int2> lists(n);
  long long total = 0;
  for (size_t i = 0; i < n; ++i) {
    lists[i] = make_int2(int(total), hc[i]);
    if (hc[i] > 0) total += hc[i];
  }
  if (total >= (1ll << 31) - 1) return LINON_OK;
  const size_t tbytes = sizeof(int) * size_t(std::max<long long>(total, 1));
  if (ctx->budget && ctx->device_bytes + n * sizeof(int2) + tbytes > ctx->budget) return LINON_OK;
  if (int st = dev_alloc(ctx, ctx->cells, n * sizeof(int2))) return st;
  if (int st = dev_alloc(ctx, ctx->cell_tris, tbytes)) return st;
  LINON_CUDA(cudaMemcpyAsync(ctx->cells.p, lists.data(), n * sizeof(int2), cudaMemcpyHostToDevice, ctx->stream));
  LINON_CUDA(launch_cell_fill(s, build_reach, static_cast<const int2*>(ctx->cells.p),
                              static_cast<int*>(ctx->cell_tris.p), ctx->stream));
  LINON_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->reach = reach;
  return LINON_OK;
}

int enter(linon_ctx* ctx) {
  if (!ctx) return set_error(LINON_EINVAL, "null context");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  return LINON_OK;
}

DevMarch dev_march(const linon_settings* st, const linon_march_params* mp) {
  DevMarch m;
  m.h_initial = mp->h_initial;
  m.t_max = mp->t_max;
  m.max_steps = mp->max_steps;
  m.adaptive = mp->adaptive;
  m.h_fine = mp->h_fine;
  m.h_fine_above = mp->h_fine_above;
  m.stop_on_hit = mp->stop_on_hit;
  m.kahan = mp->kahan;
  m.focal_length = mp->focal_length;
  m.viewport_height = mp->viewport_height;
  m.linear_mode = mp->linear_mode;
  m.field_weight = st ? st->field_weight : 1.0f;
  return m;
}

DevCamera dev_camera(const linon_camera* c) {
  DevCamera d;
  for (int k = 0; k < 3; ++k) {
    d.o[k] = c->origin[k];
    d.d[k] = c->view_direction[k];
    d.u[k] = c->up[k];
  }
  return d;
}


int check_frame_size(int32_t W, int32_t H) {
  if (W <= 0 || H <= 0) return set_error(LINON_EINVAL, "image size must be positive");
  if (int64_t(W) * H > (int64_t(1) << 31) - 1 || W > 65535 || H > 65535)
    return set_error(LINON_EINVAL, "image too large (max 65535 per side, 2^31-1 pixels)");
  return LINON_OK;
}

int check_params(const linon_march_params* mp) {
  if (!mp) return set_error(LINON_EINVAL, "null march params");
  if (!(mp->h_initial > 0.0f) || !std::isfinite(mp->h_initial))
    return set_error(LINON_EINVAL, "h_initial must be a positive finite step");
  if (mp->max_steps < 0) return set_error(LINON_EINVAL, "max_steps must be >= 0");
  if (mp->max_steps == 0) {
    if (!std::isfinite(mp->t_max)) return set_error(LINON_EINVAL, "t_max must be finite");
    // the t-loop must end: at most t_max / min(h) + 2 iterations
    float hmin = mp->adaptive ? std::min(mp->h_initial, mp->h_fine) : mp->h_initial;
    if (!(hmin > 0.0f)) return set_error(LINON_EINVAL, "adaptive h_fine must be positive");
    double iters = double(mp->t_max) / double(hmin);
    if (iters > 5e7) return set_error(LINON_EINVAL, "t_max / h exceeds 5e7 steps per ray");
    // t + h must grow: h must not vanish against t (fp32 spacing at t_max)
    float tm = std::fabs(mp->t_max);
    if (tm + hmin == tm) return set_error(LINON_EINVAL, "step h vanishes against t_max in fp32");
  }
  if (mp->max_steps > 50000000) return set_error(LINON_EINVAL, "max_steps exceeds 5e7");
  return LINON_OK;
}

// The march variant a render needs (bits of march.cuh's V_* enum).
int march_variant(const linon_march_params* mp, const linon_settings* st, bool precise) {
  int v = 0;
  if (mp->adaptive) v |= 1;
  if (mp->kahan) v |= 2;
  if (mp->max_steps > 0) v |= 4;
  if (!precise && (st ? st->field_weight : 1.0f) == 1.0f) v |= 8;
  return v;
}

std::string march_kernel_name(int v) { return "linon_march_v" + std::to_string(v); }

// Module source for one field: generated CUDA C + the kernel instantiations.
// The base module holds the capture and field-evaluation kernels and the
// march variant of the reference's own settings; other march variants are
// compiled into small modules of their own when a render first needs them.
std::string module_source(const std::string& field_cuda, const std::vector<int>& variants, bool base) {
  std::ostringstream s;
  // packed normalize: measured faster in the per-frame kernels (1080p
  // frames 63.6 -> 62.9 ms), slower in the batched ones (not defined there)
  s << "#define LINON_PACKED_NORMALIZE 1\n#include \"march.cuh\"\n" << field_cuda << R"LINON(
struct LinonField {
  // the ray's var<private> state: one functor per thread and ray
  mutable linon_user::Private pv;
  __device__ __forceinline__ wgsl::vec3f operator()(const wgsl::vec3f& pp, const wgsl::vec3f& p,
      const wgsl::vec3f& v0, const wgsl::vec3f& v, float t) const {
    return linon_user::field_function(pv, pp, p, v0, v, t);
  }
};
)LINON";
  for (int v : variants)
    s << "extern \"C\" __global__ void LINON_MARCH_BOUNDS " << march_kernel_name(v)
      << "(linon::MarchArgs a) {\n  linon::march_plain_kernel<" << v << ">(LinonField(), a);\n}\n";
  if (base)
    s << R"LINON(extern "C" __global__ void __launch_bounds__(256) linon_capture(linon::CaptureArgs a) {
  linon::capture_kernel(LinonField(), a);
}
extern "C" __global__ void __launch_bounds__(256) linon_field_eval(const float* in, float* out, int n) {
  linon::field_eval_kernel(LinonField(), in, out, n);
}
)LINON";
  return s.str();
}

// Module source of a two-ray march variant (V_PAIRS): the field in pair
// form and march_pair_kernel.
std::string module_source_pair(const std::string& field_pair_cuda, int v) {
  std::ostringstream s;
  s << "#define LINON_PAIRS 1\n#include \"march.cuh\"\n" << field_pair_cuda << R"LINON(
struct LinonFieldPair {
  mutable linon_user::Private pv;  // two rays' var<private> state, lane-wise
  __device__ __forceinline__ wgsl::vec3p operator()(const wgsl::vec3p& pp, const wgsl::vec3p& p,
      const wgsl::vec3p& v0, const wgsl::vec3p& v, wgsl::f2 t) const {
    return linon_user::field_function(pv, pp, p, v0, v, t);
  }
};
)LINON";
  s << "extern \"C\" __global__ void LINON_MARCH_BOUNDS " << march_kernel_name(v)
    << "(linon::MarchArgs a) {\n  linon::march_pair_kernel<" << (v & ~16) << ">(LinonFieldPair(), a);\n}\n";
  return s.str();
}

std::vector<std::string> module_kernels(const std::vector<int>& variants, bool base) {
  std::vector<std::string> k;
  for (int v : variants) k.push_back(march_kernel_name(v));
  if (base) {
    k.push_back("linon_capture");
    k.push_back("linon_field_eval");
  }
  return k;
}

// Base variant: the reference's t <= 5 loop with adaptive refinement,
// field_weight 1 (main_view.wgsl:227-244, main_view.rs:133-139).
int base_variant(bool precise) { return precise ? 1 : 1 | 8; }

// Kernel of march variant v for the field, compiling it on first use.
int march_kernel(const linon_field* f, int v, cudaKernel_t* out) {
  {
    auto it = f->mod->kernels.find(march_kernel_name(v));
    if (it != f->mod->kernels.end()) {
      *out = it->second;
      return LINON_OK;
    }
  }
  std::lock_guard<std::mutex> lock(f->vmu);
  auto vit = f->variants.find(v);
  if (vit == f->variants.end()) {
    std::shared_ptr<JitModule> mod;
    std::string log;
    const bool precise = (f->flags & LINON_COMPILE_PRECISE) != 0;
    const std::string src = (v & 16) ? module_source_pair(f->cuda_pair, v) : module_source(f->cuda, {v}, false);
    int st = jit_compile(src, precise, module_kernels({v}, false), mod, log);
    if (st != LINON_OK) return set_error(st, st == LINON_ECOMPILE ? log : std::string(g_last_error));
    vit = f->variants.emplace(v, mod).first;
  }
  *out = vit->second->kernels.at(march_kernel_name(v));
  return LINON_OK;
}

int field_valid(const linon_ctx* ctx, const linon_field* f) {
  if (!f || !f->mod) return set_error(LINON_EINVAL, "null or released field");
  if (f->ctx != ctx) return set_error(LINON_EINVAL, "field belongs to another context");
  return LINON_OK;
}

void copy_log(const std::string& s, char* log, size_t cap) {
  if (!log || cap == 0) return;
  size_t n = std::min(cap - 1, s.size());
  std::memcpy(log, s.data(), n);
  log[n] = '\0';
}

// Reference capture seeds: mouse_pos + 0.01 * sample_positions[i]
// (main_view.wgsl:316-325,470-471).
void reference_ring(const linon_settings* st, float out[16]) {
  static const float ring[8][2] = {{-1.0f, -1.0f}, {0.0f, -1.0f}, {1.0f, -1.0f}, {1.0f, 0.0f},
                                   {1.0f, 1.0f},   {0.0f, 1.0f},  {-1.0f, 1.0f}, {-1.0f, 0.0f}};
  for (int i = 0; i < 8; ++i) {
    // compiled with -ffp-contract=off: a product and a sum, as in the shader
    out[2 * i] = st->mouse_pos[0] + 0.01f * ring[i][0];
    out[2 * i + 1] = st->mouse_pos[1] + 0.01f * ring[i][1];
  }
}

int launch_capture(linon_ctx* ctx, const linon_field* field, const linon_camera* camera,
                   const linon_settings* settings, const linon_march_params* params, int32_t W,
                   int32_t H, const float* pos_xy, int32_t n_rays, float h, int32_t n_steps,
                   int32_t every, int record_final, float4* out, int32_t n_points) {
  // positions go to the front of the scratch buffer
  int st = dev_alloc(ctx, ctx->scratch, std::max<size_t>(ctx->scratch.bytes, sizeof(float) * 2 * n_rays + 256));
  if (st) return st;
  LINON_CUDA(cudaMemcpyAsync(ctx->scratch.p, pos_xy, sizeof(float) * 2 * n_rays,
                             cudaMemcpyHostToDevice, ctx->stream));
  CaptureArgs a;
  a.cam = dev_camera(camera);
  a.pos = static_cast<const float*>(ctx->scratch.p);
  a.out = out;
  a.W = W;
  a.H = H;
  a.focal_length = params->focal_length;
  a.viewport_height = params->viewport_height;
  a.field_weight = settings ? settings->field_weight : 1.0f;
  a.h = h;
  a.n_rays = n_rays;
  a.n_steps = n_steps;
  a.every = every;
  a.n_points = n_points;
  a.record_final = record_final;
  a.pad = 0;
  void* args[] = {&a};
  cudaKernel_t k = field->mod->kernels.at("linon_capture");
  const int threads = 32;
  LINON_CUDA(cudaLaunchKernel((const void*)k, dim3((n_rays + threads - 1) / threads), dim3(threads),
                              args, 0, ctx->stream));
  // the positions were copied from pageable memory; keep them alive until the
  // copy has happened (cudaMemcpyAsync from pageable memory returns after the
  // host buffer was read)
  return LINON_OK;
}

}  // namespace
}  // namespace linon

using namespace linon;

namespace linon {
DevScene dev_scene(const linon_ctx* ctx) {
  DevScene s;
  const float4* block = static_cast<const float4*>(ctx->scene_block.p);
  s.nodes = ctx->n_nodes ? block : nullptr;
  s.tris = block + 2 * size_t(ctx->n_nodes);
  s.face_rgb = static_cast<const float4*>(ctx->face_rgb.p);
  s.staged = block;
  s.n_tris = ctx->n_tris;
  s.n_nodes = ctx->n_nodes;
  s.staged_bytes = ctx->staged_bytes;
  s.margin = ctx->margin;
  s.grid = static_cast<const float*>(ctx->grid.p);
  s.gx = ctx->gx;
  s.gy = ctx->gy;
  s.gz = ctx->gz;
  s.gox = ctx->gox;
  s.goy = ctx->goy;
  s.goz = ctx->goz;
  s.gcell = ctx->gcell;
  s.ginv = ctx->gcell > 0.0f ? 1.0f / ctx->gcell : 0.0f;
  s.cells = static_cast<const int2*>(ctx->cells.p);
  s.cell_tris = static_cast<const int*>(ctx->cell_tris.p);
  s.reach = ctx->reach;
  return s;
}

int check_context(linon_ctx* ctx) { return enter(ctx); }
int check_field(const linon_ctx* ctx, const linon_field* f) { return field_valid(ctx, f); }
int check_image_size(int32_t W, int32_t H) { return check_frame_size(W, H); }
}  // namespace linon

extern "C" {

int linon_abi_version(void) { return LINON_ABI_VERSION; }

const char* linon_last_error(void) { return g_last_error.c_str(); }

const char* linon_status_string(int status) {
  switch (status) {
    case LINON_OK: return "ok";
    case LINON_EINVAL: return "invalid argument";
    case LINON_ECOMPILE: return "field function compilation failed";
    case LINON_ECUDA: return "CUDA error";
    case LINON_ENOMEM: return "out of memory / HBM budget exceeded";
    case LINON_ETIMEOUT: return "bounded wait timed out";
    case LINON_ENOSCENE: return "no scene uploaded";
    case LINON_EBUSY: return "busy";
    case LINON_ESTATE: return "invalid state";
    case LINON_EIO: return "file could not be read";
  }
  return "unknown status";
}

void linon_march_params_reference(linon_march_params* out) {
  if (!out) return;
  std::memset(out, 0, sizeof(*out));
  out->h_initial = 0.1f;        // main_view.wgsl:241
  out->t_max = 5.0f;            // main_view.wgsl:244
  out->max_steps = 0;
  out->adaptive = 1;            // main_view.wgsl:227 (always on, see main_view.rs:752-776)
  out->h_fine = 0.001f;         // main_view.wgsl:253
  out->h_fine_above = 0.002f;   // main_view.wgsl:252
  out->stop_on_hit = 0;
  out->kahan = 0;
  out->focal_length = 0.035f;   // main_view.wgsl:355
  out->viewport_height = 0.025f;// main_view.wgsl:356
  out->linear_mode = 0;         // main_view.wgsl:72
}

int linon_create(int device, size_t hbm_budget_bytes, linon_ctx** out) {
  LINON_TRY_BEGIN
  if (!out) return set_error(LINON_EINVAL, "null output pointer");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDeviceCount");
  if (device < 0 || device >= n) return set_error(LINON_EINVAL, "no such CUDA device");
  LINON_CUDA(cudaSetDevice(device));
  LINON_CUDA(cudaFree(nullptr));  // create / retain the primary context
  auto* ctx = new linon_ctx();
  ctx->device = device;
  ctx->budget = hbm_budget_bytes;
  e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete ctx;
    return cuda_error(e, "cudaStreamCreate");
  }
  ctx->stream = ctx->own_stream;
  e = cudaMalloc(&ctx->d_err, 256);
  if (e != cudaSuccess) {
    cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return cuda_error(e, "cudaMalloc");
  }
  cudaMemset(ctx->d_err, 0, 256);
  ctx->device_bytes = 256;
  *out = ctx;
  return LINON_OK;
  LINON_TRY_END
}

int linon_destroy(linon_ctx* ctx) {
  if (!ctx) return LINON_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  dev_free(ctx, ctx->scene_block);
  dev_free(ctx, ctx->face_rgb);
  dev_free(ctx, ctx->scratch);
  dev_free(ctx, ctx->host_io);
  dev_free(ctx, ctx->grid);
  dev_free(ctx, ctx->cells);
  dev_free(ctx, ctx->cell_tris);
  linon::batch_release(ctx);
  if (ctx->d_err) cudaFree(ctx->d_err);
  for (cudaStream_t s : ctx->band_stream)
    if (s) cudaStreamDestroy(s);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  for (cudaEvent_t e : ctx->band_done)
    if (e) cudaEventDestroy(e);
  if (ctx->band_start) cudaEventDestroy(ctx->band_start);
  if (ctx->copies_done) cudaEventDestroy(ctx->copies_done);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return LINON_OK;
}

int linon_set_stream(linon_ctx* ctx, void* stream) {
  if (int st = enter(ctx)) return st;
  ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
  return LINON_OK;
}

int linon_synchronize(linon_ctx* ctx) {
  if (int st = enter(ctx)) return st;
  LINON_CUDA(cudaStreamSynchronize(ctx->stream));
  int err = 0;
  LINON_CUDA(cudaMemcpy(&err, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) {
    cudaMemset(ctx->d_err, 0, sizeof(int));
    return set_error(LINON_ETIMEOUT, "a kernel reported a bounded-wait timeout or traversal overflow (flags " +
                                         std::to_string(err) + ")");
  }
  return LINON_OK;
}

size_t linon_device_bytes(const linon_ctx* ctx) { return ctx ? ctx->device_bytes : 0; }

int linon_scene_upload(linon_ctx* ctx, const float* xyz, uint32_t n_vertices, const uint32_t* abc,
                       uint32_t n_faces, const float* face_rgb, int build_bvh) {
  LINON_TRY_BEGIN
  if (int st = enter(ctx)) return st;
  if ((n_vertices && !xyz) || (n_faces && !abc)) return set_error(LINON_EINVAL, "null scene arrays");
  if (n_faces > (1u << 27)) return set_error(LINON_EINVAL, "too many faces (max 2^27)");
  for (uint64_t i = 0; i < uint64_t(n_faces) * 3; ++i)
    if (abc[i] >= n_vertices)
      return set_error(LINON_EINVAL, "face " + std::to_string(i / 3) + " references vertex " +
                                         std::to_string(abc[i]) + " >= " + std::to_string(n_vertices));
  BvhBuild b;
  build_scene_arrays(xyz, n_vertices, abc, n_faces, build_bvh != 0, b);
  const size_t bytes = sizeof(float4) * (b.nodes.size() + b.tris.size());
  LINON_CUDA(cudaStreamSynchronize(ctx->stream));
  dev_free(ctx, ctx->scene_block);
  dev_free(ctx, ctx->face_rgb);
  dev_free(ctx, ctx->grid);
  dev_free(ctx, ctx->cells);
  dev_free(ctx, ctx->cell_tris);
  ctx->has_scene = false;
  if (int st = dev_alloc(ctx, ctx->scene_block, std::max<size_t>(bytes, 16))) return st;
  if (!b.nodes.empty())
    LINON_CUDA(cudaMemcpy(ctx->scene_block.p, b.nodes.data(), sizeof(float4) * b.nodes.size(),
                          cudaMemcpyHostToDevice));
  if (!b.tris.empty())
    LINON_CUDA(cudaMemcpy(static_cast<float4*>(ctx->scene_block.p) + b.nodes.size(), b.tris.data(),
                          sizeof(float4) * b.tris.size(), cudaMemcpyHostToDevice));
  if (face_rgb) {
    std::vector<float4> c(n_faces);
    for (uint32_t f = 0; f < n_faces; ++f)
      c[f] = make_float4(face_rgb[3 * f], face_rgb[3 * f + 1], face_rgb[3 * f + 2], 0.0f);
    if (int st = dev_alloc(ctx, ctx->face_rgb, sizeof(float4) * std::max<uint32_t>(n_faces, 1))) return st;
    LINON_CUDA(cudaMemcpy(ctx->face_rgb.p, c.data(), sizeof(float4) * n_faces, cudaMemcpyHostToDevice));
  }
  ctx->n_tris = int(n_faces);
  ctx->n_nodes = int(b.nodes.size() / 2);
  ctx->max_depth = b.max_depth;
  ctx->margin = b.margin;
  // small scenes are staged in shared memory by one TMA bulk copy per CTA
  ctx->staged_bytes = bytes <= 16384 && bytes > 0 ? int(bytes) : 0;
  // distance grid over the root box plus a border of two cells, 128 cells
  // along the longest axis (at most 2^22 cells); skipped when the HBM budget
  // cannot hold it (the march then queries the BVH)
  dev_free(ctx, ctx->grid);
  dev_free(ctx, ctx->cells);
  dev_free(ctx, ctx->cell_tris);
  ctx->reach = 0.0f;
  ctx->gx = ctx->gy = ctx->gz = 0;
  ctx->gcell = 0.0f;
  if (!b.nodes.empty()) {
    const float4 lo = b.nodes[0], hi = b.nodes[1];
    const float ext[3] = {hi.x - lo.x, hi.y - lo.y, hi.z - lo.z};
    const float emax = std::max(ext[0], std::max(ext[1], ext[2]));
    if (std::isfinite(emax) && emax > 0.0f) {
      float cell = emax / 128.0f;
      int dims[3];
      for (;;) {
        size_t total = 1;
        for (int k = 0; k < 3; ++k) {
          dims[k] = int(std::ceil(ext[k] / cell)) + 4;
          total *= size_t(dims[k]);
        }
        if (total <= (size_t(1) << 22)) break;
        cell *= 1.25f;
      }
      const size_t gbytes = sizeof(float) * size_t(dims[0]) * dims[1] * dims[2];
      if (!ctx->budget || ctx->device_bytes + gbytes <= ctx->budget) {
        if (int st = dev_alloc(ctx, ctx->grid, gbytes)) return st;
        ctx->gx = dims[0];
        ctx->gy = dims[1];
        ctx->gz = dims[2];
        ctx->gox = lo.x - 2.0f * cell;
        ctx->goy = lo.y - 2.0f * cell;
        ctx->goz = lo.z - 2.0f * cell;
        ctx->gcell = cell;
        ctx->has_scene = true;
        const DevScene s = dev_scene(ctx);
        LINON_CUDA(launch_grid_build(s, static_cast<float*>(ctx->grid.p), ctx->stream));
        LINON_CUDA(cudaStreamSynchronize(ctx->stream));
        if (int st = build_cell_lists(ctx)) return st;
      }
    }
  }
  ctx->has_scene = true;
  return LINON_OK;
  LINON_TRY_END
}

int linon_scene_info(const linon_ctx* ctx, uint32_t* n_faces, uint32_t* n_nodes, uint32_t* max_depth) {
  if (!ctx) return set_error(LINON_EINVAL, "null context");
  if (n_faces) *n_faces = uint32_t(ctx->n_tris);
  if (n_nodes) *n_nodes = uint32_t(ctx->n_nodes);
  if (max_depth) *max_depth = ctx->max_depth;
  return LINON_OK;
}

int linon_wgsl_translate(const char* field_body, const char* helpers_src, char* out, size_t out_cap,
                         char* log, size_t log_cap) {
  LINON_TRY_BEGIN
  if (!field_body) return set_error(LINON_EINVAL, "null field body");
  wgslfe::Translation t = wgslfe::translate(field_body, helpers_src ? helpers_src : "", "linon_user");
  if (!t.ok) {
    copy_log(t.log, log, log_cap);
    return set_error(LINON_ECOMPILE, t.log);
  }
  if (out && out_cap) {
    if (t.code.size() + 1 > out_cap) return set_error(LINON_EINVAL, "output buffer too small");
    copy_log(t.code, out, out_cap);
  }
  copy_log("", log, log_cap);
  return LINON_OK;
  LINON_TRY_END
}

int linon_field_validate(const char* field_body, const char* helpers_src, int flags, char* log,
                         size_t log_cap) {
  LINON_TRY_BEGIN
  if (!field_body) return set_error(LINON_EINVAL, "null field body");
  wgslfe::Translation t = wgslfe::translate(field_body, helpers_src ? helpers_src : "", "linon_user");
  if (!t.ok) {
    copy_log(t.log, log, log_cap);
    return set_error(LINON_ECOMPILE, t.log);
  }
  std::string jlog;
  size_t bytes = 0;
  const bool precise = (flags & LINON_COMPILE_PRECISE) != 0;
  // the reference's variant (t-loop, adaptive) and the fixed-step Kahan
  // variant, each with and without the field_weight == 1 specialisation
  int st = jit_check(module_source(t.code, {1, 9, 6, 14}, true), precise, jlog, &bytes);
  if (st == LINON_OK && (flags & LINON_VALIDATE_BATCHED)) {
    // the batched kernels (persistent and one CTA per tile) with this field
    linon_field tmp;
    tmp.cuda = t.code;
    std::string blog;
    st = jit_check(batched_module_source({&tmp}), precise, blog, &bytes);
    jlog += blog;
  }
  if (st == LINON_OK && !precise) {
    // the pair form (two rays per thread), when the field has one: its
    // absence or a compile failure only means one ray per thread
    wgslfe::Translation tp = wgslfe::translate(field_body, helpers_src ? helpers_src : "", "linon_user", true);
    std::string plog;
    size_t pbytes = 0;
    const int pst = tp.ok && !tp.has_private ? jit_check(module_source_pair(tp.code, 14 | 16), false, plog, &pbytes)
                                             : LINON_ECOMPILE;
    jlog += pst == LINON_OK ? "\npair form: compiles\n" + plog : "\npair form: not available\n";
  }
  copy_log(jlog, log, log_cap);
  if (st != LINON_OK) return set_error(st, jlog);
  return LINON_OK;
  LINON_TRY_END
}

int linon_field_compile(linon_ctx* ctx, const char* field_body, const char* helpers_src, int flags,
                        linon_field** out, char* log, size_t log_cap) {
  LINON_TRY_BEGIN
  if (int st = enter(ctx)) return st;
  if (!field_body || !out) return set_error(LINON_EINVAL, "null field body or output pointer");
  *out = nullptr;
  wgslfe::Translation t = wgslfe::translate(field_body, helpers_src ? helpers_src : "", "linon_user");
  if (!t.ok) {
    copy_log(t.log, log, log_cap);
    return set_error(LINON_ECOMPILE, t.log);
  }
  const bool precise = (flags & LINON_COMPILE_PRECISE) != 0;
  std::shared_ptr<JitModule> mod;
  std::string jlog;
  const std::vector<int> base = {base_variant(precise)};
  int st = jit_compile(module_source(t.code, base, true), precise, module_kernels(base, true), mod, jlog);
  if (st != LINON_OK) {
    std::string msg = st == LINON_ECOMPILE ? jlog : g_last_error;
    copy_log(msg, log, log_cap);
    return set_error(st, msg);
  }
  auto* f = new linon_field();
  f->ctx = ctx;
  f->body = field_body;
  f->helpers = helpers_src ? helpers_src : "";
  f->cuda = t.code;
  // no pair form with var<private> state: an integer or boolean private
  // variable would be one value for both rays of a thread
  if (!precise && !t.has_private) {
    wgslfe::Translation tp = wgslfe::translate(field_body, helpers_src ? helpers_src : "", "linon_user", true);
    if (tp.ok) f->cuda_pair = tp.code;
  }
  f->stateful = t.has_private;
  f->flags = flags;
  f->flops_arith = t.flops_arith;
  f->flops_transc = t.flops_transc;
  f->mod = mod;
  copy_log(jlog, log, log_cap);
  *out = f;
  return LINON_OK;
  LINON_TRY_END
}

int linon_field_release(linon_ctx* ctx, linon_field* field) {
  if (!field) return LINON_OK;
  if (field->ctx != ctx) return set_error(LINON_EINVAL, "field belongs to another context");
  delete field;  // the compiled module stays cached for the process
  return LINON_OK;
}

int linon_field_pair_state(const linon_field* field) {
  if (!field) return -1;
  if (field->cuda_pair.empty()) return -1;
  return field->pair_state;
}

int linon_field_flops(const linon_field* field, int32_t* arith, int32_t* transcendental) {
  if (!field) return set_error(LINON_EINVAL, "null field");
  if (arith) *arith = field->flops_arith;
  if (transcendental) *transcendental = field->flops_transc;
  return LINON_OK;
}

const char* linon_field_cuda_source(const linon_field* field) {
  return field ? field->cuda.c_str() : nullptr;
}

namespace {

int render_checks(linon_ctx* ctx, const linon_field* field, const linon_camera* camera,
                  const linon_march_params* params, int32_t width, int32_t height) {
  if (int st = field_valid(ctx, field)) return st;
  if (!camera) return set_error(LINON_EINVAL, "null camera");
  if (int st = check_params(params)) return st;
  if (int st = check_frame_size(width, height)) return st;
  if (!ctx->has_scene) return set_error(LINON_ENOSCENE, "render before linon_scene_upload");
  return LINON_OK;
}

// One launch of the plain march kernel over rows [row0, row1) of the frame
// (any rows: the 8x16 tiles start at row0, and a pixel's ray depends on its
// own row and column alone).
int launch_rows(linon_ctx* ctx, const linon_field* field, const linon_camera* camera,
                const linon_settings* settings, const linon_march_params* params, const linon_frame* out,
                int row0, int row1, cudaStream_t stream) {
  MarchArgs a;
  a.m = dev_march(settings, params);
  a.cam = dev_camera(camera);
  a.scene = dev_scene(ctx);
  a.frame.W = out->width;
  a.frame.H = out->height;
  a.frame.color = reinterpret_cast<uchar4*>(out->color);
  a.frame.mapping = reinterpret_cast<float4*>(out->mapping);
  a.frame.hit = out->hit_id;
  a.frame.steps = out->steps;
  a.tile_w = 8;
  a.tile_h = 16;
  a.row0 = row0;
  a.row1 = row1;
  a.err = ctx->d_err;
  cudaKernel_t k;
  const bool precise = (field->flags & LINON_COMPILE_PRECISE) != 0;
  const int v = march_variant(params, settings, precise);
  // Two rays per thread (march_pair_kernel) for fixed step budgets without
  // adaptive retries, early stop or linear mode, when the field has a pair
  // form that compiles (the first such render compiles it).  Pairs halve
  // the FP32 issue of the field and the step but leave the FMA pipe's work
  // as it is, run sines and cosines lane by lane, and hold more registers
  // (fewer warps per SM, CTAs with twice the work).  Measured at 1080p x
  // 4000 steps (ms, one ray / two rays per thread; FP32 operations and
  // transcendentals per evaluation): translation_x (4, 0) 11.76 / 10.87,
  // roessler (6, 0) 15.47 / 14.29, lorenz (8, 0) 19.72 / 18.58, scaled
  // Lorenz (14, 0) 21.10 / 20.13, lens (24, 1) 29.25 / 27.63; but linear
  // (0, 0) 6.34 / 8.02, twist (16, 2) 19.58 / 21.84, rotation (28, 2)
  // 26.52 / 27.13, and the scaled Lorenz field at 1024^2 x 2000 (under 8
  // waves of pair CTAs) 7.05 / 8.34.  Rule: at least 4 FP32 operations and
  // at most one transcendental per evaluation, and a frame of at least 8
  // waves of the pair kernel's resident CTAs.
  // LINON_RAY_PAIRS=0 / =1 forces one ray / two rays per thread.
  const char* force = std::getenv("LINON_RAY_PAIRS");
  bool pairs = !precise && (v & 4) && !(v & 1) && !params->stop_on_hit && !params->linear_mode &&
               !field->cuda_pair.empty() && field->pair_state >= 0 && !(force && force[0] == '0');
  if (pairs && !(force && force[0] == '1'))
    pairs = field->flops_arith >= 4 && field->flops_transc <= 1;
  if (pairs) {
    if (march_kernel(field, v | 16, &k) == LINON_OK) {
      field->pair_state = 1;
      if (!(force && force[0] == '1')) {
        int occ = 0, sms = 0;
        LINON_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void*)k, 128,
                                                                 size_t(a.scene.staged_bytes)));
        LINON_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
        // the whole frame's CTAs: row bands of one frame (linon_render_host)
        // are launched back to back on two streams and overlap
        const long long ctas = (long long)((out->width + 15) / 16) * ((out->height + 15) / 16);
        pairs = ctas >= 8LL * sms * std::max(occ, 1);
      }
      if (pairs) a.tile_w = 16;
    } else {
      field->pair_state = -1;
      pairs = false;
    }
  }
  if (!pairs)
    if (int st = march_kernel(field, v, &k)) return st;
  dim3 grid((out->width + a.tile_w - 1) / a.tile_w, (row1 - row0 + a.tile_h - 1) / a.tile_h);
  void* args[] = {&a};
  LINON_CUDA(cudaLaunchKernel((const void*)k, grid, dim3((pairs ? a.tile_w / 2 : a.tile_w) * a.tile_h), args,
                              size_t(a.scene.staged_bytes), stream));
  return LINON_OK;
}

}  // namespace

int linon_render(linon_ctx* ctx, const linon_field* field, const linon_camera* camera,
                 const linon_settings* settings, const linon_march_params* params,
                 const linon_frame* out) {
  LINON_TRY_BEGIN
  if (int st = enter(ctx)) return st;
  if (!out) return set_error(LINON_EINVAL, "null frame");
  if (int st = render_checks(ctx, field, camera, params, out->width, out->height)) return st;
  return launch_rows(ctx, field, camera, settings, params, out, 0, out->height, ctx->stream);
  LINON_TRY_END
}

int linon_render_rows(linon_ctx* ctx, const linon_field* field, const linon_camera* camera,
                      const linon_settings* settings, const linon_march_params* params,
                      const linon_frame* out, int32_t row0, int32_t row1) {
  LINON_TRY_BEGIN
  if (int st = enter(ctx)) return st;
  if (!out) return set_error(LINON_EINVAL, "null frame");
  if (int st = render_checks(ctx, field, camera, params, out->width, out->height)) return st;
  if (row0 < 0 || row1 < row0 || row1 > out->height)
    return set_error(LINON_EINVAL, "rows must satisfy 0 <= row0 <= row1 <= height");
  if (row0 == row1) return LINON_OK;
  return launch_rows(ctx, field, camera, settings, params, out, row0, row1, ctx->stream);
  LINON_TRY_END
}

int linon_field_eval(linon_ctx* ctx, const linon_field* field, const float* in, float* out, int64_t n) {
  LINON_TRY_BEGIN
  if (int st = enter(ctx)) return st;
  if (int st = field_valid(ctx, field)) return st;
  if (n < 0 || n > (int64_t(1) << 31) - 1) return set_error(LINON_EINVAL, "n out of range");
  if (n == 0) return LINON_OK;
  if (!in || !out) return set_error(LINON_EINVAL, "null field_eval buffers");
  cudaKernel_t k = field->mod->kernels.at("linon_field_eval");
  int nn = int(n);
  void* args[] = {&in, &out, &nn};
  LINON_CUDA(cudaLaunchKernel((const void*)k, dim3(unsigned((n + 255) / 256)), dim3(256), args, 0, ctx->stream));
  return LINON_OK;
  LINON_TRY_END
}

int linon_render_host(linon_ctx* ctx, const linon_field* field, const linon_camera* camera,
                      const linon_settings* settings, const linon_march_params* params,
                      int32_t width, int32_t height, uint8_t* color, float* mapping, int32_t* hit_id,
                      int32_t* steps) {
  LINON_TRY_BEGIN
  if (int st = enter(ctx)) return st;
  if (int st = render_checks(ctx, field, camera, params, width, height)) return st;
  const size_t n = size_t(width) * height;
  const size_t need = n * (4 + 16 + 4 + 4) + 64;
  if (int st = dev_alloc(ctx, ctx->host_io, need)) return st;
  char* base = static_cast<char*>(ctx->host_io.p);
  linon_frame f;
  f.width = width;
  f.height = height;
  f.mapping = mapping ? reinterpret_cast<float*>(base) : nullptr;
  f.color = color ? reinterpret_cast<uint8_t*>(base + n * 16) : nullptr;
  f.hit_id = hit_id ? reinterpret_cast<int32_t*>(base + n * 20) : nullptr;
  f.steps = steps ? reinterpret_cast<int32_t*>(base + n * 24) : nullptr;
  // Bands of rows: each band's planes go to the host while later bands
  // render (the kernel is compute-bound, the copies ride on the copy
  // engine); consecutive bands alternate between two streams so one band's
  // last CTAs overlap the next band's first.  Small frames take one band.
  const int tile_h = 16;
  const int nb = n >= (size_t(1) << 18) ? 8 : 1;
  const int band = ((height + nb - 1) / nb + tile_h - 1) / tile_h * tile_h;
  if (!ctx->copy_stream) {
    for (auto& s : ctx->band_stream) LINON_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    LINON_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    for (auto& e : ctx->band_done) LINON_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    LINON_CUDA(cudaEventCreateWithFlags(&ctx->band_start, cudaEventDisableTiming));
    LINON_CUDA(cudaEventCreateWithFlags(&ctx->copies_done, cudaEventDisableTiming));
  }
  // the bands start after the work already queued on the context's stream
  LINON_CUDA(cudaEventRecord(ctx->band_start, ctx->stream));
  for (auto s : ctx->band_stream) LINON_CUDA(cudaStreamWaitEvent(s, ctx->band_start, 0));
  int b = 0;
  for (int r0 = 0; r0 < height; r0 += band, ++b) {
    const int r1 = std::min(height, r0 + band);
    cudaStream_t s = ctx->band_stream[b & 1];
    if (int st = launch_rows(ctx, field, camera, settings, params, &f, r0, r1, s)) return st;
    LINON_CUDA(cudaEventRecord(ctx->band_done[b], s));
    LINON_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->band_done[b], 0));
    const size_t p0 = size_t(r0) * width, pn = size_t(r1 - r0) * width;
    if (mapping)
      LINON_CUDA(cudaMemcpyAsync(mapping + 4 * p0, f.mapping + 4 * p0, pn * 16, cudaMemcpyDeviceToHost,
                                 ctx->copy_stream));
    if (color)
      LINON_CUDA(cudaMemcpyAsync(color + 4 * p0, f.color + 4 * p0, pn * 4, cudaMemcpyDeviceToHost,
                                 ctx->copy_stream));
    if (hit_id)
      LINON_CUDA(cudaMemcpyAsync(hit_id + p0, f.hit_id + p0, pn * 4, cudaMemcpyDeviceToHost, ctx->copy_stream));
    if (steps)
      LINON_CUDA(cudaMemcpyAsync(steps + p0, f.steps + p0, pn * 4, cudaMemcpyDeviceToHost, ctx->copy_stream));
  }
  // later work on the context's stream follows the copies
  LINON_CUDA(cudaEventRecord(ctx->copies_done, ctx->copy_stream));
  LINON_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->copies_done, 0));
  return linon_synchronize(ctx);
  LINON_TRY_END
}

int linon_overlay(linon_ctx* ctx, const linon_settings* settings, int32_t width, int32_t height,
                  const uint8_t* ray_casting, const float* mapping, uint8_t* target, float* exponents,
                  int srgb, int fp64) {
  LINON_TRY_BEGIN
  if (int st = enter(ctx)) return st;
  if (!settings || !ray_casting || !target) return set_error(LINON_EINVAL, "null overlay argument");
  if (int st = check_frame_size(width, height)) return st;
  if (settings->overlay_mode == 1 && !mapping) return set_error(LINON_EINVAL, "overlay mode 1 needs the mapping");
  if (settings->central_difference_delta < 1 || settings->central_difference_delta > 10000)
    return set_error(LINON_EINVAL, "central_difference_delta must be in 1..10000");
  OverlayArgs a;
  a.in = reinterpret_cast<const uchar4*>(ray_casting);
  a.mapping = reinterpret_cast<const float4*>(mapping);
  a.out = reinterpret_cast<uchar4*>(target);
  a.exponents = exponents;
  a.W = width;
  a.H = height;
  a.mode = settings->overlay_mode;
  a.delta = settings->central_difference_delta;
  a.scaling = settings->lyapunov_scaling;
  a.srgb = srgb;
  LINON_CUDA(launch_overlay(a, fp64 != 0, ctx->stream));
  return LINON_OK;
  LINON_TRY_END
}

int linon_ftle(linon_ctx* ctx, const linon_camera* camera, const linon_march_params* params,
               int32_t width, int32_t height, const float* mapping, float horizon_T, float* exponents) {
  LINON_TRY_BEGIN
  if (int st = enter(ctx)) return st;
  if (!camera || !params || !mapping || !exponents) return set_error(LINON_EINVAL, "null ftle argument");
  if (int st = check_frame_size(width, height)) return st;
  if (!(horizon_T > 0.0f)) return set_error(LINON_EINVAL, "horizon T must be positive");
  FtleArgs a;
  a.cam = dev_camera(camera);
  a.mapping = reinterpret_cast<const float4*>(mapping);
  a.out = exponents;
  a.W = width;
  a.H = height;
  a.focal_length = params->focal_length;
  a.viewport_height = params->viewport_height;
  a.half_over_T = 0.5 / double(horizon_T);
  LINON_CUDA(launch_ftle(a, ctx->stream));
  return LINON_OK;
  LINON_TRY_END
}

int linon_capture_reference(linon_ctx* ctx, const linon_field* field, const linon_camera* camera,
                            const linon_settings* settings, const linon_march_params* params,
                            int32_t width, int32_t height, const float* positions,
                            linon_ray_sample* out) {
  LINON_TRY_BEGIN
  if (int st = enter(ctx)) return st;
  if (int st = field_valid(ctx, field)) return st;
  if (!camera || !settings || !params || !out) return set_error(LINON_EINVAL, "null capture argument");
  if (int st = check_frame_size(width, height)) return st;
  float pos[16];
  if (positions) std::memcpy(pos, positions, sizeof pos);
  else reference_ring(settings, pos);
  // 8 rays x 100 samples: h = 0.001, 5000 steps, every 50th (main_view.wgsl:286-309)
  const size_t tmp_off = 256;
  if (int st = dev_alloc(ctx, ctx->scratch, std::max<size_t>(ctx->scratch.bytes, tmp_off + sizeof(float4) * 800)))
    return st;
  float4* tmp = reinterpret_cast<float4*>(static_cast<char*>(ctx->scratch.p) + tmp_off);
  if (int st = launch_capture(ctx, field, camera, settings, params, width, height, pos, 8, 0.001f,
                              5000, 50, 0, tmp, 100))
    return st;
  LINON_CUDA(launch_pack_samples(tmp, out, 8, 100, ctx->stream));
  return LINON_OK;
  LINON_TRY_END
}

int linon_capture_paths(linon_ctx* ctx, const linon_field* field, const linon_camera* camera,
                        const linon_settings* settings, const linon_march_params* params, int32_t width,
                        int32_t height, const float* pos_xy, int32_t n_rays, float h, int32_t n_steps,
                        int32_t record_every, float* out) {
  LINON_TRY_BEGIN
  if (int st = enter(ctx)) return st;
  if (int st = field_valid(ctx, field)) return st;
  if (!camera || !params || !pos_xy || !out) return set_error(LINON_EINVAL, "null capture argument");
  if (int st = check_frame_size(width, height)) return st;
  if (n_rays <= 0 || n_rays > (1 << 20)) return set_error(LINON_EINVAL, "n_rays must be in 1..2^20");
  if (n_steps < 0 || n_steps > 10000000) return set_error(LINON_EINVAL, "n_steps must be in 0..1e7");
  if (record_every <= 0) return set_error(LINON_EINVAL, "record_every must be positive");
  if (!(h > 0.0f) || !std::isfinite(h)) return set_error(LINON_EINVAL, "h must be positive");
  const int32_t n_points = (n_steps + record_every - 1) / record_every + 1;
  return launch_capture(ctx, field, camera, settings, params, width, height, pos_xy, n_rays, h, n_steps,
                        record_every, 1, reinterpret_cast<float4*>(out), n_points);
  LINON_TRY_END
}

int linon_outline_select(linon_ctx* ctx, const float* exponents, int32_t width, int32_t height,
                         float min_exp, int32_t* pix_out, float* pos_out) {
  LINON_TRY_BEGIN
  if (int st = enter(ctx)) return st;
  if (!exponents || !pix_out) return set_error(LINON_EINVAL, "null outline argument");
  if (int st = check_frame_size(width, height)) return st;
  const size_t off = 256 + sizeof(float4) * 800;
  if (int st = dev_alloc(ctx, ctx->scratch, std::max<size_t>(ctx->scratch.bytes, off + 9 * 8))) return st;
  unsigned long long* slots = reinterpret_cast<unsigned long long*>(static_cast<char*>(ctx->scratch.p) + off);
  LINON_CUDA(launch_outline(exponents, width, height, min_exp, slots, ctx->stream));
  unsigned long long k[9];
  LINON_CUDA(cudaMemcpyAsync(k, slots, sizeof k, cudaMemcpyDeviceToHost, ctx->stream));
  LINON_CUDA(cudaStreamSynchronize(ctx->stream));
  const uint64_t W = uint64_t(width), H = uint64_t(height);
  for (int g = 0; g < 8; ++g) {
    int64_t x = 0, y = 0;
    if (k[8] != 0) {
      if (g % 2 == 0) {
        uint64_t p = k[g] & 0xffffffffull;
        x = int64_t(p / H);
        y = int64_t(p % H);
      } else if (k[g] != ~0ull) {
        uint64_t p = k[g];
        switch (g) {
          case 1: y = int64_t(W - 1 - p / W); x = int64_t(p % W); break;
          case 3: x = int64_t(W - 1 - p / H); y = int64_t(p % H); break;
          case 5: y = int64_t(p / W); x = int64_t(p % W); break;
          case 7: x = int64_t(p / H); y = int64_t(p % H); break;
        }
      }
    }
    pix_out[2 * g] = int32_t(x);
    pix_out[2 * g + 1] = int32_t(y);
    if (pos_out) {
      // main_view.wgsl:467-468
      pos_out[2 * g] = float(x) / (float(width) - 1.0f);
      pos_out[2 * g + 1] = (float(height) - 1.0f - float(y)) / (float(height) - 1.0f);
    }
  }
  return LINON_OK;
  LINON_TRY_END
}

int linon_exponent_quantile(linon_ctx* ctx, const float* exponents, int32_t width, int32_t height,
                            int32_t border, double q, float* out) {
  LINON_TRY_BEGIN
  if (int st = enter(ctx)) return st;
  if (!exponents || !out) return set_error(LINON_EINVAL, "null quantile argument");
  if (int st = check_frame_size(width, height)) return st;
  if (border < 0 || 2 * border >= width || 2 * border >= height)
    return set_error(LINON_EINVAL, "border leaves no interior pixels");
  if (!(q >= 0.0 && q <= 1.0)) return set_error(LINON_EINVAL, "quantile must be in [0,1]");
  const size_t off = 256 + sizeof(float4) * 800 + 128;
  if (int st = dev_alloc(ctx, ctx->scratch, std::max<size_t>(ctx->scratch.bytes, off + 4096 * 4))) return st;
  unsigned* hist = reinterpret_cast<unsigned*>(static_cast<char*>(ctx->scratch.p) + off);
  const uint64_t n = uint64_t(width - 2 * border) * uint64_t(height - 2 * border);
  uint64_t rank = uint64_t(std::floor(q * double(n - 1)));  // nearest-rank (lower) quantile
  unsigned prefix = 0;
  const int passes[3][2] = {{20, 12}, {8, 12}, {0, 8}};  // (shift, bits)
  int high = 32;
  std::vector<unsigned> h(4096);
  for (int p = 0; p < 3; ++p) {
    const int shift = passes[p][0], bits = passes[p][1];
    LINON_CUDA(launch_quantile_hist(exponents, width, height, border, prefix, high, shift, bits, hist,
                                    ctx->stream));
    LINON_CUDA(cudaMemcpyAsync(h.data(), hist, sizeof(unsigned) << bits, cudaMemcpyDeviceToHost, ctx->stream));
    LINON_CUDA(cudaStreamSynchronize(ctx->stream));
    uint64_t acc = 0;
    int bin = (1 << bits) - 1;
    for (int b = 0; b < (1 << bits); ++b) {
      if (acc + h[size_t(b)] > rank) { bin = b; break; }
      acc += h[size_t(b)];
    }
    rank -= acc;
    prefix = (prefix << bits) | unsigned(bin);
    high = shift;
  }
  unsigned key = prefix;
  unsigned u = (key & 0x80000000u) ? (key & 0x7fffffffu) : ~key;
  float f;
  std::memcpy(&f, &u, 4);
  *out = f;
  return LINON_OK;
  LINON_TRY_END
}

int linon_outline_indices(uint16_t* out, size_t cap) {
  // src/ray_samples.rs:29-49: 4 sides of the 3x3 ring, 99 quads each
  const uint16_t sides[4][3] = {{0, 1, 2}, {2, 3, 4}, {4, 5, 6}, {6, 7, 0}};
  const uint16_t S = 100;
  const size_t need = 4 * 99 * 4 * 3;
  if (!out) return int(need);
  if (cap < need) return -set_error(LINON_EINVAL, "index buffer too small");
  size_t n = 0;
  for (auto& s : sides) {
    for (uint16_t i = 0; i + 1 < S; ++i) {
      const uint16_t a = uint16_t(s[0] * S + i), b = uint16_t(s[1] * S + i), c = uint16_t(s[2] * S + i);
      const uint16_t tri[4][3] = {{a, uint16_t(b + 1), uint16_t(a + 1)},
                                  {a, b, uint16_t(b + 1)},
                                  {b, c, uint16_t(b + 1)},
                                  {c, uint16_t(c + 1), uint16_t(b + 1)}};
      for (auto& t : tri)
        for (uint16_t v : t) out[n++] = v;
    }
  }
  return int(n);
}

int linon_check_bounded_wait(linon_ctx* ctx, int32_t polls) {
  LINON_TRY_BEGIN
  if (int st = enter(ctx)) return st;
  if (polls < 1 || polls > (1 << 24)) return set_error(LINON_EINVAL, "polls must be in [1, 2^24]");
  LINON_CUDA(launch_bounded_wait_check(ctx->d_err, polls, ctx->stream));
  return linon_synchronize(ctx);
  LINON_TRY_END
}

int linon_probe_fp32_peak(linon_ctx* ctx, double* tflops) {
  LINON_TRY_BEGIN
  if (int st = enter(ctx)) return st;
  if (!tflops) return set_error(LINON_EINVAL, "null output");
  int sms = 0;
  LINON_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  const size_t off = 256 + sizeof(float4) * 800 + 128 + 4096 * 4;
  if (int st = dev_alloc(ctx, ctx->scratch, std::max<size_t>(ctx->scratch.bytes, off + 64))) return st;
  float* sink = reinterpret_cast<float*>(static_cast<char*>(ctx->scratch.p) + off);
  const int blocks = sms * 8, threads = 256, iters = 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  LINON_CUDA(launch_fp32_probe(sink, blocks, threads, 256, ctx->stream));  // warm-up
  double best = 0;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0, ctx->stream);
    LINON_CUDA(launch_fp32_probe(sink, blocks, threads, iters, ctx->stream));
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flops = double(blocks) * threads * iters * 16.0 * 8.0 * 2.0;
    best = std::max(best, flops / (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *tflops = best;
  return LINON_OK;
  LINON_TRY_END
}

}  // extern "C"
