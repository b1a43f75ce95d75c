// serve.cpp — continuous batching of ray-casting requests.
//
// The reference redraws one view per UI event (Application::render,
// src/application.rs:492-528; Enhance and Outline re-renders,
// src/main_view.rs:778-829; clicks trigger ray-sample capture,
// src/main_view.wgsl:377-480).  A serving deployment receives these as a
// stream of independent requests of different sizes.  Here a scheduler thread
// owns the context:
//   * submit() queues a request (inputs copied) and returns an id;
//   * requests are admitted in arrival order as long as their output memory
//     fits the HBM budget (outputs come from the stream-ordered pool);
//   * each admitted group (a wave) goes to a free slot (a pair of streams):
//     frames / Enhance re-renders / overlay renders of the wave in ONE
//     batched launch (the configured schedule), then the overlays, while
//     captures run on the slot's second stream;
//   * up to `slots` waves are on the GPU at once, so requests that arrive
//     while a wave runs start in the next slot without waiting for it;
//   * completion is detected by polling the waves' events; results stay on
//     the device until released.
// Scene, compiled fields and the batch module stay resident for the life of
// the server.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <thread>

#include "internal.hpp"
#include "kernels.hpp"

namespace linon {
namespace {

using Clock = std::chrono::steady_clock;

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct Request {
  uint64_t id = 0;
  linon_request req{};
  std::vector<float> pos;  // capture positions (copied at submit)
  int status = LINON_EBUSY;
  bool done = false, released = false;
  double t_submit = 0, t_admit = 0, t_done = 0;
  size_t bytes = 0;
  char* dev = nullptr;
  linon_result res{};
  int n_points = 0;
};

struct Slot {
  cudaStream_t main = nullptr, aux = nullptr;
  cudaEvent_t ev_main = nullptr, ev_aux = nullptr;
  BatchView* views_dev = nullptr;
  unsigned long long* counter = nullptr;
  unsigned long long* sums_host = nullptr;  // pinned
  unsigned long long* sums_dev = nullptr;
  bool busy = false;
  std::vector<Request*> reqs;
  int wave = -1;
};

}  // namespace
}  // namespace linon

struct linon_server {
  linon_ctx* ctx = nullptr;
  std::vector<const linon_field*> fields;
  std::shared_ptr<linon::JitModule> mod;
  linon_serve_config cfg{};
  linon_batch_tuning tuning{};
  std::vector<linon::Slot> slots;
  cudaStream_t free_stream = nullptr;
  std::mutex mu;
  std::condition_variable cv, done_cv;
  std::deque<linon::Request*> pending;
  std::map<uint64_t, std::unique_ptr<linon::Request>> all;
  uint64_t next_id = 1;
  size_t used = 0, peak = 0;
  uint64_t submitted = 0, completed = 0, failed = 0, waves = 0;
  bool stop = false;
  int sticky = 0;  // a CUDA error that poisoned the server
  std::string sticky_msg;
  std::thread th;
  linon::Clock::time_point t0;
};

namespace linon {
namespace {

double now_ms(const linon_server* s) {
  return std::chrono::duration<double, std::milli>(Clock::now() - s->t0).count();
}

size_t request_bytes(const linon_request& r, int* n_points) {
  size_t b = 0;
  *n_points = 0;
  if (r.kind == LINON_REQ_CAPTURE) {
    *n_points = (r.n_steps + r.record_every - 1) / r.record_every + 1;
    b += align256(sizeof(float) * 2 * size_t(r.n_rays));
    b += align256(size_t(r.n_rays) * size_t(*n_points) * 16);
    return b;
  }
  const size_t n = size_t(r.width) * size_t(r.height);
  b += align256(n * 16) + align256(n * 4) * 3;  // mapping, color, hit, steps
  if (r.kind == LINON_REQ_OVERLAY) b += align256(n * 4) * 2;  // target, exponents
  return b;
}

int validate_request(const linon_server* s, const linon_request& r) {
  if (r.kind < LINON_REQ_FRAME || r.kind > LINON_REQ_CAPTURE) return set_error(LINON_EINVAL, "unknown request kind");
  if (r.field_index < 0 || r.field_index >= int(s->fields.size()))
    return set_error(LINON_EINVAL, "field_index out of range");
  if (r.width <= 0 || r.height <= 0 || r.width > 65535 || r.height > 65535)
    return set_error(LINON_EINVAL, "bad image size");
  const linon_march_params& p = r.params;
  if (r.kind == LINON_REQ_CAPTURE) {
    if (r.n_rays <= 0 || r.n_rays > (1 << 20) || !r.pos_xy) return set_error(LINON_EINVAL, "capture needs 1..2^20 rays and positions");
    if (r.n_steps < 0 || r.n_steps > 10000000 || r.record_every <= 0 || !(r.h > 0.0f))
      return set_error(LINON_EINVAL, "bad capture steps");
    return LINON_OK;
  }
  if (!(p.h_initial > 0.0f) || p.max_steps < 0 || p.max_steps > 50000000)
    return set_error(LINON_EINVAL, "bad march parameters");
  if (p.max_steps == 0) {
    float hmin = p.adaptive ? std::min(p.h_initial, p.h_fine) : p.h_initial;
    if (!(hmin > 0.0f) || double(p.t_max) / hmin > 5e7 || std::fabs(p.t_max) + hmin == std::fabs(p.t_max))
      return set_error(LINON_EINVAL, "t-loop would not terminate");
  }
  if (r.kind == LINON_REQ_OVERLAY &&
      (r.settings.central_difference_delta < 1 || r.settings.central_difference_delta > 10000))
    return set_error(LINON_EINVAL, "central_difference_delta must be in 1..10000");
  return LINON_OK;
}

void fill_result(Request* q) {
  linon_result& o = q->res;
  o.kind = q->req.kind;
  o.n_points = q->n_points;
  if (!q->dev) return;
  char* p = q->dev;
  if (q->req.kind == LINON_REQ_CAPTURE) {
    p += align256(sizeof(float) * 2 * size_t(q->req.n_rays));
    o.paths = reinterpret_cast<float*>(p);
    return;
  }
  const size_t n = size_t(q->req.width) * size_t(q->req.height);
  o.frame.width = q->req.width;
  o.frame.height = q->req.height;
  o.frame.mapping = reinterpret_cast<float*>(p);
  p += align256(n * 16);
  o.frame.color = reinterpret_cast<uint8_t*>(p);
  p += align256(n * 4);
  o.frame.hit_id = reinterpret_cast<int32_t*>(p);
  p += align256(n * 4);
  o.frame.steps = reinterpret_cast<int32_t*>(p);
  p += align256(n * 4);
  if (q->req.kind == LINON_REQ_OVERLAY) {
    o.overlay = reinterpret_cast<uint8_t*>(p);
    p += align256(n * 4);
    o.exponents = reinterpret_cast<float*>(p);
  }
}

// Enqueues one wave on a slot.  Called without the lock held.
int launch_wave(linon_server* s, Slot& sl) {
  linon_ctx* ctx = s->ctx;
  std::vector<linon_view> views;
  std::vector<Request*> renders;
  for (Request* q : sl.reqs) {
    if (q->req.kind == LINON_REQ_CAPTURE) {
      // positions at the front of the request's allocation
      float* pos = reinterpret_cast<float*>(q->dev);
      LINON_CUDA(cudaMemcpyAsync(pos, q->pos.data(), sizeof(float) * q->pos.size(), cudaMemcpyHostToDevice, sl.aux));
      CaptureArgs a;
      std::memset(&a, 0, sizeof a);
      for (int k = 0; k < 3; ++k) {
        a.cam.o[k] = q->req.camera.origin[k];
        a.cam.d[k] = q->req.camera.view_direction[k];
        a.cam.u[k] = q->req.camera.up[k];
      }
      a.pos = pos;
      a.out = reinterpret_cast<float4*>(q->res.paths);
      a.W = q->req.width;
      a.H = q->req.height;
      a.focal_length = q->req.params.focal_length;
      a.viewport_height = q->req.params.viewport_height;
      a.field_weight = q->req.settings.field_weight;
      a.h = q->req.h;
      a.n_rays = q->req.n_rays;
      a.n_steps = q->req.n_steps;
      a.every = q->req.record_every;
      a.n_points = q->n_points;
      a.record_final = 1;
      void* args[] = {&a};
      cudaKernel_t k = s->fields[size_t(q->req.field_index)]->mod->kernels.at("linon_capture");
      LINON_CUDA(cudaLaunchKernel((const void*)k, dim3(unsigned((a.n_rays + 31) / 32)), dim3(32), args, 0, sl.aux));
    } else {
      linon_view v{};
      v.camera = q->req.camera;
      v.settings = q->req.settings;
      v.params = q->req.params;
      v.width = q->req.width;
      v.height = q->req.height;
      v.field_index = q->req.field_index;
      v.out = q->res.frame;
      views.push_back(v);
      renders.push_back(q);
    }
  }
  if (!views.empty()) {
    std::vector<BatchView> tab;
    int n_blocks = 0;
    const long long total = batch_table(views.data(), int(views.size()), s->tuning, tab, &n_blocks);
    LINON_CUDA(cudaMemcpyAsync(sl.views_dev, tab.data(), sizeof(BatchView) * tab.size(), cudaMemcpyHostToDevice,
                               sl.main));
    if (int st = batch_launch(ctx, s->mod, s->tuning, sl.views_dev, int(views.size()), total, n_blocks, sl.counter,
                              sl.main, batch_kernel_name(views.data(), int(views.size()), s->tuning)))
      return st;
    for (size_t i = 0; i < renders.size(); ++i) {
      Request* q = renders[i];
      if (q->req.kind == LINON_REQ_OVERLAY) {
        OverlayArgs oa;
        oa.in = reinterpret_cast<const uchar4*>(q->res.frame.color);
        oa.mapping = reinterpret_cast<const float4*>(q->res.frame.mapping);
        oa.out = reinterpret_cast<uchar4*>(q->res.overlay);
        oa.exponents = q->res.exponents;
        oa.W = q->req.width;
        oa.H = q->req.height;
        oa.mode = 1;
        oa.delta = q->req.settings.central_difference_delta;
        oa.scaling = q->req.settings.lyapunov_scaling;
        oa.srgb = 0;
        LINON_CUDA(cudaMemsetAsync(q->res.exponents, 0, sizeof(float) * size_t(oa.W) * oa.H, sl.main));
        LINON_CUDA(launch_overlay(oa, q->req.fp64_overlay != 0, sl.main));
      }
      LINON_CUDA(launch_sum_steps(q->res.frame.steps, (long long)q->req.width * q->req.height, sl.sums_dev + i,
                                  sl.main));
    }
    LINON_CUDA(cudaMemcpyAsync(sl.sums_host, sl.sums_dev, sizeof(unsigned long long) * renders.size(),
                               cudaMemcpyDeviceToHost, sl.main));
  }
  LINON_CUDA(cudaEventRecord(sl.ev_main, sl.main));
  LINON_CUDA(cudaEventRecord(sl.ev_aux, sl.aux));
  return LINON_OK;
}

void finish_wave(linon_server* s, Slot& sl, int status) {
  const double t = now_ms(s);
  size_t ri = 0;
  for (Request* q : sl.reqs) {
    if (q->req.kind != LINON_REQ_CAPTURE) {
      q->res.ray_steps = status == LINON_OK ? int64_t(sl.sums_host[ri]) : 0;
      ++ri;
    } else {
      q->res.ray_steps = status == LINON_OK ? int64_t(q->req.n_rays) * q->req.n_steps : 0;
    }
    q->status = status;
    q->done = true;
    q->t_done = t;
    if (status == LINON_OK) s->completed++;
    else s->failed++;
  }
  sl.reqs.clear();
  sl.busy = false;
}

void scheduler(linon_server* s) {
  cudaSetDevice(s->ctx->device);
  std::unique_lock<std::mutex> lock(s->mu);
  for (;;) {
    // 1. retire finished waves
    bool any_busy = false;
    for (Slot& sl : s->slots) {
      if (!sl.busy) continue;
      cudaError_t a = cudaEventQuery(sl.ev_main), b = cudaEventQuery(sl.ev_aux);
      if (a == cudaSuccess && b == cudaSuccess) {
        finish_wave(s, sl, LINON_OK);
      } else if ((a != cudaSuccess && a != cudaErrorNotReady) || (b != cudaSuccess && b != cudaErrorNotReady)) {
        s->sticky = LINON_ECUDA;
        s->sticky_msg = std::string("wave failed: ") + cudaGetErrorString(a != cudaSuccess ? a : b);
        finish_wave(s, sl, LINON_ECUDA);
      } else {
        any_busy = true;
      }
    }
    s->done_cv.notify_all();
    if (s->stop && !any_busy) break;
    // 2. admit and launch a wave on a free slot
    Slot* free_slot = nullptr;
    for (Slot& sl : s->slots)
      if (!sl.busy) {
        free_slot = &sl;
        break;
      }
    if (free_slot && !s->pending.empty() && !s->stop && !s->sticky) {
      Slot& sl = *free_slot;
      while (!s->pending.empty() && int(sl.reqs.size()) < s->cfg.max_wave) {
        Request* q = s->pending.front();
        if (s->cfg.hbm_budget && s->used + q->bytes > s->cfg.hbm_budget) break;  // wait for memory
        void* p = nullptr;
        // allocated in the order of the stream that will use it
        cudaError_t e = cudaMallocAsync(&p, q->bytes, q->req.kind == LINON_REQ_CAPTURE ? sl.aux : sl.main);
        if (e != cudaSuccess) {
          cudaGetLastError();
          if (sl.reqs.empty() && !any_busy) {  // nothing will free memory: fail it
            s->pending.pop_front();
            q->status = LINON_ENOMEM;
            q->done = true;
            q->t_done = now_ms(s);
            s->failed++;
            continue;
          }
          break;
        }
        s->pending.pop_front();
        q->dev = static_cast<char*>(p);
        s->used += q->bytes;
        s->peak = std::max(s->peak, s->used);
        q->t_admit = now_ms(s);
        fill_result(q);
        sl.reqs.push_back(q);
      }
      if (!sl.reqs.empty()) {
        sl.busy = true;
        sl.wave = int(s->waves++);
        for (Request* q : sl.reqs) q->res.wave = sl.wave;
        lock.unlock();
        int st = launch_wave(s, sl);
        lock.lock();
        if (st != LINON_OK) {
          s->sticky = st;
          s->sticky_msg = std::string("wave launch failed: ") + linon_last_error();
          cudaStreamSynchronize(sl.main);
          cudaStreamSynchronize(sl.aux);
          finish_wave(s, sl, st);
        }
        continue;
      }
    }
    if (s->stop && s->pending.empty() && !any_busy) break;
    if (s->stop) {
      // fail what is still queued
      while (!s->pending.empty()) {
        Request* q = s->pending.front();
        s->pending.pop_front();
        q->status = LINON_ESTATE;
        q->done = true;
        q->t_done = now_ms(s);
        s->failed++;
      }
    }
    // 3. sleep: short while waves run (event polling), else until work arrives
    if (any_busy) s->cv.wait_for(lock, std::chrono::microseconds(20));
    else s->cv.wait_for(lock, std::chrono::milliseconds(50));
  }
  s->done_cv.notify_all();
}

void copy_result(const Request* q, linon_result* out) {
  *out = q->res;
  out->status = q->done ? q->status : LINON_EBUSY;
  out->t_submit_ms = q->t_submit;
  out->t_admit_ms = q->t_admit;
  out->t_done_ms = q->t_done;
}

}  // namespace
}  // namespace linon

using namespace linon;

extern "C" {

int linon_serve_start(linon_ctx* ctx, const linon_field* const* fields, int32_t n_fields,
                      const linon_serve_config* cfg, linon_server** out) {
  try {
    if (!ctx || !out) return set_error(LINON_EINVAL, "null context or output");
    *out = nullptr;
    if (!fields || n_fields <= 0 || n_fields > LINON_MAX_BATCH_FIELDS) return set_error(LINON_EINVAL, "1..8 fields");
    for (int i = 0; i < n_fields; ++i)
      if (!fields[i] || fields[i]->ctx != ctx) return set_error(LINON_EINVAL, "field of another context");
    if (!ctx->has_scene) return set_error(LINON_ENOSCENE, "serve before linon_scene_upload");
    LINON_CUDA(cudaSetDevice(ctx->device));
    auto s = std::make_unique<linon_server>();
    s->ctx = ctx;
    s->fields.assign(fields, fields + n_fields);
    if (cfg) s->cfg = *cfg;
    if (s->cfg.slots <= 0) s->cfg.slots = 2;
    if (s->cfg.slots > 8) s->cfg.slots = 8;
    if (s->cfg.max_wave <= 0) s->cfg.max_wave = 256;
    if (int st = batch_tuning(ctx, &s->cfg.tuning, s->tuning)) return st;
    if (any_stateful(fields, n_fields)) s->tuning.refill_below = 0;  // the queue of warp tiles instead
    if (int st = batch_module(ctx, fields, n_fields, s->tuning, s->mod)) return st;
    // keep freed pool memory cached (no release to the OS between waves)
    cudaMemPool_t pool;
    LINON_CUDA(cudaDeviceGetDefaultMemPool(&pool, ctx->device));
    uint64_t thr = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    s->slots.resize(size_t(s->cfg.slots));
    for (Slot& sl : s->slots) {
      LINON_CUDA(cudaStreamCreateWithFlags(&sl.main, cudaStreamNonBlocking));
      LINON_CUDA(cudaStreamCreateWithFlags(&sl.aux, cudaStreamNonBlocking));
      LINON_CUDA(cudaEventCreateWithFlags(&sl.ev_main, cudaEventDisableTiming));
      LINON_CUDA(cudaEventCreateWithFlags(&sl.ev_aux, cudaEventDisableTiming));
      LINON_CUDA(cudaMalloc(&sl.views_dev, sizeof(BatchView) * size_t(s->cfg.max_wave)));
      LINON_CUDA(cudaMalloc(&sl.counter, 256));
      LINON_CUDA(cudaMalloc(&sl.sums_dev, sizeof(unsigned long long) * size_t(s->cfg.max_wave)));
      LINON_CUDA(cudaMallocHost(&sl.sums_host, sizeof(unsigned long long) * size_t(s->cfg.max_wave)));
    }
    LINON_CUDA(cudaStreamCreateWithFlags(&s->free_stream, cudaStreamNonBlocking));
    s->t0 = Clock::now();
    linon_server* raw = s.release();
    raw->th = std::thread(scheduler, raw);
    *out = raw;
    return LINON_OK;
  } catch (const std::exception& e) {
    return set_error(LINON_EINVAL, std::string("internal error: ") + e.what());
  }
}

int linon_serve_submit(linon_server* s, const linon_request* req, uint64_t* id) {
  try {
    if (!s || !req || !id) return set_error(LINON_EINVAL, "null argument");
    if (int st = validate_request(s, *req)) return st;
    auto q = std::make_unique<Request>();
    q->req = *req;
    if (req->kind == LINON_REQ_CAPTURE) q->pos.assign(req->pos_xy, req->pos_xy + 2 * size_t(req->n_rays));
    q->req.pos_xy = nullptr;
    q->bytes = request_bytes(q->req, &q->n_points);
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) return set_error(LINON_ESTATE, "server stopped");
    if (s->sticky) return set_error(s->sticky, "server failed earlier: " + s->sticky_msg);
    if (s->cfg.hbm_budget && q->bytes > s->cfg.hbm_budget)
      return set_error(LINON_ENOMEM, "request needs " + std::to_string(q->bytes) + " bytes, above the budget of " +
                                         std::to_string(s->cfg.hbm_budget));
    q->id = s->next_id++;
    q->t_submit = now_ms(s);
    *id = q->id;
    s->pending.push_back(q.get());
    s->all[q->id] = std::move(q);
    s->submitted++;
    s->cv.notify_one();
    return LINON_OK;
  } catch (const std::exception& e) {
    return set_error(LINON_EINVAL, std::string("internal error: ") + e.what());
  }
}

int linon_serve_poll(linon_server* s, uint64_t id, linon_result* out) {
  if (!s || !out) return set_error(LINON_EINVAL, "null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return set_error(LINON_EINVAL, "unknown or released request id");
  copy_result(it->second.get(), out);
  return LINON_OK;
}

int linon_serve_wait(linon_server* s, uint64_t id, double timeout_ms, linon_result* out) {
  if (!s || !out) return set_error(LINON_EINVAL, "null argument");
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return set_error(LINON_EINVAL, "unknown or released request id");
  Request* q = it->second.get();
  const auto deadline = Clock::now() + std::chrono::microseconds(int64_t(std::max(0.0, timeout_ms) * 1000.0));
  while (!q->done) {
    if (s->done_cv.wait_until(lock, deadline) == std::cv_status::timeout && !q->done) {
      copy_result(q, out);
      return set_error(LINON_ETIMEOUT, "request " + std::to_string(id) + " still pending");
    }
  }
  copy_result(q, out);
  return LINON_OK;
}

int linon_serve_release(linon_server* s, uint64_t id) {
  if (!s) return set_error(LINON_EINVAL, "null server");
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return set_error(LINON_EINVAL, "unknown or released request id");
  Request* q = it->second.get();
  if (!q->done) return set_error(LINON_EBUSY, "request still pending");
  if (q->dev) {
    cudaSetDevice(s->ctx->device);
    cudaFreeAsync(q->dev, s->free_stream);
    s->used -= q->bytes;
  }
  s->all.erase(it);
  s->cv.notify_one();
  return LINON_OK;
}

int linon_serve_copy(linon_server* s, uint64_t id, int32_t plane, void* dst, size_t bytes) {
  if (!s || !dst) return set_error(LINON_EINVAL, "null argument");
  const void* src = nullptr;
  size_t have = 0;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return set_error(LINON_EINVAL, "unknown or released request id");
    const Request* q = it->second.get();
    if (!q->done || q->status != LINON_OK) return set_error(LINON_ESTATE, "request not finished successfully");
    const size_t n = size_t(q->req.width) * size_t(q->req.height);
    const linon_result& r = q->res;
    switch (plane) {
      case 0: src = r.frame.color; have = n * 4; break;
      case 1: src = r.frame.mapping; have = n * 16; break;
      case 2: src = r.frame.hit_id; have = n * 4; break;
      case 3: src = r.frame.steps; have = n * 4; break;
      case 4: src = r.overlay; have = n * 4; break;
      case 5: src = r.exponents; have = n * 4; break;
      case 6: src = r.paths; have = size_t(q->req.n_rays) * size_t(q->n_points) * 16; break;
      default: return set_error(LINON_EINVAL, "plane must be 0..6");
    }
  }
  if (!src) return set_error(LINON_EINVAL, "the request has no such plane");
  if (bytes < have) return set_error(LINON_EINVAL, "destination smaller than the plane (" + std::to_string(have) + " bytes)");
  cudaSetDevice(s->ctx->device);
  LINON_CUDA(cudaMemcpy(dst, src, have, cudaMemcpyDefault));
  return LINON_OK;
}

int linon_serve_stats(linon_server* s, linon_serve_counters* out) {
  if (!s || !out) return set_error(LINON_EINVAL, "null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->failed = s->failed;
  out->waves = s->waves;
  out->bytes_in_use = s->used;
  out->bytes_peak = s->peak;
  return LINON_OK;
}

int linon_serve_stop(linon_server* s) {
  if (!s) return LINON_OK;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
    s->cv.notify_all();
  }
  if (s->th.joinable()) s->th.join();
  cudaSetDevice(s->ctx->device);
  for (auto& kv : s->all)
    if (kv.second->dev) cudaFreeAsync(kv.second->dev, s->free_stream);
  cudaStreamSynchronize(s->free_stream);
  for (Slot& sl : s->slots) {
    cudaStreamSynchronize(sl.main);
    cudaStreamSynchronize(sl.aux);
    cudaFree(sl.views_dev);
    cudaFree(sl.counter);
    cudaFree(sl.sums_dev);
    cudaFreeHost(sl.sums_host);
    cudaEventDestroy(sl.ev_main);
    cudaEventDestroy(sl.ev_aux);
    cudaStreamDestroy(sl.main);
    cudaStreamDestroy(sl.aux);
  }
  cudaStreamDestroy(s->free_stream);
  const int sticky = s->sticky;
  const std::string msg = s->sticky_msg;
  delete s;
  return sticky ? set_error(sticky, "server had failed: " + msg) : LINON_OK;
}

}  // extern "C"
