/*
 * linon.h — C ABI of the GB300 nonlinear ray-casting engine.
 *
 * This is the drop-in boundary for linon's `MainView` compute dispatch
 * (src/main_view.rs).  A host (the reference's Rust `Application`, a Python
 * binding, a C++ service) owns the scene and frame buffers, hands plain
 * pointers and sizes across this ABI and gets status codes back.  No C++
 * exceptions cross it, no torch types appear in it.
 *
 * Conventions
 *  - Every function returns an int status (LINON_OK == 0) unless documented
 *    otherwise; the message of the last failing call on the calling thread is
 *    available from linon_last_error().
 *  - "device pointer" means memory on the context's CUDA device (cudaMalloc,
 *    torch CUDA tensors, ...).  Frame images use the reference's storage
 *    texture order: row 0 is the TOP row, i.e. the row written by the
 *    invocation with gid.y == H-1 (src/main_view.wgsl:342).
 *  - A context is single-threaded, like MainView on the winit thread
 *    (src/application.rs:492-528); use one context per host thread.  Work is
 *    enqueued on the context's stream (linon_set_stream); functions that hand
 *    results back in host memory synchronise that stream before returning.
 */
#ifndef LINON_H
#define LINON_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LINON_ABI_VERSION 2  /* 2: linon_batch_tuning.schedule */

/* ---- status codes ------------------------------------------------------ */
enum linon_status {
  LINON_OK = 0,
  LINON_EINVAL = 1,    /* bad argument (null pointer, size out of range)        */
  LINON_ECOMPILE = 2,  /* field source rejected by the WGSL front end or NVRTC;
                          the log holds the diagnostics (main_view.rs:657-679)  */
  LINON_ECUDA = 3,     /* CUDA runtime / driver error                           */
  LINON_ENOMEM = 4,    /* allocation failed or the HBM budget would be exceeded */
  LINON_ETIMEOUT = 5,  /* a bounded device- or host-side wait ran out           */
  LINON_ENOSCENE = 6,  /* render called before linon_scene_upload               */
  LINON_EBUSY = 7,     /* serving queue full / context busy                     */
  LINON_ESTATE = 8,    /* call not valid in the current state                   */
  LINON_EIO = 9        /* a file could not be read                              */
};

/* ---- data ABI (byte-compatible with the reference's uniforms) ---------- */

/* CameraUniform, src/main_view.rs:12-19 and src/main_view.wgsl:7-12 (112 B).
 * Only origin.xyz, view_direction.xyz and up.xyz are read (as in the shader). */
typedef struct linon_camera {
  float origin[4];
  float view_direction[4];
  float up[4];
  float view_matrix[16];
} linon_camera;

/* Settings, src/main_view.rs:43-51 and src/main_view.wgsl:16-23 (24 B). */
typedef struct linon_settings {
  float field_weight;              /* blend of the RK4 direction, 0..1      */
  float mouse_pos[2];              /* clicked position in [0,1]^2, y up     */
  int32_t overlay_mode;            /* 0 = passthrough, 1 = Lyapunov         */
  int32_t central_difference_delta;/* 1..10 pixels                          */
  float lyapunov_scaling;          /* 1..100                                */
} linon_settings;

/* RaySample, src/main_view.wgsl:55-58 and src/ray_samples.rs:8-27 (32 B). */
typedef struct linon_ray_sample {
  float position[4];
  float color[4];
} linon_ray_sample;

/* Ray-march control.  linon_march_params_reference() fills the values the
 * reference shader hard-codes (main_view.wgsl:227,241-255,267-269,355-356). */
typedef struct linon_march_params {
  float h_initial;        /* RK4 step (0.1; Enhance uses 0.001)               */
  float t_max;            /* loop while t <= t_max when max_steps == 0 (5.0)  */
  int32_t max_steps;      /* > 0: run exactly this many accepted steps         */
  int32_t adaptive;       /* adaptive refinement of main_view.wgsl:251-255     */
  float h_fine;           /* refined step (0.001)                              */
  float h_fine_above;     /* refine only while h > this (0.002)                */
  int32_t stop_on_hit;    /* end the ray at its first hit (no endpoint march)  */
  int32_t kahan;          /* compensated (Kahan) sums for position and t       */
  float focal_length;     /* main_view.wgsl:355 (0.035)                        */
  float viewport_height;  /* main_view.wgsl:356 (0.025)                        */
  int32_t linear_mode;    /* main_view.wgsl:72,368-370: straight ray, max 100  */
  int32_t reserved;
} linon_march_params;

/* Output planes of one rendered frame (all device pointers, any may be NULL). */
typedef struct linon_frame {
  int32_t width;
  int32_t height;
  uint8_t* color;    /* W*H*4 rgba8 — the `ttarget` of main_view.wgsl:2     */
  float* mapping;    /* W*H*4 rgba32f endpoint (x,y,z,1) — main_view.wgsl:5 */
  int32_t* hit_id;   /* W*H face index of the first hit, -1 for a miss     */
  int32_t* steps;    /* W*H accepted RK4 steps                              */
} linon_frame;

/* One view of a batched launch. */
typedef struct linon_view {
  linon_camera camera;
  linon_settings settings;
  linon_march_params params;
  int32_t width;
  int32_t height;
  int32_t field_index;  /* index into the `fields` array of the batch call */
  int32_t reserved;
  linon_frame out;      /* device output planes (width/height ignored)     */
} linon_view;

/* Predefined field functions, src/functions.rs:1-13, plus the stub body of
 * main_view.wgsl:148 and the four field functions of the benchmark configs. */
enum linon_predefined {
  LINON_FIELD_CUSTOM = 0,                   /* empty body (a compile error)  */
  LINON_FIELD_MIRAGE_SPHERICAL = 1,
  LINON_FIELD_MIRAGE_PLANE = 2,
  LINON_FIELD_MIRAGE_SPHERICAL_SIGMOID = 3, /* the reference's default       */
  LINON_FIELD_MIRAGE_PLANE_SIGMOID = 4,
  LINON_FIELD_TRANSLATION_X = 5,
  LINON_FIELD_TRANSLATION_Z = 6,
  LINON_FIELD_ROTATION = 7,
  LINON_FIELD_LORENZ = 8,
  LINON_FIELD_ROESSLER = 9,
  LINON_FIELD_IDENTITY = 10,                /* `return v;` (wgsl:148 stub)  */
  LINON_FIELD_LINEAR = 11,                  /* `return v0;`                   */
  LINON_FIELD_TWIST = 12,                   /* rotateY(v0, 0.5 * p.y)         */
  LINON_FIELD_LENS = 13,                    /* point-lens bending             */
  LINON_FIELD_LORENZ_SCALED = 14,           /* 0.05 * Lorenz + v0             */
  LINON_FIELD_COUNT = 15
};

/* linon_field_compile flags */
enum linon_compile_flags {
  LINON_COMPILE_PRECISE = 1,  /* no FMA contraction, IEEE div/sqrt everywhere:
                                 op-for-op the FP32 restatement of the shader */
  LINON_VALIDATE_BATCHED = 2  /* linon_field_validate only: also compile the
                                 batched kernels (linon_render_batch) with it */
};

typedef struct linon_ctx linon_ctx;
typedef struct linon_field linon_field;

/* ---- library ------------------------------------------------------------ */
int linon_abi_version(void);
/* The reference reports shader errors as Err(wgpu::Error) from
 * reload_shader (main_view.rs:657-679) and panics on runtime errors
 * (main_view.rs:675); here every failure is a status code, with its message
 * kept per thread.                                                          */
const char* linon_last_error(void);
const char* linon_status_string(int status);
/* Source text of a predefined field body (functions.rs:33-128) or NULL. */
const char* linon_predefined_source(int id);
/* Display name of a predefined field (functions.rs:15-30) or NULL. */
const char* linon_predefined_name(int id);
/* Reference constants for the march (main_view.wgsl:227,241,252,355-356). */
void linon_march_params_reference(linon_march_params* out);

/* ---- context: replaces MainView::new (main_view.rs:82-458) -------------- */
/* hbm_budget_bytes == 0 means "no budget".                                  */
int linon_create(int device, size_t hbm_budget_bytes, linon_ctx** out);
int linon_destroy(linon_ctx* ctx);
/* cudaStream_t to enqueue on (NULL = the context's own stream).             */
int linon_set_stream(linon_ctx* ctx, void* cuda_stream);
int linon_synchronize(linon_ctx* ctx);
/* Bytes of device memory the context holds (scene, BVH, caches, slabs).    */
size_t linon_device_bytes(const linon_ctx* ctx);

/* ---- scene: replaces MainView::update_model (main_view.rs:460-488) ------
 * xyz: n_vertices*3 floats (12 B stride, wgsl:33-42); abc: n_faces*3 u32
 * (12 B stride, wgsl:44-53); face_rgb: optional n_faces*3 floats replacing
 * |normal| as the shading colour.  Host pointers; the data is copied.
 * build_bvh != 0 builds a BVH whose hits equal the brute-force loop's
 * (main_view.wgsl:182-198); 0 keeps the brute-force scan.                  */
int linon_scene_upload(linon_ctx* ctx, const float* xyz, uint32_t n_vertices,
                       const uint32_t* abc, uint32_t n_faces,
                       const float* face_rgb, int build_bvh);
/* BVH statistics of the current scene: nodes, leaves, max depth.          */
int linon_scene_info(const linon_ctx* ctx, uint32_t* n_faces, uint32_t* n_nodes,
                     uint32_t* max_depth);

/* ---- OBJ ingestion: replaces the dropped-file path, src/main.rs:139-156
 * (tobj 4.0.2 `load_obj` with triangulate = true, models[0].mesh) and
 * Application::load_model (src/application.rs:199-226).
 * Positions come in the order of their first reference by a face of the
 * model (tobj's default multi-index export); faces are triangles (quads and
 * polygons as fans around their first vertex, points and lines as
 * zero-area triangles).  `model` selects tobj's models[model]: files are
 * split into models at "o" / "g" records and at "usemtl" switches between
 * materials named in the "mtllib" files.  LINON_OBJ_NORMALIZE applies
 * normalize_vertices (src/vertices.rs:3-17) as load_model does; the
 * reported centre is get_center (src/vertices.rs:19-57) of the returned
 * positions.  Errors: LINON_EIO (file unreadable), LINON_EINVAL with
 * "obj line N: ..." (malformed record, index out of range, no such model);
 * *out is NULL then.  The mesh is host memory owned by the caller.        */
typedef struct linon_mesh linon_mesh;
#define LINON_OBJ_NORMALIZE 1u
int linon_obj_load(const char* path, uint32_t model, uint32_t flags, linon_mesh** out);
/* The same from text in memory; "mtllib" files are looked up in mtl_dir
 * (NULL: no material file is read and every material name is unknown).    */
int linon_obj_parse(const char* text, size_t len, const char* mtl_dir, uint32_t model,
                    uint32_t flags, linon_mesh** out);
/* Vertex / triangle counts, the number of models in the file and the
 * bounding-box centre of the returned positions (any pointer may be NULL). */
int linon_mesh_info(const linon_mesh* mesh, uint32_t* n_vertices, uint32_t* n_faces,
                    uint32_t* n_models, float center[3]);
const float* linon_mesh_positions(const linon_mesh* mesh); /* n_vertices*3 */
const uint32_t* linon_mesh_faces(const linon_mesh* mesh);  /* n_faces*3    */
void linon_mesh_free(linon_mesh* mesh);
/* normalize_vertices (src/vertices.rs:3-17) in place over n_floats
 * coordinates: one min and max over all of them, x' = (x-min)/(max-min)*2-1
 * in f32; then get_center (src/vertices.rs:19-57) into center (may be NULL;
 * needs n_floats >= 3).  Equal min and max give non-finite results, as in
 * the reference.                                                          */
int linon_normalize_vertices(float* xyz, size_t n_floats, float center[3]);

/* ---- field functions: replaces MainView::reload_shader
 *      (main_view.rs:649-690) and with_field_function (main_view.rs:852-861)
 * field_body: WGSL statements of `fn field_function(p_prev, p, v0, v, t)`.
 * helpers_src: optional WGSL `fn` declarations callable from the body (the
 * "additional helper functions" of README.md:46).  On failure the status is
 * LINON_ECOMPILE and `log` holds the diagnostics (NUL-terminated, truncated
 * to log_cap).                                                              */
int linon_field_compile(linon_ctx* ctx, const char* field_body,
                        const char* helpers_src, int flags, linon_field** out,
                        char* log, size_t log_cap);
int linon_field_release(linon_ctx* ctx, linon_field* field);
/* No counterpart in the reference (naga exposes no such count).  Counted
 * FP32 operations of one field evaluation (from the front end IR):
 * arithmetic ops and transcendental calls.                                 */
int linon_field_flops(const linon_field* field, int32_t* arith, int32_t* transcendental);
/* The CUDA C the front end generated for the field (for diagnostics).      */
const char* linon_field_cuda_source(const linon_field* field);
/* Whether fixed-step renders of this field can run two rays per thread (no
 * counterpart in the reference, whose shader marches one ray per
 * invocation): 1 the pair kernels compiled (a render uses them when the
 * field has at least 4 FP32 operations and at most one transcendental per
 * evaluation and the frame fills at least 8 waves of the pair kernel's
 * resident CTAs; the environment variable LINON_RAY_PAIRS=0 / =1 forces
 * one / two rays per thread), 0 the field has a pair form not tried yet,
 * -1 it has none (a branch on a value, var<private> state, a precise
 * module) or it did not compile.                                           */
int linon_field_pair_state(const linon_field* field);
/* Front end + NVRTC compile for sm_103a without loading (no GPU needed): the
 * naga validation step of create_shader_module (main_view.rs:662-665).  On
 * success `log` holds the compiler/ptxas report (registers, spills).       */
int linon_field_validate(const char* field_body, const char* helpers_src, int flags,
                         char* log, size_t log_cap);
/* Lower WGSL to CUDA C without a context or GPU (front end only): the
 * WGSL-to-IR half of create_shader_module, with CUDA C as the output.      */
int linon_wgsl_translate(const char* field_body, const char* helpers_src,
                         char* out, size_t out_cap, char* log, size_t log_cap);

/* ---- ray casting: the first dispatch of MainView::render
 *      (main_view.rs:831-843, main_view.wgsl:339-376)                      */
int linon_render(linon_ctx* ctx, const linon_field* field,
                 const linon_camera* camera, const linon_settings* settings,
                 const linon_march_params* params, const linon_frame* out);
/* No counterpart in the reference (it renders whole frames).
 * Rows [row0, row1) of the same width x height frame (the primary rays of
 * those rows, stored at their rows of `out`; other rows untouched): one
 * shard of a frame split by rows across GPUs (no exchange; an overlay over
 * a shard renders 2 * central_difference_delta halo rows on each inner
 * side).                                                                    */
int linon_render_rows(linon_ctx* ctx, const linon_field* field,
                      const linon_camera* camera, const linon_settings* settings,
                      const linon_march_params* params, const linon_frame* out,
                      int32_t row0, int32_t row1);
/* Evaluates the field at n points: in = n x 13 floats (p_prev.xyz, p.xyz,
 * v0.xyz, v.xyz, t), out = n x 3 floats; both device pointers.  This is the
 * field_function of main_view.wgsl:148 called on its own (field probes,
 * glyph visualisation).                                                    */
int linon_field_eval(linon_ctx* ctx, const linon_field* field, const float* in,
                     float* out, int64_t n);
/* linon_render with host output buffers (copied back; NULL planes are
 * skipped).  The reference keeps its frames in textures and never reads
 * them back; this is the call a host without device memory of its own
 * makes.                                                                    */
int linon_render_host(linon_ctx* ctx, const linon_field* field,
                      const linon_camera* camera, const linon_settings* settings,
                      const linon_march_params* params, int32_t width,
                      int32_t height, uint8_t* color, float* mapping,
                      int32_t* hit_id, int32_t* steps);

/* ---- overlay: the second dispatch (main_view.rs:844-846,
 *      overlay.wgsl:99-165).  exponents is indexed y*W+x (the reference
 *      indexes y*H+x, identical for square images).  srgb != 0 selects
 *      overlay_web (sRGB encode).  fp64 != 0 does the neighbour differences
 *      and eigenvalues in FP64; 0 keeps the shader's FP32 arithmetic.      */
int linon_overlay(linon_ctx* ctx, const linon_settings* settings,
                  int32_t width, int32_t height, const uint8_t* ray_casting,
                  const float* mapping, uint8_t* target, float* exponents,
                  int srgb, int fp64);
/* No counterpart in the reference (its overlay is the eigenvalue form
 * above).  Finite-time exponent: ln(max over the 4-neighbourhood of
 * |endpoint difference| / initial direction separation) / T, in FP64.      */
int linon_ftle(linon_ctx* ctx, const linon_camera* camera,
               const linon_march_params* params, int32_t width, int32_t height,
               const float* mapping, float horizon_T, float* exponents);

/* ---- path capture: sample_rays (main_view.wgsl:281-314,470-479) --------
 * Reference form: the 8 rays around settings->mouse_pos (or, when
 * positions != NULL, at the 8 given normalised positions), 5000 steps of
 * h = 0.001, every 50th position -> 800 RaySamples (device pointer).      */
int linon_capture_reference(linon_ctx* ctx, const linon_field* field,
                            const linon_camera* camera,
                            const linon_settings* settings,
                            const linon_march_params* params, int32_t width,
                            int32_t height, const float* positions,
                            linon_ray_sample* out);
/* General form: n_rays rays at normalised positions pos_xy (host, n*2),
 * n_steps RK4 steps of size h, recording the position before every
 * record_every-th step and the final position: out is device memory of
 * n_rays * n_points float4, n_points = ceil(n_steps/record_every) + 1.     */
int linon_capture_paths(linon_ctx* ctx, const linon_field* field,
                        const linon_camera* camera,
                        const linon_settings* settings,
                        const linon_march_params* params, int32_t width,
                        int32_t height, const float* pos_xy, int32_t n_rays,
                        float h, int32_t n_steps, int32_t record_every,
                        float* out);

/* Path capture that allocates nothing.  No counterpart in the reference.
 * For callers that cannot allocate device memory: a click handler on an
 * interactive UI thread with a frame budget (an allocation or free can
 * synchronise the whole device), or a host that gave the context a fixed
 * memory budget.  Same arguments, checks and output as linon_capture_paths;
 * the start positions are staged in a fixed device array inside the library
 * (LINON_NOALLOC_MAX_RAYS rays, 128 KB, held on every GPU that loads the
 * library until the process exits) instead of the context's scratch buffer,
 * and no cudaMalloc/cudaFree or other allocating routine is called.
 * n_rays > LINON_NOALLOC_MAX_RAYS fails with LINON_EINVAL.  pos_xy is
 * ordinary (pageable) host memory, read before the call returns.  The first
 * call on a device looks up the array's device address (set-up done once per
 * device); make that first call before any stream capture, and do not use
 * the library across a cudaDeviceReset.  Every call shares the one array:
 * calls whose work overlaps on the GPU (other streams or contexts) race on
 * it and must be serialised by the caller.                                  */
#define LINON_NOALLOC_MAX_RAYS 16384
int linon_capture_paths_noalloc(linon_ctx* ctx, const linon_field* field,
                                const linon_camera* camera,
                                const linon_settings* settings,
                                const linon_march_params* params,
                                int32_t width, int32_t height,
                                const float* pos_xy, int32_t n_rays, float h,
                                int32_t n_steps, int32_t record_every,
                                float* out);

/* ---- outline rays (main_view.wgsl:381-468, main_view.rs:804-829) --------
 * Finds the 8 extremal pixels whose exponent >= min_exp exactly as the
 * shader's sequential scans do; exponents is a device pointer indexed
 * y*W+x.  pix_out (host, 8*2 int) gets the pixels, pos_out (host, 8*2
 * float) the normalised positions fed to linon_capture_reference.        */
int linon_outline_select(linon_ctx* ctx, const float* exponents, int32_t width,
                         int32_t height, float min_exp, int32_t* pix_out,
                         float* pos_out);
/* Exponent value at the given quantile (0..1) over the interior pixels
 * (no counterpart in the reference, whose outline uses the fixed threshold
 * 0.8; the p95 threshold selects the outline pixels of a Lyapunov frame).  */
int linon_exponent_quantile(linon_ctx* ctx, const float* exponents,
                            int32_t width, int32_t height, int32_t border,
                            double q, float* out);
/* Outline-mesh index list of src/ray_samples.rs:29-49 (396 u16 triangles).
 * Returns the number of u16 written, or a negative status.                */
int linon_outline_indices(uint16_t* out, size_t cap);

/* ---- batched rendering: many views in one launch -----------------------
 * No counterpart in the reference, which renders one view per
 * MainView::render (main_view.rs:831-849).  Views of any size, camera, step size and field go into one launch.  The
 * views' pixels are cut into tiles, views with the largest step budget
 * first.  Schedules: one CTA per 8x16-pixel tile of every view, the
 * hardware balancing the CTAs (2, the default); a persistent kernel whose
 * CTAs take 8x16-pixel tiles from a device work queue (3); a persistent
 * kernel whose warps take 32-ray tiles from a device work queue and march
 * each to the end (1, refill_below = 0) or retire finished rays and refill
 * free lanes every `quantum` steps once fewer than refill_below lanes march
 * (1, refill_below > 0).  fields[] may hold up to LINON_MAX_BATCH_FIELDS
 * distinct fields; views[i].field_index selects.                           */
#define LINON_MAX_BATCH_FIELDS 8
typedef struct linon_batch_tuning {
  int32_t quantum;          /* lane refills: RK4 steps between retire/refill
                               (0 = auto)                                   */
  int32_t block_threads;    /* threads per CTA (0 = auto)                  */
  int32_t ctas_per_sm;      /* resident CTAs per SM (0 = auto)             */
  int32_t tile_w, tile_h;   /* pixel tile handed out per queue pop (0=auto) */
  int32_t refill_below;     /* 0: warps take whole tiles; > 0: refill free
                               lanes once fewer than this many march        */
  int32_t schedule;         /* 0 auto (= 2), 1 persistent queue of warp
                               tiles (the fields above), 2 one CTA per
                               8x16-pixel tile of every view (hardware
                               scheduling), 3 persistent queue of 8x16-pixel
                               CTA tiles (128-thread CTAs)                  */
} linon_batch_tuning;
int linon_render_batch(linon_ctx* ctx, const linon_field* const* fields,
                       int32_t n_fields, const linon_view* views,
                       int32_t n_views, const linon_batch_tuning* tuning);
/* Plain reference: one linon_render launch per view, back to back.        */
int linon_render_views_plain(linon_ctx* ctx, const linon_field* const* fields,
                             int32_t n_fields, const linon_view* views,
                             int32_t n_views);
/* Sweep tuning candidates on the given batch and keep the fastest.        */
int linon_autotune_batch(linon_ctx* ctx, const linon_field* const* fields,
                         int32_t n_fields, const linon_view* views,
                         int32_t n_views, linon_batch_tuning* best,
                         double* best_ms);

/* ---- serving: continuous batching of requests ---------------------------
 * No counterpart in the reference, which redraws one view per UI event
 * (application.rs:492-528).  A server owns a scheduler thread and the context (do not use the context
 * from other threads while it runs).  Requests of any kind and size are
 * queued at submit, admitted in arrival order as their output memory fits the
 * HBM budget, and launched in waves: all frames / Enhance re-renders /
 * overlay renders admitted together go into one persistent batched launch,
 * overlays and captures follow on the wave's streams.  `slots` waves can be
 * on the GPU at once, so requests arriving while others run start without
 * waiting for them.  Results stay in device memory until released.        */
enum linon_request_kind {
  LINON_REQ_FRAME = 0,    /* ray-cast frame (Enhance: smaller h_initial)    */
  LINON_REQ_OVERLAY = 1,  /* frame + Lyapunov overlay (exponents)           */
  LINON_REQ_CAPTURE = 2   /* ray-sample capture: n_rays full polylines      */
};
typedef struct linon_request {
  int32_t kind;
  int32_t field_index;          /* into the server's field table            */
  linon_camera camera;
  linon_settings settings;
  linon_march_params params;
  int32_t width, height;
  int32_t fp64_overlay;         /* overlay: FP64 differencing               */
  int32_t n_rays;               /* capture: rays at pos_xy (host, n_rays*2, */
  int32_t n_steps;              /*   copied at submit), n_steps of size h,  */
  int32_t record_every;         /*   one point every record_every steps     */
  float h;
  int32_t reserved;
  const float* pos_xy;
} linon_request;
typedef struct linon_serve_config {
  size_t hbm_budget;            /* bytes of request outputs (0 = unlimited) */
  int32_t slots;                /* waves in flight (default 2)              */
  int32_t max_wave;             /* requests per wave (default 256)          */
  linon_batch_tuning tuning;    /* of the batched launch (zeros = auto)     */
} linon_serve_config;
typedef struct linon_result {
  int32_t status;               /* LINON_OK done, LINON_EBUSY queued or
                                   running, else the request's error        */
  int32_t kind;
  double t_submit_ms, t_admit_ms, t_done_ms;  /* server clock              */
  int64_t ray_steps;            /* accepted RK4 steps of the request        */
  linon_frame frame;            /* device planes (frames, overlays)         */
  uint8_t* overlay;             /* overlay target rgba8 (device)            */
  float* exponents;             /* overlay exponents (device)               */
  float* paths;                 /* capture: n_rays * n_points float4        */
  int32_t n_points;
  int32_t wave;                 /* wave the request ran in                  */
} linon_result;
typedef struct linon_serve_counters {
  uint64_t submitted, completed, failed, waves;
  size_t bytes_in_use, bytes_peak;
} linon_serve_counters;
typedef struct linon_server linon_server;
int linon_serve_start(linon_ctx* ctx, const linon_field* const* fields, int32_t n_fields,
                      const linon_serve_config* cfg, linon_server** out);
int linon_serve_submit(linon_server* server, const linon_request* req, uint64_t* id);
/* Non-blocking; out->status is LINON_EBUSY while the request is pending.  */
int linon_serve_poll(linon_server* server, uint64_t id, linon_result* out);
/* Waits at most timeout_ms; LINON_ETIMEOUT if the request is still pending. */
int linon_serve_wait(linon_server* server, uint64_t id, double timeout_ms, linon_result* out);
/* Copies one output plane of a finished request into dst (host or device
 * memory, cudaMemcpyDefault), synchronously.  plane: 0 color, 1 mapping,
 * 2 hit_id, 3 steps, 4 overlay target, 5 exponents, 6 capture paths.       */
int linon_serve_copy(linon_server* server, uint64_t id, int32_t plane, void* dst, size_t bytes);
/* Frees the request's device outputs (after it finished).                 */
int linon_serve_release(linon_server* server, uint64_t id);
int linon_serve_stats(linon_server* server, linon_serve_counters* out);
/* Finishes the waves on the GPU, fails still-queued requests, joins.      */
int linon_serve_stop(linon_server* server);

/* ---- measurement (no counterpart in the reference) ----------------------
 * Measured FP32 throughput of the device (independent FFMA chains on every
 * SM, best of 5 launches timed with CUDA events), in TFLOP/s.             */
int linon_probe_fp32_peak(linon_ctx* ctx, double* tflops);

/* ---- failure path (no counterpart in the reference) ---------------------
 * Runs one CTA that waits, with the march kernels' bounded mbarrier wait, on
 * a barrier that nothing completes (no copy is issued), for at most `polls`
 * polls (1..2^24): the wait runs out, the kernel sets error bit 1 and
 * returns, and the call returns what linon_synchronize reports for it:
 * LINON_ETIMEOUT (error word cleared; the context stays usable).            */
int linon_check_bounded_wait(linon_ctx* ctx, int32_t polls);

#ifdef __cplusplus
}
#endif
#endif /* LINON_H */
