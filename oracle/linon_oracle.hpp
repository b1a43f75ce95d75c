// linon_oracle.hpp — CPU restatement of linon's ray-casting path.
//
// TEST INFRASTRUCTURE ONLY.  This header is the oracle the CUDA engine in
// linon_gb300/ is compared against: only tests/, __graft_entry__.smoke() and
// bench.py's CPU baseline leg may use it, and never as the thing measured or
// shipped.
//
// It restates, operation for operation and in the shader's evaluation order,
//   src/main_view.wgsl:78-146  helpers (rotateX/Y/Z, translate, refraction_index,
//                              refraction, point_plane_distance, sigmoid)
//   src/main_view.wgsl:150-175 hit_triangle (Moeller-Trumbore, eps 1e-7, no culling)
//   src/main_view.wgsl:177-220 ray_color (closest hit over all faces, shading)
//   src/main_view.wgsl:229-279 nonlinear_ray_color (RK4 march, adaptive step)
//   src/main_view.wgsl:281-314 sample_rays (path capture)
//   src/main_view.wgsl:339-376 main_view (primary ray generation, stores)
//   src/overlay.wgsl:4-40,99-135 Lyapunov overlay
//   src/functions.rs:33-128    the predefined field functions
// templated on the scalar: `float` is the FP32-faithful form (compile with
// -ffp-contract=off and without -ffast-math), `double` the FP64 accuracy
// oracle, `CountingFloat` counts FP32 operations per ray step.
//
// Parity status: pinned against the reference's shader source, not its
// runtime.  The reference is WGSL executed through wgpu/naga on a graphics
// API; neither a graphics stack nor a Rust toolchain exists where this project
// is built or measured, and the reference ships no tests, golden vectors or
// fixtures for this path.  Its shader text itself, lowered on the host with
// the bindings made private (tests/golden/make_shader_pins.py), gives the
// fixtures this file is held to bit for bit (tests/golden/shader_pins.npz,
// checked by tests/test_shader_pins.py).
//
// Where WGSL leaves the result implementation-defined, this file fixes one
// choice and the CUDA engine follows it:
//   * dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z ; M*v sums columns in order.
//   * normalize(v) = v / sqrt(dot(v,v)) ; length(v) = sqrt(dot(v,v)).
//   * clamp(e,lo,hi) = min(max(e,lo),hi) (the first of the two forms the
//     WGSL spec allows), so the shader's clamp(-1.0, 1.0, x) is min(1, x).
//   * min/max follow IEEE fmin/fmax (a NaN operand yields the other one).
//   * pow(10.0, -10.0) is the correctly rounded constant 1e-10.
//   * rgba8unorm stores round half to even after clamping to [0,1].
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace linon_oracle {

// ---------------------------------------------------------------------------
// Scalar operations.  Overloaded per scalar type so that CountingFloat can
// count them; float and double map to the C library.
// ---------------------------------------------------------------------------
struct OpCounts {
  long long add = 0, mul = 0, div = 0, sqrt = 0, cmp = 0, transc = 0;
  long long arith() const { return add + mul + div + sqrt; }
};
inline OpCounts& counts() {
  static thread_local OpCounts c;
  return c;
}

// A float that counts the operations done on it (single-threaded use).
struct CountingFloat {
  float v;
  CountingFloat() : v(0.f) {}
  CountingFloat(double x) : v(float(x)) {}
  explicit operator float() const { return v; }
};
inline CountingFloat operator+(CountingFloat a, CountingFloat b) { counts().add++; return CountingFloat(a.v + b.v); }
inline CountingFloat operator-(CountingFloat a, CountingFloat b) { counts().add++; return CountingFloat(a.v - b.v); }
inline CountingFloat operator*(CountingFloat a, CountingFloat b) { counts().mul++; return CountingFloat(a.v * b.v); }
inline CountingFloat operator/(CountingFloat a, CountingFloat b) { counts().div++; return CountingFloat(a.v / b.v); }
inline CountingFloat operator-(CountingFloat a) { return CountingFloat(-a.v); }
inline bool operator<(CountingFloat a, CountingFloat b) { counts().cmp++; return a.v < b.v; }
inline bool operator>(CountingFloat a, CountingFloat b) { counts().cmp++; return a.v > b.v; }
inline bool operator<=(CountingFloat a, CountingFloat b) { counts().cmp++; return a.v <= b.v; }
inline bool operator>=(CountingFloat a, CountingFloat b) { counts().cmp++; return a.v >= b.v; }
inline bool operator==(CountingFloat a, CountingFloat b) { counts().cmp++; return a.v == b.v; }
inline CountingFloat& operator+=(CountingFloat& a, CountingFloat b) { a = a + b; return a; }

inline float s_sqrt(float x) { return std::sqrt(x); }
inline double s_sqrt(double x) { return std::sqrt(x); }
inline float s_sin(float x) { return std::sin(x); }
inline double s_sin(double x) { return std::sin(x); }
inline float s_cos(float x) { return std::cos(x); }
inline double s_cos(double x) { return std::cos(x); }
inline float s_exp(float x) { return std::exp(x); }
inline double s_exp(double x) { return std::exp(x); }
inline float s_pow(float x, float y) { return std::pow(x, y); }
inline double s_pow(double x, double y) { return std::pow(x, y); }
inline float s_abs(float x) { return std::fabs(x); }
inline double s_abs(double x) { return std::fabs(x); }
inline float s_min(float a, float b) { return std::fmin(a, b); }
inline double s_min(double a, double b) { return std::fmin(a, b); }
inline float s_max(float a, float b) { return std::fmax(a, b); }
inline double s_max(double a, double b) { return std::fmax(a, b); }

inline CountingFloat s_sqrt(CountingFloat x) { counts().sqrt++; return CountingFloat(std::sqrt(x.v)); }
inline CountingFloat s_sin(CountingFloat x) { counts().transc++; return CountingFloat(std::sin(x.v)); }
inline CountingFloat s_cos(CountingFloat x) { counts().transc++; return CountingFloat(std::cos(x.v)); }
inline CountingFloat s_exp(CountingFloat x) { counts().transc++; return CountingFloat(std::exp(x.v)); }
inline CountingFloat s_pow(CountingFloat x, CountingFloat y) { counts().transc++; return CountingFloat(std::pow(x.v, y.v)); }
inline CountingFloat s_abs(CountingFloat x) { return CountingFloat(std::fabs(x.v)); }
inline CountingFloat s_min(CountingFloat a, CountingFloat b) { counts().cmp++; return CountingFloat(std::fmin(a.v, b.v)); }
inline CountingFloat s_max(CountingFloat a, CountingFloat b) { counts().cmp++; return CountingFloat(std::fmax(a.v, b.v)); }

// ---------------------------------------------------------------------------
// TraceFloat: a float that records every operation on a tape, so that the
// operations a ray's endpoint actually depends on can be counted (the
// roofline's algorithmic work).  Rules:
//   * liveness: the roots are the values the caller marks (the endpoint)
//     and the operands of comparisons on loop-variant values (control
//     flow); an operation is counted only if a root depends on it;
//   * loop invariance: literals and march parameters are invariant, values
//     marked by mark_carried (the state a step hands to the next) are not,
//     and an operation on invariant operands only is invariant -- computed
//     once per launch, not per step, so it is not counted;
//   * launch constants: a product with an invariant 1 or 0, a sum with an
//     invariant 0 and a quotient by an invariant 1 are not operations (the
//     kernel variants specialise field_weight == 1; the rotation matrices'
//     structural zeros and ones).
// Negation and abs are free; min/max are comparisons, not FP32 arithmetic.
// ---------------------------------------------------------------------------
enum TraceKind : uint8_t { TK_LEAF, TK_ADD, TK_MUL, TK_DIV, TK_SQRT, TK_TRANSC, TK_FREE, TK_CMP };
struct Tape {
  std::vector<uint8_t> kind, inv;
  std::vector<int32_t> a, b;
  std::vector<int32_t> roots;
  int32_t push(uint8_t k, int32_t x, int32_t y, bool invariant) {
    kind.push_back(k);
    inv.push_back(invariant ? 1 : 0);
    a.push_back(x);
    b.push_back(y);
    return int32_t(kind.size() - 1);
  }
  void clear() { kind.clear(); inv.clear(); a.clear(); b.clear(); roots.clear(); }
  // live, loop-variant operations by kind
  void count(long long out[8]) const {
    std::vector<uint8_t> live(kind.size(), 0);
    for (int32_t r : roots) live[r] = 1;
    for (int64_t i = int64_t(kind.size()) - 1; i >= 0; --i) {
      if (!live[i]) continue;
      if (a[i] >= 0) live[a[i]] = 1;
      if (b[i] >= 0) live[b[i]] = 1;
    }
    for (int k = 0; k < 8; ++k) out[k] = 0;
    for (size_t i = 0; i < kind.size(); ++i)
      if (live[i] && !inv[i]) out[kind[i]]++;
  }
};
inline Tape& tape() {
  static thread_local Tape t;
  return t;
}

struct TraceFloat {
  float v;
  int32_t id;
  TraceFloat() : v(0.f), id(tape().push(TK_LEAF, -1, -1, true)) {}
  TraceFloat(double x) : v(float(x)), id(tape().push(TK_LEAF, -1, -1, true)) {}
  TraceFloat(float val, int32_t node, int) : v(val), id(node) {}
  explicit operator float() const { return v; }
};
inline bool tr_inv(TraceFloat x) { return tape().inv[x.id] != 0; }
inline bool tr_is(TraceFloat x, float c) { return tr_inv(x) && x.v == c; }
inline TraceFloat tr_op(TraceKind k, TraceFloat x, TraceFloat y, float v) {
  return TraceFloat(v, tape().push(k, x.id, y.id, tr_inv(x) && tr_inv(y)), 0);
}
inline TraceFloat tr_op1(TraceKind k, TraceFloat x, float v) {
  return TraceFloat(v, tape().push(k, x.id, -1, tr_inv(x)), 0);
}
inline TraceFloat tr_const(float v) { return TraceFloat(v, tape().push(TK_LEAF, -1, -1, true), 0); }
inline TraceFloat operator+(TraceFloat a, TraceFloat b) {
  const float v = a.v + b.v;
  if (tr_is(a, 0.0f)) return TraceFloat(v, b.id, 0);
  if (tr_is(b, 0.0f)) return TraceFloat(v, a.id, 0);
  return tr_op(TK_ADD, a, b, v);
}
inline TraceFloat operator-(TraceFloat a, TraceFloat b) {
  const float v = a.v - b.v;
  if (tr_is(b, 0.0f)) return TraceFloat(v, a.id, 0);
  if (tr_is(a, 0.0f)) return tr_op1(TK_FREE, b, v);
  return tr_op(TK_ADD, a, b, v);
}
inline TraceFloat operator*(TraceFloat a, TraceFloat b) {
  const float v = a.v * b.v;
  if (tr_is(a, 0.0f) || tr_is(b, 0.0f)) return tr_const(v);
  if (tr_is(a, 1.0f)) return TraceFloat(v, b.id, 0);
  if (tr_is(b, 1.0f)) return TraceFloat(v, a.id, 0);
  return tr_op(TK_MUL, a, b, v);
}
inline TraceFloat operator/(TraceFloat a, TraceFloat b) {
  const float v = a.v / b.v;
  if (tr_is(b, 1.0f)) return TraceFloat(v, a.id, 0);
  return tr_op(TK_DIV, a, b, v);
}
inline TraceFloat operator-(TraceFloat a) { return tr_op1(TK_FREE, a, -a.v); }
inline void tr_control(TraceFloat a, TraceFloat b) {
  if (!tr_inv(a)) tape().roots.push_back(a.id);
  if (!tr_inv(b)) tape().roots.push_back(b.id);
}
inline bool operator<(TraceFloat a, TraceFloat b) { tr_control(a, b); return a.v < b.v; }
inline bool operator>(TraceFloat a, TraceFloat b) { tr_control(a, b); return a.v > b.v; }
inline bool operator<=(TraceFloat a, TraceFloat b) { tr_control(a, b); return a.v <= b.v; }
inline bool operator>=(TraceFloat a, TraceFloat b) { tr_control(a, b); return a.v >= b.v; }
inline bool operator==(TraceFloat a, TraceFloat b) { tr_control(a, b); return a.v == b.v; }
inline TraceFloat& operator+=(TraceFloat& a, TraceFloat b) { a = a + b; return a; }
inline TraceFloat s_sqrt(TraceFloat x) { return tr_op1(TK_SQRT, x, std::sqrt(x.v)); }
inline TraceFloat s_sin(TraceFloat x) { return tr_op1(TK_TRANSC, x, std::sin(x.v)); }
inline TraceFloat s_cos(TraceFloat x) { return tr_op1(TK_TRANSC, x, std::cos(x.v)); }
inline TraceFloat s_exp(TraceFloat x) { return tr_op1(TK_TRANSC, x, std::exp(x.v)); }
inline TraceFloat s_pow(TraceFloat x, TraceFloat y) { return tr_op(TK_TRANSC, x, y, std::pow(x.v, y.v)); }
inline TraceFloat s_abs(TraceFloat x) { return tr_op1(TK_FREE, x, std::fabs(x.v)); }
inline TraceFloat s_min(TraceFloat a, TraceFloat b) { return tr_op(TK_CMP, a, b, std::fmin(a.v, b.v)); }
inline TraceFloat s_max(TraceFloat a, TraceFloat b) { return tr_op(TK_CMP, a, b, std::fmax(a.v, b.v)); }

// Marks the state one march step hands to the next (loop-variant); a no-op
// for the arithmetic scalars.
inline void mark_carried(float&) {}
inline void mark_carried(double&) {}
inline void mark_carried(CountingFloat&) {}
inline void mark_carried(TraceFloat& x) { x.id = tape().push(TK_FREE, x.id, -1, false); }

template <class T> inline T lit(double x) { return T(x); }
template <> inline float lit<float>(double x) { return float(x); }

// ---------------------------------------------------------------------------
// vec3 / vec4
// ---------------------------------------------------------------------------
template <class T> struct V3 {
  T x, y, z;
  V3() : x(0), y(0), z(0) {}
  V3(T a, T b, T c) : x(a), y(b), z(c) {}
};
template <class T> struct V4 {
  T x, y, z, w;
};
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline T dot(V3<T> a, V3<T> b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <class T> inline V3<T> cross(V3<T> a, V3<T> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> inline T length(V3<T> a) { return s_sqrt(dot(a, a)); }
template <class T> inline V3<T> normalize(V3<T> a) {
  T l = s_sqrt(dot(a, a));
  return {a.x / l, a.y / l, a.z / l};
}
template <class T> inline V3<T> vabs(V3<T> a) { return {s_abs(a.x), s_abs(a.y), s_abs(a.z)}; }
template <class T> inline void mark_carried(V3<T>& a) {
  mark_carried(a.x);
  mark_carried(a.y);
  mark_carried(a.z);
}
// WGSL reflect(e1, e2) = e1 - 2 * dot(e2, e1) * e2
template <class T> inline V3<T> reflect(V3<T> e1, V3<T> e2) {
  T d = lit<T>(2.0) * dot(e2, e1);
  return e1 - d * e2;
}
// mat3x3(c0, c1, c2) * v, columns summed in order (column-major WGSL).
template <class T> inline V3<T> mat3_mul(V3<T> c0, V3<T> c1, V3<T> c2, V3<T> v) {
  return (c0 * v.x + c1 * v.y) + c2 * v.z;
}

// ---------------------------------------------------------------------------
// Helpers, src/main_view.wgsl:76-146
// ---------------------------------------------------------------------------
template <class T> inline T PI() { return lit<T>(3.141592653589793); }

template <class T> inline V3<T> rotateX(V3<T> v, T phi) {  // wgsl:78-84
  T c = s_cos(phi), s = s_sin(phi);
  T z = lit<T>(0.0), o = lit<T>(1.0);
  return mat3_mul(V3<T>(o, z, z), V3<T>(z, c, s), V3<T>(z, -s, c), v);
}
template <class T> inline V3<T> rotateY(V3<T> v, T phi) {  // wgsl:86-92
  T c = s_cos(phi), s = s_sin(phi);
  T z = lit<T>(0.0), o = lit<T>(1.0);
  return mat3_mul(V3<T>(c, z, -s), V3<T>(z, o, z), V3<T>(s, z, c), v);
}
template <class T> inline V3<T> rotateZ(V3<T> v, T phi) {  // wgsl:94-100 (third column is zero)
  T c = s_cos(phi), s = s_sin(phi);
  T z = lit<T>(0.0);
  return mat3_mul(V3<T>(c, s, z), V3<T>(-s, c, z), V3<T>(z, z, z), v);
}
template <class T> inline V3<T> translate(V3<T> v, T dx, T dy, T dz) {  // wgsl:102-108
  return {v.x + dx, v.y + dy, v.z + dz};
}
template <class T> inline T refraction_index(T t) {  // wgsl:111-117
  T air_pressure = lit<T>(101325.0);
  T c1 = lit<T>(0.0000104);
  T c2 = lit<T>(0.00366);
  T one = lit<T>(1.0);
  T p10 = lit<T>(1e-10);  // pow(10.0, -10.0)
  return c1 * air_pressure * (one + air_pressure * (lit<T>(60.1) - lit<T>(0.972) * t) * p10) /
         (one + c2 * t);
}
template <class T> inline V3<T> refraction(T t_in, T t_out, V3<T> v_in, V3<T> n) {  // wgsl:119-136
  T eta_in = refraction_index(t_in);
  T eta_out = refraction_index(t_out);
  T cosi = s_min(s_max(lit<T>(-1.0), lit<T>(1.0)), dot(v_in, n));  // clamp(-1.0, 1.0, x)
  V3<T> n_ref = n;
  if (cosi < lit<T>(0.0)) {
    cosi = -cosi;
  } else {
    n_ref = -n;
  }
  T eta = eta_in / eta_out;
  T k = lit<T>(1.0) - eta * eta * (lit<T>(1.0) - cosi * cosi);
  if (k < lit<T>(0.0)) return reflect(v_in, n_ref);
  return eta * v_in + (eta * cosi - s_sqrt(k)) * n_ref;
}
template <class T> inline T point_plane_distance(V3<T> p, V3<T> n, V3<T> p0) {  // wgsl:138-142
  T d = dot(p0, n);
  return s_abs(dot(p, n) - d);
}
template <class T> inline T sigmoid(T x) { return lit<T>(1.0) / (lit<T>(1.0) + s_exp(-x)); }  // wgsl:144-146
template <class T> inline T clamp_wgsl(T e, T lo, T hi) { return s_min(s_max(e, lo), hi); }

// ---------------------------------------------------------------------------
// Field functions.  Ids follow enum linon_predefined in include/linon.h.
// Bodies: src/functions.rs:33-128; stub: main_view.wgsl:148.
// ---------------------------------------------------------------------------
enum FieldId {
  F_CUSTOM = 0, F_MIRAGE_SPHERICAL = 1, F_MIRAGE_PLANE = 2, F_MIRAGE_SPHERICAL_SIGMOID = 3,
  F_MIRAGE_PLANE_SIGMOID = 4, F_TRANSLATION_X = 5, F_TRANSLATION_Z = 6, F_ROTATION = 7,
  F_LORENZ = 8, F_ROESSLER = 9, F_IDENTITY = 10, F_LINEAR = 11, F_TWIST = 12, F_LENS = 13,
  F_LORENZ_SCALED = 14, F_COUNT = 15
};

template <class T>
inline V3<T> mirage_spherical(V3<T> p_prev, V3<T> p, V3<T> v, bool sig) {  // functions.rs:36-50,67-81
  T t_env = lit<T>(15.0), t_src = lit<T>(200.0), max_dist = lit<T>(0.25);
  V3<T> center(lit<T>(-0.5), lit<T>(0.5), lit<T>(-0.5));
  V3<T> center_dest = p - center;
  V3<T> normal = normalize(center_dest);
  T dist_in = length(p_prev - center);
  T dist_out = length(center_dest);
  T part_in, part_out;
  if (sig) {
    part_in = clamp_wgsl(lit<T>(0.0), lit<T>(1.0), sigmoid(dist_in / max_dist * lit<T>(12.0) - lit<T>(6.0)));
    part_out = clamp_wgsl(lit<T>(0.0), lit<T>(1.0), sigmoid(dist_out / max_dist * lit<T>(12.0) - lit<T>(6.0)));
  } else {
    part_in = clamp_wgsl(lit<T>(0.0), lit<T>(1.0), dist_in / max_dist);
    part_out = clamp_wgsl(lit<T>(0.0), lit<T>(1.0), dist_out / max_dist);
  }
  T t_in = part_in * t_env + (lit<T>(1.0) - part_in) * t_src;
  T t_out = part_out * t_env + (lit<T>(1.0) - part_out) * t_src;
  return refraction(t_in, t_out, v, normal);
}
template <class T>
inline V3<T> mirage_plane(V3<T> p_prev, V3<T> p, V3<T> v, bool sig) {  // functions.rs:52-65,83-96
  T t_env = lit<T>(15.0), t_src = lit<T>(30.0), max_dist = lit<T>(0.01);
  V3<T> plane_p0(lit<T>(0.0), lit<T>(0.1), lit<T>(0.0));
  V3<T> plane_n(lit<T>(0.0), lit<T>(1.0), lit<T>(0.0));
  T dist_in = point_plane_distance(p_prev, plane_n, plane_p0);
  T dist_out = point_plane_distance(p, plane_n, plane_p0);
  T part_in, part_out;
  if (sig) {
    part_in = clamp_wgsl(lit<T>(0.0), lit<T>(1.0), sigmoid(dist_in / max_dist * lit<T>(12.0) - lit<T>(6.0)));
    part_out = clamp_wgsl(lit<T>(0.0), lit<T>(1.0), sigmoid(dist_out / max_dist * lit<T>(12.0) - lit<T>(6.0)));
  } else {
    part_in = clamp_wgsl(lit<T>(0.0), lit<T>(1.0), dist_in / max_dist);
    part_out = clamp_wgsl(lit<T>(0.0), lit<T>(1.0), dist_out / max_dist);
  }
  T t_in = part_in * t_env + (lit<T>(1.0) - part_in) * t_src;
  T t_out = part_out * t_env + (lit<T>(1.0) - part_out) * t_src;
  return refraction(t_in, t_out, v, plane_n);
}

template <class T>
inline V3<T> field_eval(int id, V3<T> p_prev, V3<T> p, V3<T> v0, V3<T> v, T t) {
  switch (id) {
    case F_MIRAGE_SPHERICAL: return mirage_spherical(p_prev, p, v, false);
    case F_MIRAGE_PLANE: return mirage_plane(p_prev, p, v, false);
    case F_MIRAGE_SPHERICAL_SIGMOID: return mirage_spherical(p_prev, p, v, true);
    case F_MIRAGE_PLANE_SIGMOID: return mirage_plane(p_prev, p, v, true);
    case F_TRANSLATION_X: {  // functions.rs:98-101
      T dx = lit<T>(0.5) * t, dy = lit<T>(0.0), dz = lit<T>(0.0);
      return translate(v0, dx, dy, dz);
    }
    case F_TRANSLATION_Z: {  // functions.rs:103-106
      T dx = lit<T>(0.0), dy = lit<T>(0.0), dz = lit<T>(0.5) * t;
      return translate(v0, dx, dy, dz);
    }
    case F_ROTATION:  // functions.rs:108
      return normalize(v0 + rotateZ(v0, PI<T>() * t));
    case F_LORENZ: {  // functions.rs:109-116
      T rho = lit<T>(28.0), sigma = lit<T>(10.0), beta = lit<T>(8.0 / 3.0);
      return {sigma * (p.y - p.x), p.x * (rho - p.z) - p.y, p.x * p.y - beta * p.z};
    }
    case F_ROESSLER: {  // functions.rs:118-125
      T a = lit<T>(0.1), b = lit<T>(0.1), c = lit<T>(14.0);
      return {-p.y - p.z, p.x + a * p.y, b + p.z * (p.x - c)};
    }
    case F_IDENTITY: return v;  // main_view.wgsl:148
    case F_LINEAR: return v0;
    case F_TWIST: return rotateY(v0, lit<T>(0.5) * p.y);
    case F_LENS: {  // normalize(v - 0.05 * p / pow(dot(p, p) + 0.01, 1.5))
      T den = s_pow(dot(p, p) + lit<T>(0.01), lit<T>(1.5));
      return normalize(v - (lit<T>(0.05) * p) / den);
    }
    case F_LORENZ_SCALED: {  // 0.05 * vec3(sigma(p.y-p.x), p.x(rho-p.z)-p.y, p.x p.y - beta p.z) + v0
      T sigma = lit<T>(10.0), rho = lit<T>(28.0), beta = lit<T>(8.0 / 3.0);
      V3<T> l(sigma * (p.y - p.x), p.x * (rho - p.z) - p.y, p.x * p.y - beta * p.z);
      return lit<T>(0.05) * l + v0;
    }
    default: {
      T nan = lit<T>(std::numeric_limits<double>::quiet_NaN());
      return {nan, nan, nan};
    }
  }
}

// ---------------------------------------------------------------------------
// Scene
// ---------------------------------------------------------------------------
// Candidate search for large scenes (the oracle's own, not the shader's):
// a uniform grid over the triangles' bounding boxes, each inflated by a
// margin far above any rounding of the Moeller-Trumbore quantities.  A
// segment is tested against the triangles listed in the cells its inflated
// box overlaps; since the closest hit is the lexicographic minimum of
// (t, face index) -- the brute-force loop's strict `<` in face order -- the
// order and repetition of candidates do not matter, and the result equals
// the loop over all faces (held bit for bit by a CPU test).
struct Accel {
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  double cell = 1.0, margin = 0.0;
  int n[3] = {0, 0, 0};
  std::vector<float> box;        // n_faces * 6 (inflated lo.xyz, hi.xyz)
  std::vector<uint32_t> start;   // cells + 1
  std::vector<uint32_t> items;   // face indices per cell
};

struct Scene {
  std::vector<float> xyz;      // n_vertices * 3
  std::vector<uint32_t> abc;   // n_faces * 3
  std::vector<float> face_rgb; // empty or n_faces * 3
  const Accel* accel = nullptr;  // NULL: every face is tested (the shader's loop)
  uint32_t n_faces() const { return uint32_t(abc.size() / 3); }
};

// Builds the grid: `res` cells along the longest axis of the scene's box.
inline void build_accel(const Scene& s, Accel& g, int res = 64) {
  const uint32_t nf = s.n_faces();
  g.box.assign(size_t(nf) * 6, 0.0f);
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (uint32_t i = 0; i < nf; ++i)
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) {
        const double x = s.xyz[3 * size_t(s.abc[3 * i + k]) + c];
        lo[c] = std::fmin(lo[c], x);
        hi[c] = std::fmax(hi[c], x);
      }
  double ext = 0.0;
  for (int c = 0; c < 3; ++c) ext = std::fmax(ext, hi[c] - lo[c]);
  if (!(ext > 0.0)) ext = 1.0;
  g.margin = 1e-3 * ext + 1e-6;
  for (uint32_t i = 0; i < nf; ++i)
    for (int c = 0; c < 3; ++c) {
      double a = 1e300, b = -1e300;
      for (int k = 0; k < 3; ++k) {
        const double x = s.xyz[3 * size_t(s.abc[3 * i + k]) + c];
        a = std::fmin(a, x);
        b = std::fmax(b, x);
      }
      g.box[6 * size_t(i) + c] = float(a - g.margin);
      g.box[6 * size_t(i) + 3 + c] = float(b + g.margin);
    }
  for (int c = 0; c < 3; ++c) {
    g.lo[c] = lo[c] - 2.0 * g.margin;
    g.hi[c] = hi[c] + 2.0 * g.margin;
  }
  double gext = 0.0;
  for (int c = 0; c < 3; ++c) gext = std::fmax(gext, g.hi[c] - g.lo[c]);
  g.cell = gext / res;
  for (int c = 0; c < 3; ++c) g.n[c] = std::max(1, int(std::ceil((g.hi[c] - g.lo[c]) / g.cell)));
  const size_t ncell = size_t(g.n[0]) * g.n[1] * g.n[2];
  std::vector<uint32_t> count(ncell + 1, 0);
  auto range = [&](uint32_t i, int c, int& a, int& b) {
    a = std::clamp(int(std::floor((double(g.box[6 * size_t(i) + c]) - g.lo[c]) / g.cell)), 0, g.n[c] - 1);
    b = std::clamp(int(std::floor((double(g.box[6 * size_t(i) + 3 + c]) - g.lo[c]) / g.cell)), 0, g.n[c] - 1);
  };
  for (int pass = 0; pass < 2; ++pass) {
    if (pass == 1) {
      g.start.assign(ncell + 1, 0);
      for (size_t c = 0; c < ncell; ++c) g.start[c + 1] = g.start[c] + count[c];
      g.items.assign(g.start[ncell], 0);
      std::fill(count.begin(), count.end(), 0);
    }
    for (uint32_t i = 0; i < nf; ++i) {
      int a[3], b[3];
      for (int c = 0; c < 3; ++c) range(i, c, a[c], b[c]);
      for (int z = a[2]; z <= b[2]; ++z)
        for (int y = a[1]; y <= b[1]; ++y)
          for (int x = a[0]; x <= b[0]; ++x) {
            const size_t cidx = (size_t(z) * g.n[1] + y) * g.n[0] + x;
            if (pass == 1) g.items[g.start[cidx] + count[cidx]] = i;
            count[cidx]++;
          }
    }
  }
}

template <class T> inline V3<T> vertex(const Scene& s, uint32_t i) {
  return V3<T>(lit<T>(s.xyz[3 * i]), lit<T>(s.xyz[3 * i + 1]), lit<T>(s.xyz[3 * i + 2]));
}

// hit_triangle, main_view.wgsl:150-175
template <class T>
inline T hit_triangle(V3<T> v0, V3<T> v1, V3<T> v2, V3<T> origin, V3<T> direction) {
  const T eps = lit<T>(0.0000001);
  V3<T> edge1 = v1 - v0;
  V3<T> edge2 = v2 - v0;
  V3<T> h = cross(direction, edge2);
  T a = dot(edge1, h);
  if (a > -eps && a < eps) return lit<T>(-1.0);
  T f = lit<T>(1.0) / a;
  V3<T> s = origin - v0;
  T u = f * dot(s, h);
  if (u < lit<T>(0.0) || u > lit<T>(1.0)) return lit<T>(-1.0);
  V3<T> q = cross(s, edge1);
  T v = f * dot(direction, q);
  if (v < lit<T>(0.0) || u + v > lit<T>(1.0)) return lit<T>(-1.0);
  T t = f * dot(edge2, q);
  if (t > eps) return t;
  return lit<T>(-1.0);
}

template <class T> struct ColorHit {
  V4<T> color;  // rgb + alpha (= hit distance, 0 for a miss)
  int32_t face;
};

// ray_color, main_view.wgsl:177-220.  Closest hit over all faces with strict
// `<`, so ties keep the lower face index.
template <class T> inline double to_double(T x) { return double(x); }
template <> inline double to_double<CountingFloat>(CountingFloat x) { return double(x.v); }
template <> inline double to_double<TraceFloat>(TraceFloat x) { return double(x.v); }

// Candidate faces of a segment from the grid; false when the grid does not
// apply (no grid, non-finite segment, or a segment spanning more cells than
// there are faces), and the caller tests every face.
template <class T>
inline bool grid_candidates(const Scene& sc, V3<T> origin, V3<T> direction, T max_dist,
                            std::vector<uint32_t>& out) {
  const Accel* g = sc.accel;
  if (!g) return false;
  const double o[3] = {to_double(origin.x), to_double(origin.y), to_double(origin.z)};
  const double d[3] = {to_double(direction.x), to_double(direction.y), to_double(direction.z)};
  const double L = to_double(max_dist);
  double smin[3], smax[3];
  for (int c = 0; c < 3; ++c) {
    if (!std::isfinite(o[c]) || !std::isfinite(d[c]) || !std::isfinite(L)) return false;
    const double e = o[c] + d[c] * L;
    smin[c] = std::fmin(o[c], e) - g->margin;
    smax[c] = std::fmax(o[c], e) + g->margin;
  }
  out.clear();
  int a[3], b[3];
  for (int c = 0; c < 3; ++c) {
    if (smax[c] < g->lo[c] || smin[c] > g->hi[c]) return true;  // outside every face's box
    a[c] = std::clamp(int(std::floor((smin[c] - g->lo[c]) / g->cell)), 0, g->n[c] - 1);
    b[c] = std::clamp(int(std::floor((smax[c] - g->lo[c]) / g->cell)), 0, g->n[c] - 1);
  }
  const double cells = double(b[0] - a[0] + 1) * (b[1] - a[1] + 1) * (b[2] - a[2] + 1);
  if (cells > double(sc.n_faces())) return false;
  for (int z = a[2]; z <= b[2]; ++z)
    for (int y = a[1]; y <= b[1]; ++y)
      for (int x = a[0]; x <= b[0]; ++x) {
        const size_t cidx = (size_t(z) * g->n[1] + y) * g->n[0] + x;
        for (uint32_t k = g->start[cidx]; k < g->start[cidx + 1]; ++k) {
          const uint32_t i = g->items[k];
          const float* bx = &g->box[6 * size_t(i)];
          if (smax[0] < bx[0] || smin[0] > bx[3] || smax[1] < bx[1] || smin[1] > bx[4] ||
              smax[2] < bx[2] || smin[2] > bx[5])
            continue;
          out.push_back(i);
        }
      }
  return true;
}

template <class T>
inline ColorHit<T> ray_color(const Scene& sc, V3<T> origin, V3<T> direction, T max_dist) {
  T t = lit<T>(-1.0);
  V3<T> d1, d2;
  int32_t face = -1;
  const uint32_t nf = sc.n_faces();
  auto test = [&](uint32_t i) {
    V3<T> a = vertex<T>(sc, sc.abc[3 * i]);
    V3<T> b = vertex<T>(sc, sc.abc[3 * i + 1]);
    V3<T> c = vertex<T>(sc, sc.abc[3 * i + 2]);
    T t_new = hit_triangle(a, b, c, origin, direction);
    // strict `<` in face order == lexicographic minimum of (t, face)
    if (t_new > lit<T>(0.0) && t_new < max_dist &&
        (t < lit<T>(0.0) || t_new < t || (!(t < t_new) && int32_t(i) < face))) {
      t = t_new;
      d1 = b - a;
      d2 = c - a;
      face = int32_t(i);
    }
  };
  static thread_local std::vector<uint32_t> cand;
  if (grid_candidates(sc, origin, direction, max_dist, cand)) {
    for (uint32_t i : cand) test(i);
  } else {
    for (uint32_t i = 0; i < nf; ++i) test(i);
  }
  ColorHit<T> r;
  if (t > lit<T>(0.0) && t < max_dist) {
    V3<T> normal = normalize(cross(d1, d2));
    // ambient 0.01, light colour (1,1,1), shininess 64 (main_view.wgsl:65-70)
    T intensity = s_max(dot(normal, -direction), lit<T>(0.0));
    if (intensity == lit<T>(0.0)) intensity = s_max(dot(-normal, -direction), lit<T>(0.0));
    T spec = s_pow(intensity, lit<T>(64.0));
    T shade = (lit<T>(0.01) + intensity) + spec;
    V3<T> base = vabs(normal);
    if (!sc.face_rgb.empty()) {
      base = V3<T>(lit<T>(sc.face_rgb[3 * face]), lit<T>(sc.face_rgb[3 * face + 1]),
                   lit<T>(sc.face_rgb[3 * face + 2]));
    }
    r.color = {shade * base.x, shade * base.y, shade * base.z, t};
    r.face = face;
    return r;
  }
  r.color = {lit<T>(0.0), lit<T>(0.0), lit<T>(0.0), lit<T>(0.0)};
  r.face = -1;
  return r;
}

// ---------------------------------------------------------------------------
// March parameters (mirror of linon_march_params, in the oracle's own terms)
// ---------------------------------------------------------------------------
struct March {
  float h_initial = 0.1f;
  float t_max = 5.0f;
  int max_steps = 0;  // 0: loop while t <= t_max
  bool adaptive = true;
  float h_fine = 0.001f;
  float h_fine_above = 0.002f;
  bool stop_on_hit = false;
  bool kahan = false;
  float field_weight = 1.0f;
  float focal_length = 0.035f;
  float viewport_height = 0.025f;
  bool linear_mode = false;
};

template <class T> struct RayResult {
  V4<T> color;       // alpha forced to 1
  V4<T> mapping;     // endpoint (x,y,z,1)
  int32_t face;      // first hit face or -1
  int32_t steps;     // accepted RK4 steps
  int32_t retries;   // rejected (adaptive) steps
};

// Kahan-compensated accumulator step: sum += x with carry c.
template <class T> inline void kahan_add(T& sum, T& c, T x) {
  T y = x - c;
  T t = sum + y;
  c = (t - sum) - y;
  sum = t;
}

// nonlinear_ray_color, main_view.wgsl:229-279, generalised by March.
template <class T>
inline RayResult<T> nonlinear_ray_color(const Scene& sc, int field, V3<T> start_point,
                                        V3<T> start_dir, const March& m) {
  RayResult<T> res;
  const T field_weight = lit<T>(m.field_weight);
  bool has_color = false;
  V4<T> color{lit<T>(0.0), lit<T>(0.0), lit<T>(0.0), lit<T>(0.0)};
  int32_t face = -1;
  V3<T> cur_point = start_point;
  V3<T> cur_dir = start_dir;
  T t = lit<T>(0.0);
  V3<T> last_v(lit<T>(0.0), lit<T>(0.0), lit<T>(0.0));
  T last_diff = lit<T>(-1.0);
  const T h_initial = lit<T>(m.h_initial);
  const T h_fine = lit<T>(m.h_fine);
  const T h_fine_above = lit<T>(m.h_fine_above);
  const T t_max = lit<T>(m.t_max);
  T h = h_initial;
  V3<T> comp_p;  // Kahan carries
  T comp_t = lit<T>(0.0);
  int32_t steps = 0, retries = 0;
  const T half = lit<T>(0.5), two = lit<T>(2.0), six = lit<T>(6.0), ten = lit<T>(10.0);

  for (;;) {
    // the state this step receives from the previous one (for TraceFloat)
    mark_carried(cur_point);
    mark_carried(cur_dir);
    mark_carried(t);
    mark_carried(comp_p);
    mark_carried(comp_t);
    if (m.adaptive) {  // otherwise h stays h_initial and these are unused
      mark_carried(h);
      mark_carried(last_v);
      mark_carried(last_diff);
    }
    if (m.max_steps > 0) {
      if (steps >= m.max_steps) break;
    } else {
      if (!(t <= t_max)) break;
    }
    // Runge-Kutta method (main_view.wgsl:245-250)
    V3<T> k1 = field_eval<T>(field, cur_point, cur_point, start_dir, cur_dir, t);
    V3<T> k2 = field_eval<T>(field, cur_point, cur_point + (half * h) * k1, start_dir, k1, t + half * h);
    V3<T> k3 = field_eval<T>(field, cur_point, cur_point + (half * h) * k2, start_dir, k2, t + half * h);
    V3<T> k4 = field_eval<T>(field, cur_point, cur_point + h * k3, start_dir, k3, t + h);
    V3<T> v = (((k1 + two * k2) + two * k3) + k4) / six;
    T diff = length(v - last_v);
    if (m.adaptive && last_diff >= lit<T>(0.0) && diff > ten * last_diff && h > h_fine_above) {
      h = h_fine;  // main_view.wgsl:252-255: refine and retry without advancing
      retries++;
      continue;
    }
    cur_dir = (lit<T>(1.0) - field_weight) * cur_dir + field_weight * v;
    V3<T> step_dir = cur_dir * h;
    if (!has_color) {
      ColorHit<T> ch = ray_color(sc, cur_point, normalize(step_dir), length(step_dir));
      color = ch.color;
      has_color = color.w > lit<T>(0.0);
      if (has_color) face = ch.face;
    }
    if (m.kahan) {
      kahan_add(cur_point.x, comp_p.x, step_dir.x);
      kahan_add(cur_point.y, comp_p.y, step_dir.y);
      kahan_add(cur_point.z, comp_p.z, step_dir.z);
      kahan_add(t, comp_t, h);
    } else {
      cur_point = cur_point + step_dir;
      t = t + h;
    }
    last_v = v;
    // (h only leaves h_initial through the adaptive refinement above, so the
    // restore needs m.adaptive; the guard changes no result)
    if (m.adaptive && two * diff < last_diff && h < h_initial) h = h_initial;
    last_diff = diff;
    steps++;
    if (m.stop_on_hit && has_color) break;
  }
  res.mapping = {cur_point.x, cur_point.y, cur_point.z, lit<T>(1.0)};
  color.w = lit<T>(1.0);
  if (!has_color) color = {lit<T>(0.0), lit<T>(0.0), lit<T>(0.0), lit<T>(1.0)};
  res.color = color;
  res.face = face;
  res.steps = steps;
  res.retries = retries;
  return res;
}

// ---------------------------------------------------------------------------
// Camera and primary rays, main_view.wgsl:347-366
// ---------------------------------------------------------------------------
struct Camera {
  float origin[3];
  float view_direction[3];
  float up[3];
};

template <class T> struct CameraBasis {
  V3<T> origin, view_direction, nh, nv;
  T width, height, vw, vh, focal;
};

template <class T>
inline CameraBasis<T> camera_basis(const Camera& c, int W, int H, const March& m) {
  CameraBasis<T> b;
  b.width = lit<T>(double(W));
  b.height = lit<T>(double(H));
  T aspect = b.width / b.height;
  b.origin = V3<T>(lit<T>(c.origin[0]), lit<T>(c.origin[1]), lit<T>(c.origin[2]));
  b.view_direction =
      V3<T>(lit<T>(c.view_direction[0]), lit<T>(c.view_direction[1]), lit<T>(c.view_direction[2]));
  V3<T> up(lit<T>(c.up[0]), lit<T>(c.up[1]), lit<T>(c.up[2]));
  b.focal = lit<T>(m.focal_length);
  b.vh = lit<T>(m.viewport_height);
  b.vw = aspect * b.vh;
  V3<T> w = -b.view_direction;
  V3<T> horizontal = cross(up, w);
  V3<T> vertical = cross(w, horizontal);
  b.nh = normalize(horizontal);
  b.nv = normalize(vertical);
  return b;
}

// Direction for invocation (gx, gy) (gy counts from the bottom row).
template <class T> inline V3<T> primary_dir(const CameraBasis<T>& b, int gx, int gy) {
  T u = lit<T>(double(gx)) / (b.width - lit<T>(1.0)) * b.vw - lit<T>(0.5) * b.vw;
  T v = lit<T>(double(gy)) / (b.height - lit<T>(1.0)) * b.vh - lit<T>(0.5) * b.vh;
  V3<T> s = (u * b.nh + v * b.nv) + b.focal * b.view_direction;
  return normalize(s);
}
// Direction for a normalised position (main_view.wgsl:475-478).
template <class T> inline V3<T> position_dir(const CameraBasis<T>& b, T px, T py) {
  T u2 = px * b.vw - lit<T>(0.5) * b.vw;
  T v2 = py * b.vh - lit<T>(0.5) * b.vh;
  V3<T> s2 = (u2 * b.nh + v2 * b.nv) + b.focal * b.view_direction;
  return normalize(s2);
}

// rgba8unorm store: clamp to [0,1], scale by 255, round half to even.
inline uint8_t unorm8(float x) {
  float c = std::fmin(std::fmax(x, 0.0f), 1.0f);
  return uint8_t(std::nearbyint(c * 255.0f));
}

// Render one pixel given its storage row (row 0 = top).
template <class T>
inline RayResult<T> render_pixel(const Scene& sc, int field, const CameraBasis<T>& b, int W, int H,
                                 int x, int row, const March& m) {
  int gy = H - 1 - row;
  V3<T> dir = primary_dir(b, x, gy);
  if (m.linear_mode) {  // main_view.wgsl:368-370
    ColorHit<T> ch = ray_color(sc, b.origin, dir, lit<T>(100.0));
    RayResult<T> r;
    r.color = ch.color;  // alpha = hit distance, as stored by the shader
    r.mapping = {lit<T>(0.0), lit<T>(0.0), lit<T>(0.0), lit<T>(0.0)};
    r.face = ch.face;
    r.steps = 0;
    r.retries = 0;
    return r;
  }
  (void)W;
  return nonlinear_ray_color(sc, field, b.origin, dir, m);
}

// sample_rays, main_view.wgsl:281-314: records the position before every
// `every`-th step; n_steps steps of size h, no intersection, no adaptivity.
// With record_final the final position follows the recorded ones (slot
// ceil(n_steps / every), the general capture's layout).
template <class T>
inline void sample_ray(int field, V3<T> start_point, V3<T> start_dir, T field_weight, T h,
                       int n_steps, int every, bool record_final, float* out /* npts*4 */) {
  V3<T> cur_point = start_point, cur_dir = start_dir;
  T t = lit<T>(0.0);
  const T half = lit<T>(0.5), two = lit<T>(2.0), six = lit<T>(6.0);
  for (int i = 0; i < n_steps; ++i) {
    V3<T> k1 = field_eval<T>(field, cur_point, cur_point, start_dir, cur_dir, t);
    V3<T> k2 = field_eval<T>(field, cur_point, cur_point + (half * h) * k1, start_dir, k1, t + half * h);
    V3<T> k3 = field_eval<T>(field, cur_point, cur_point + (half * h) * k2, start_dir, k2, t + half * h);
    V3<T> k4 = field_eval<T>(field, cur_point, cur_point + h * k3, start_dir, k3, t + h);
    V3<T> v = (((k1 + two * k2) + two * k3) + k4) / six;
    cur_dir = (lit<T>(1.0) - field_weight) * cur_dir + field_weight * v;
    V3<T> step_dir = cur_dir * h;
    if (i % every == 0) {
      float* o = out + 4 * (i / every);
      o[0] = float(cur_point.x); o[1] = float(cur_point.y); o[2] = float(cur_point.z); o[3] = 1.0f;
    }
    cur_point = cur_point + step_dir;
    t = t + h;
  }
  if (record_final) {  // after the ceil(n_steps / every) recorded points
    float* o = out + 4 * ((n_steps + every - 1) / every);
    o[0] = float(cur_point.x); o[1] = float(cur_point.y); o[2] = float(cur_point.z); o[3] = 1.0f;
  }
}

// ---------------------------------------------------------------------------
// Overlay, src/overlay.wgsl:4-40,99-135 (FP32 as written, or FP64)
// ---------------------------------------------------------------------------
template <class T> inline T lyapunov_exponent(const float* mapping, int W, int x, int y, int delta) {
  auto ld = [&](int xx, int yy) {
    const float* q = mapping + 4 * (size_t(yy) * W + xx);
    return V3<T>(lit<T>(q[0]), lit<T>(q[1]), lit<T>(q[2]));
  };
  V3<T> x_next = ld(x + delta, y), x_prev = ld(x - delta, y);
  V3<T> y_next = ld(x, y + delta), y_prev = ld(x, y - delta);
  V3<T> g0 = lit<T>(0.5) * (x_next - x_prev);
  V3<T> g1 = lit<T>(0.5) * (y_next - y_prev);
  // m = transpose(G) * G
  T m00 = dot(g0, g0), m01 = dot(g0, g1), m10 = dot(g1, g0), m11 = dot(g1, g1);
  // mat2eigenvalues -> mat2invariants -> vec2squareroots (overlay.wgsl:4-40)
  // m[0] = (m00, m01) column 0, m[1] = (m10, m11) column 1
  T a0 = m00 * m11 - m01 * m10;  // det: m[0].x*m[1].y - m[0].y*m[1].x
  T a1 = -(m00 + m11);
  T discrim = a1 * a1 - lit<T>(4.0) * a0;
  T e0, e1;
  if (discrim >= lit<T>(0.0)) {
    T root = s_sqrt(discrim);
    e0 = (-a1 - root) / lit<T>(2.0);
    e1 = (-a1 + root) / lit<T>(2.0);
  } else {
    T root = s_sqrt(-discrim);
    e0 = -a1 / lit<T>(2.0);
    e1 = root / lit<T>(2.0);
  }
  return s_sqrt(s_max(e0, e1));
}

// overlay(): returns the colour to store; writes the exponent when computed.
// rgba: input ray-casting image (rgba8), row-major rows of the storage texture.
template <class T>
inline void overlay_pixel(const uint8_t* rgba, const float* mapping, int W, int H, int x, int y,
                          int overlay_mode, int delta, float scaling, float out_rgba[4],
                          float* exponents, bool* wrote_exponent) {
  const uint8_t* c8 = rgba + 4 * (size_t(y) * W + x);
  float color[4] = {c8[0] / 255.0f, c8[1] / 255.0f, c8[2] / 255.0f, c8[3] / 255.0f};
  for (int i = 0; i < 4; ++i) out_rgba[i] = color[i];
  *wrote_exponent = false;
  if (overlay_mode == 0) return;
  int padding = delta * 2;
  if (x < padding || y < padding || x >= W - padding || y >= H - padding) return;
  if (overlay_mode == 1) {
    T exponent = lyapunov_exponent<T>(mapping, W, x, y, delta);
    float e = float(exponent);
    float scaled;
    if (sizeof(T) == sizeof(double)) {
      scaled = float(std::exp(double(scaling) * double(exponent) - 5.0));
    } else {
      scaled = std::exp(scaling * e - 5.0f);
    }
    exponents[size_t(y) * W + x] = scaled;
    *wrote_exponent = true;
    if (scaled >= 0.8f) {
      float alpha = std::fmin(1.0f, scaled) * 0.5f;
      for (int i = 0; i < 4; ++i) out_rgba[i] = alpha * 1.0f + (1.0f - alpha) * color[i];
    }
  }
}

inline float srgb_from_linear(float c) {  // overlay.wgsl:148-154
  if (c < 0.0031308f) return c / 12.92f;
  return 1.055f * std::pow(c, 1.0f / 2.4f) - 0.055f;
}

// ---------------------------------------------------------------------------
// Outline-ray selection, main_view.wgsl:381-468 (the shader's 8 scans, with
// the exponent buffer indexed y*stride+x).  Returns pixel (x,y) per slot.
// ---------------------------------------------------------------------------
inline void outline_select(const float* e, int W, int H, int stride, float min_exp, int px[8],
                           int py[8]) {
  auto E = [&](int x, int y) { return e[size_t(y) * stride + x]; };
  for (int g = 0; g < 8; ++g) {
    int bx = 0, by = 0, sum = 0;
    bool found = false;
    switch (g) {
      case 0:  // bottom left
        for (int x = 0; x < W; ++x)
          for (int y = 0; y < H; ++y)
            if (E(x, y) >= min_exp && (W - x) + y >= sum) { bx = x; by = y; sum = (W - x) + y; }
        break;
      case 1:  // bottom middle (the shader starts y at size.x - 1)
        for (int y = W - 1; y >= 0 && !found; --y)
          for (int x = 0; x < W && !found; ++x)
            if (y < H && E(x, y) >= min_exp) { bx = x; by = y; found = true; }
        break;
      case 2:  // bottom right
        for (int x = 0; x < W; ++x)
          for (int y = 0; y < H; ++y)
            if (E(x, y) >= min_exp && x + y >= sum) { bx = x; by = y; sum = x + y; }
        break;
      case 3:  // middle right
        for (int x = W - 1; x >= 0 && !found; --x)
          for (int y = 0; y < H && !found; ++y)
            if (E(x, y) >= min_exp) { bx = x; by = y; found = true; }
        break;
      case 4:  // top right
        for (int x = 0; x < W; ++x)
          for (int y = 0; y < H; ++y)
            if (E(x, y) >= min_exp && x + (H - y) >= sum) { bx = x; by = y; sum = x + (H - y); }
        break;
      case 5:  // top middle
        for (int y = 0; y < H && !found; ++y)
          for (int x = 0; x < W && !found; ++x)
            if (E(x, y) >= min_exp) { bx = x; by = y; found = true; }
        break;
      case 6:  // top left
        for (int x = 0; x < W; ++x)
          for (int y = 0; y < H; ++y)
            if (E(x, y) >= min_exp && (W - x) + (H - y) >= sum) {
              bx = x; by = y; sum = (W - x) + (H - y);
            }
        break;
      case 7:  // middle left
        for (int x = 0; x < W && !found; ++x)
          for (int y = 0; y < H && !found; ++y)
            if (E(x, y) >= min_exp) { bx = x; by = y; found = true; }
        break;
    }
    px[g] = bx;
    py[g] = by;
  }
}

}  // namespace linon_oracle
