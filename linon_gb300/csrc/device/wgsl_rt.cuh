// wgsl_rt.cuh — the WGSL value types, builtins and linon helper functions
// that field functions lowered by the WGSL front end are written against.
//
// Compiled three ways: by NVRTC into every march module (device), by nvcc into
// the ahead-of-time kernels, and by a host C++ compiler when the test suite
// checks the front end's output on the CPU.  No system headers are needed on
// the device side (NVRTC provides the CUDA math functions).
//
// Semantics follow the WGSL spec; where WGSL leaves a choice to the
// implementation this file makes the same choice as the FP32 restatement of
// the shader (dot sums x,y then z; M*v sums columns in order; clamp(e,lo,hi)
// = min(max(e,lo),hi); min/max are IEEE fmin/fmax).  With LINON_PRECISE
// defined every builtin is op-for-op that restatement; otherwise normalize and
// inverseSqrt use the hardware reciprocal square root.
#pragma once

#if defined(__CUDACC__)
#define WG_HD __host__ __device__ __forceinline__
#else
#define WG_HD inline
#include <math.h>
#endif

namespace wgsl {

// ---------------------------------------------------------------------------
// scalar math
// ---------------------------------------------------------------------------
// Reciprocal square root of fast modules: the special-function unit's
// approximation with a subnormal argument flushed to zero (result +inf).
// rsqrtf keeps subnormal arguments exact by scaling them, which costs a
// compare and two predicated multiplies around every call; the only inputs
// that need it are squared lengths below 2^-126 (vectors shorter than
// 1.1e-19), whose normalisation then gives inf or NaN instead of a unit
// vector.
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ float rsqrt_ftz(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
#endif
WG_HD float rsqrt_(float x) {
#if defined(__CUDA_ARCH__) && !defined(LINON_PRECISE)
  return rsqrt_ftz(x);
#else
  return 1.0f / sqrtf(x);
#endif
}
WG_HD float fmin_(float a, float b) { return fminf(a, b); }
WG_HD float fmax_(float a, float b) { return fmaxf(a, b); }
WG_HD int imin_(int a, int b) { return a < b ? a : b; }
WG_HD int imax_(int a, int b) { return a > b ? a : b; }
WG_HD unsigned umin_(unsigned a, unsigned b) { return a < b ? a : b; }
WG_HD unsigned umax_(unsigned a, unsigned b) { return a > b ? a : b; }
WG_HD float f32_from_bits(unsigned u) {
  union { unsigned u; float f; } c;
  c.u = u;
  return c.f;
}
// f32 -> i32 / u32 conversions saturate (WGSL conversion rules); NaN -> 0
WG_HD int to_i32(float x) {
  if (!(x == x)) return 0;
  if (x >= 2147483520.0f) return 2147483647;
  if (x <= -2147483648.0f) return -2147483647 - 1;
  return int(x);
}
WG_HD int to_i32(int x) { return x; }
WG_HD int to_i32(unsigned x) { return int(x); }
WG_HD unsigned to_u32(float x) {
  if (!(x == x) || x <= 0.0f) return 0u;
  if (x >= 4294967040.0f) return 4294967295u;
  return unsigned(x);
}
WG_HD unsigned to_u32(int x) { return unsigned(x); }
WG_HD unsigned to_u32(unsigned x) { return x; }

// Sine and cosine of one argument with one range reduction (fast modules).
// Method: Cody & Waite's additive reduction x = k * P + r, the period split
// into floats, each product applied by an FMA.
// Default: P = 2 pi = P1 + P2 + e (|e| < 7.1e-15) and sin(r), cos(r) from
// the special-function unit, whose documented absolute error on [-pi, pi]
// is 2^-21.41.  For pi <= |x| < 2^22, x and k * P1 are multiples of 2^-22
// and differ by less than 4, so x - k * P1 is exact; the one rounding of
// the P2 step and k * |e| < 4.7e-9 leave the reduced argument within
// 1.3e-7 of the exact x - k * 2 pi (a third term of the split would change
// it by no more than k * |e|).  Measured against FP64: < 5e-7 for
// |x| <= 3000, < 1e-6 for |x| < 2^22 (there the rounding of x / (2 pi) can
// leave |r| a little above pi); beyond, the error grows with |x|, like the
// special-function unit's own; inf and NaN give NaN.  No quadrant
// bookkeeping or range branch is needed.  With LINON_SINCOS_POLY: P = pi/2,
// the Taylor series of sin to r^9 and of cos to r^10 on |r| <= pi/4
// (truncation below 2.5e-9 relative) and the quadrant's swap and signs
// (error below 2.5e-7); |x| >= 65536 takes the CUDA library's sincosf.
WG_HD void sincos_fast(float x, float* s, float* c) {
#if defined(__CUDA_ARCH__)
#if !defined(LINON_SINCOS_POLY)
  const float k = rintf(x * 0x1.45f306p-3f);  // x / (2 pi)
  float r = fmaf(-k, 0x1.921fb6p+2f, x);      // 2 pi = P1 + P2 + e
  r = fmaf(-k, -0x1.777a5cp-23f, r);
  *s = __sinf(r);
  *c = __cosf(r);
#else
  if (!(fabsf(x) < 65536.0f)) {
    sincosf(x, s, c);
    return;
  }
  const float q = rintf(x * 0x1.45f306p-1f);  // x * 2/pi
  float r = fmaf(-q, 0x1.921fb6p+0f, x);      // pi/2 = P1 + P2 + P3
  r = fmaf(-q, -0x1.777a5cp-25f, r);
  r = fmaf(-q, -0x1.ee59dap-50f, r);
  const float r2 = r * r;
  float ps = fmaf(r2, 2.75573192e-6f, -1.98412698e-4f);  // 1/9!, -1/7!
  ps = fmaf(r2, ps, 8.33333333e-3f);                       // 1/5!
  ps = fmaf(r2, ps, -1.66666667e-1f);                      // -1/3!
  const float sn = fmaf(r * r2, ps, r);
  float pc = fmaf(r2, -2.75573192e-7f, 2.48015873e-5f);   // -1/10!, 1/8!
  pc = fmaf(r2, pc, -1.38888889e-3f);                      // -1/6!
  pc = fmaf(r2, pc, 4.16666667e-2f);                       // 1/4!
  pc = fmaf(r2, pc, -0.5f);                                // -1/2!
  const float cs = fmaf(r2, pc, 1.0f);
  const int qi = int(q) & 3;
  const float a = (qi & 1) ? cs : sn;
  const float b = (qi & 1) ? sn : cs;
  *s = (qi & 2) ? -a : a;
  *c = ((qi + 1) & 2) ? -b : b;
#endif
#else
  *s = sinf(x);
  *c = cosf(x);
#endif
}

// sin/cos for the helpers: the shared reduction in fast modules, the CUDA
// library functions in precise modules (as the restatement uses its libm).
WG_HD void sincos_(float x, float* s, float* c) {
#if defined(LINON_PRECISE) || !defined(__CUDA_ARCH__)
  *s = sinf(x);
  *c = cosf(x);
#else
  sincos_fast(x, s, c);
#endif
}

WG_HD float sin_(float x) {
  float s, c;
  sincos_(x, &s, &c);
  return s;
}
WG_HD float cos_(float x) {
  float s, c;
  sincos_(x, &s, &c);
  return c;
}

// pow with an exponent known at the call site (the front end emits this for
// constant exponents).  Fast modules evaluate the common rational exponents
// with sqrt and products; precise modules keep powf.
WG_HD float pow_k(float x, float k) {
#if !defined(LINON_PRECISE) && defined(__CUDA_ARCH__)
  if (k == 1.0f) return x;
  if (k == 2.0f) return x * x;
  if (k == 3.0f) return x * x * x;
  if (k == 4.0f) { const float y = x * x; return y * y; }
  if (k == 0.5f) return sqrtf(x);
  if (k == 1.5f) return x * sqrtf(x);
  if (k == -0.5f) return rsqrt_ftz(x);
  if (k == -1.0f) return 1.0f / x;
  if (k == -1.5f) { const float r = rsqrt_ftz(x); return r * r * r; }
  if (k == -2.0f) { const float r = 1.0f / x; return r * r; }
  if (k == -3.0f) { const float r = 1.0f / x; return r * r * r; }
#endif
  return powf(x, k);
}

// a / pow(x, k) with k known at the call site (emitted by the front end):
// precise modules divide as written; fast modules multiply by pow(x, -k),
// which for k = 1.5 is rsqrt(x)^3 instead of a square root and a division.
template <class A> WG_HD A div_pow_k(const A& a, float x, float k) {
#if !defined(LINON_PRECISE) && defined(__CUDA_ARCH__)
  return a * pow_k(x, -k);
#else
  return a / powf(x, k);
#endif
}

// ---------------------------------------------------------------------------
// vectors
// ---------------------------------------------------------------------------
template <class T, int N> struct vec;

// (s * v) / pow(x, k) and (v * s) / pow(x, k), s a scalar, v a vector:
// precise modules evaluate as written; fast modules form the scalar factor
// s * pow(x, -k) first and scale v once (one multiply per component instead
// of two).
template <class V> WG_HD V div_pow_k_sv(float s, const V& v, float x, float k);
template <class V> WG_HD V div_pow_k_vs(const V& v, float s, float x, float k);

template <class T> struct vec<T, 2> {
  T x, y;
  WG_HD vec() : x(T(0)), y(T(0)) {}
  WG_HD vec(T a, T b) : x(a), y(b) {}
  WG_HD explicit vec(T s) : x(s), y(s) {}
  template <class U> WG_HD explicit vec(const vec<U, 2>& o) : x(T(o.x)), y(T(o.y)) {}
  WG_HD T& operator[](int i) { return i == 0 ? x : y; }
  WG_HD T operator[](int i) const { return i == 0 ? x : y; }
};
template <class T> struct vec<T, 3> {
  T x, y, z;
  WG_HD vec() : x(T(0)), y(T(0)), z(T(0)) {}
  WG_HD vec(T a, T b, T c) : x(a), y(b), z(c) {}
  WG_HD explicit vec(T s) : x(s), y(s), z(s) {}
  WG_HD vec(const vec<T, 2>& a, T c) : x(a.x), y(a.y), z(c) {}
  WG_HD vec(T a, const vec<T, 2>& b) : x(a), y(b.x), z(b.y) {}
  template <class U> WG_HD explicit vec(const vec<U, 3>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
  WG_HD T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  WG_HD T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> struct vec<T, 4> {
  T x, y, z, w;
  WG_HD vec() : x(T(0)), y(T(0)), z(T(0)), w(T(0)) {}
  WG_HD vec(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
  WG_HD explicit vec(T s) : x(s), y(s), z(s), w(s) {}
  WG_HD vec(const vec<T, 3>& a, T d) : x(a.x), y(a.y), z(a.z), w(d) {}
  WG_HD vec(T a, const vec<T, 3>& b) : x(a), y(b.x), z(b.y), w(b.z) {}
  WG_HD vec(const vec<T, 2>& a, const vec<T, 2>& b) : x(a.x), y(a.y), z(b.x), w(b.y) {}
  WG_HD vec(const vec<T, 2>& a, T c, T d) : x(a.x), y(a.y), z(c), w(d) {}
  WG_HD vec(T a, const vec<T, 2>& b, T d) : x(a), y(b.x), z(b.y), w(d) {}
  WG_HD vec(T a, T b, const vec<T, 2>& c) : x(a), y(b), z(c.x), w(c.y) {}
  template <class U>
  WG_HD explicit vec(const vec<U, 4>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)), w(T(o.w)) {}
  WG_HD T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  WG_HD T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

// array<T, N>: value semantics (copied on assignment and by value into
// functions), zero-initialised by default; a runtime index is clamped to
// [0, N-1] (wgpu's default bounds-check policy).
template <class T, int N>
struct arr {
  T v[N];
  WG_HD arr() : v{} {}
  template <class... A>
  WG_HD explicit arr(const T& a0, const A&... a) : v{a0, T(a)...} {
    static_assert(sizeof...(A) + 1 == N, "array constructor with the wrong number of elements");
  }
  WG_HD T& operator[](int i) { return v[i < 0 ? 0 : (i >= N ? N - 1 : i)]; }
  WG_HD const T& operator[](int i) const { return v[i < 0 ? 0 : (i >= N ? N - 1 : i)]; }
  WG_HD T& operator[](unsigned i) { return v[i >= unsigned(N) ? unsigned(N - 1) : i]; }
  WG_HD const T& operator[](unsigned i) const { return v[i >= unsigned(N) ? unsigned(N - 1) : i]; }
};

// s * x^-k; for k = 1.5 as (s r)(r r), r = rsqrt(x): two dependent
// multiplies after the square root instead of three
WG_HD float scaled_pow_neg_k(float s, float x, float k) {
#if !defined(LINON_PRECISE) && defined(__CUDA_ARCH__)
  if (k == 1.5f) {
    const float r = rsqrt_ftz(x);
    return (s * r) * (r * r);
  }
#endif
  return s * pow_k(x, -k);
}
template <class V> WG_HD V div_pow_k_sv(float s, const V& v, float x, float k) {
#if !defined(LINON_PRECISE) && defined(__CUDA_ARCH__)
  return v * scaled_pow_neg_k(s, x, k);
#else
  return (s * v) / powf(x, k);
#endif
}
template <class V> WG_HD V div_pow_k_vs(const V& v, float s, float x, float k) {
#if !defined(LINON_PRECISE) && defined(__CUDA_ARCH__)
  return v * scaled_pow_neg_k(s, x, k);
#else
  return (v * s) / powf(x, k);
#endif
}

// bitcast<T>(e): the bits of a 32-bit scalar (or of each vector component)
// reinterpreted as another 32-bit scalar type.
template <class To, class From>
struct Bitcast {
  static WG_HD To go(const From& x) {
    static_assert(sizeof(To) == 4 && sizeof(From) == 4, "bitcast of 32-bit types");
    union {
      From f;
      To t;
    } c;
    c.f = x;
    return c.t;
  }
};
template <class To, class From, int N>
struct Bitcast<vec<To, N>, vec<From, N>> {
  static WG_HD vec<To, N> go(const vec<From, N>& x) {
    vec<To, N> r;
    for (int i = 0; i < N; ++i) r[i] = Bitcast<To, From>::go(x[i]);
    return r;
  }
};
template <class To, class From>
WG_HD To bitcast_(const From& x) {
  return Bitcast<To, From>::go(x);
}

typedef vec<float, 2> vec2f;
typedef vec<float, 3> vec3f;
typedef vec<float, 4> vec4f;
typedef vec<int, 2> vec2i;
typedef vec<int, 3> vec3i;
typedef vec<int, 4> vec4i;
typedef vec<unsigned, 2> vec2u;
typedef vec<unsigned, 3> vec3u;
typedef vec<unsigned, 4> vec4u;
typedef vec<bool, 2> vec2b;
typedef vec<bool, 3> vec3b;
typedef vec<bool, 4> vec4b;

// swizzle: swz<i,j,...>(v) evaluates v once.
template <int A, int B, class T, int N> WG_HD vec<T, 2> swz(const vec<T, N>& v) {
  return vec<T, 2>(v[A], v[B]);
}
template <int A, int B, int C, class T, int N> WG_HD vec<T, 3> swz(const vec<T, N>& v) {
  return vec<T, 3>(v[A], v[B], v[C]);
}
template <int A, int B, int C, int D, class T, int N> WG_HD vec<T, 4> swz(const vec<T, N>& v) {
  return vec<T, 4>(v[A], v[B], v[C], v[D]);
}

#define WG_VEC_BINOP(OP)                                                         \
  template <class T, int N> WG_HD vec<T, N> operator OP(const vec<T, N>& a,     \
                                                         const vec<T, N>& b) {  \
    vec<T, N> r;                                                                 \
    for (int i = 0; i < N; ++i) r[i] = a[i] OP b[i];                             \
    return r;                                                                    \
  }                                                                              \
  template <class T, int N> WG_HD vec<T, N> operator OP(const vec<T, N>& a, T s) { \
    vec<T, N> r;                                                                 \
    for (int i = 0; i < N; ++i) r[i] = a[i] OP s;                                \
    return r;                                                                    \
  }                                                                              \
  template <class T, int N> WG_HD vec<T, N> operator OP(T s, const vec<T, N>& a) { \
    vec<T, N> r;                                                                 \
    for (int i = 0; i < N; ++i) r[i] = s OP a[i];                                \
    return r;                                                                    \
  }
WG_VEC_BINOP(+)
WG_VEC_BINOP(-)
WG_VEC_BINOP(*)
WG_VEC_BINOP(/)
// bitwise operators of integer vectors (bool vectors use land / lor)
WG_VEC_BINOP(&)
WG_VEC_BINOP(|)
WG_VEC_BINOP(^)
#undef WG_VEC_BINOP

#if !defined(LINON_PRECISE) && defined(__CUDA_ARCH__)
// Fast modules divide a float vector by a scalar with one reciprocal.
template <int N> WG_HD vec<float, N> operator/(const vec<float, N>& a, float s) {
  const float r = 1.0f / s;
  vec<float, N> o;
  for (int i = 0; i < N; ++i) o[i] = a[i] * r;
  return o;
}
#endif

template <class T, int N> WG_HD vec<T, N> operator-(const vec<T, N>& a) {
  vec<T, N> r;
  for (int i = 0; i < N; ++i) r[i] = -a[i];
  return r;
}
template <class T, int N> WG_HD vec<T, N> operator~(const vec<T, N>& a) {  // integer vectors
  vec<T, N> r;
  for (int i = 0; i < N; ++i) r[i] = ~a[i];
  return r;
}
template <int N> WG_HD vec<bool, N> operator!(const vec<bool, N>& a) {
  vec<bool, N> r;
  for (int i = 0; i < N; ++i) r[i] = !a[i];
  return r;
}
template <class T, int N> WG_HD vec<T, N>& operator+=(vec<T, N>& a, const vec<T, N>& b) { a = a + b; return a; }
template <class T, int N> WG_HD vec<T, N>& operator-=(vec<T, N>& a, const vec<T, N>& b) { a = a - b; return a; }
template <class T, int N> WG_HD vec<T, N>& operator*=(vec<T, N>& a, const vec<T, N>& b) { a = a * b; return a; }
template <class T, int N> WG_HD vec<T, N>& operator/=(vec<T, N>& a, const vec<T, N>& b) { a = a / b; return a; }
template <class T, int N> WG_HD vec<T, N>& operator+=(vec<T, N>& a, T b) { a = a + b; return a; }
template <class T, int N> WG_HD vec<T, N>& operator-=(vec<T, N>& a, T b) { a = a - b; return a; }
template <class T, int N> WG_HD vec<T, N>& operator*=(vec<T, N>& a, T b) { a = a * b; return a; }
template <class T, int N> WG_HD vec<T, N>& operator/=(vec<T, N>& a, T b) { a = a / b; return a; }

// component-wise comparisons (vector results)
#define WG_VEC_CMP(NAME, OP)                                                            \
  template <class T, int N> WG_HD vec<bool, N> NAME(const vec<T, N>& a, const vec<T, N>& b) { \
    vec<bool, N> r;                                                                     \
    for (int i = 0; i < N; ++i) r[i] = a[i] OP b[i];                                    \
    return r;                                                                           \
  }                                                                                     \
  template <class T> WG_HD bool NAME(T a, T b) { return a OP b; }
WG_VEC_CMP(cmp_lt, <)
WG_VEC_CMP(cmp_le, <=)
WG_VEC_CMP(cmp_gt, >)
WG_VEC_CMP(cmp_ge, >=)
WG_VEC_CMP(cmp_eq, ==)
WG_VEC_CMP(cmp_ne, !=)
#undef WG_VEC_CMP
template <int N> WG_HD vec<bool, N> land(const vec<bool, N>& a, const vec<bool, N>& b) {
  vec<bool, N> r;
  for (int i = 0; i < N; ++i) r[i] = a[i] && b[i];
  return r;
}
template <int N> WG_HD vec<bool, N> lor(const vec<bool, N>& a, const vec<bool, N>& b) {
  vec<bool, N> r;
  for (int i = 0; i < N; ++i) r[i] = a[i] || b[i];
  return r;
}

// ---------------------------------------------------------------------------
// matrices (column major, C columns of R rows)
// ---------------------------------------------------------------------------
template <int C, int R> struct mat {
  vec<float, R> c[C];
  WG_HD mat() {}
  WG_HD vec<float, R>& operator[](int i) { return c[i]; }
  WG_HD const vec<float, R>& operator[](int i) const { return c[i]; }
};
template <int R> WG_HD mat<2, R> make_mat(const vec<float, R>& a, const vec<float, R>& b) {
  mat<2, R> m; m.c[0] = a; m.c[1] = b; return m;
}
template <int R>
WG_HD mat<3, R> make_mat(const vec<float, R>& a, const vec<float, R>& b, const vec<float, R>& c) {
  mat<3, R> m; m.c[0] = a; m.c[1] = b; m.c[2] = c; return m;
}
template <int R>
WG_HD mat<4, R> make_mat(const vec<float, R>& a, const vec<float, R>& b, const vec<float, R>& c,
                         const vec<float, R>& d) {
  mat<4, R> m; m.c[0] = a; m.c[1] = b; m.c[2] = c; m.c[3] = d; return m;
}
// matrix * vector: columns summed in order
template <int C, int R> WG_HD vec<float, R> operator*(const mat<C, R>& m, const vec<float, C>& v) {
  vec<float, R> r = m.c[0] * v[0];
  for (int k = 1; k < C; ++k) r = r + m.c[k] * v[k];
  return r;
}
template <int C, int R> WG_HD vec<float, C> operator*(const vec<float, R>& v, const mat<C, R>& m) {
  vec<float, C> r;
  for (int i = 0; i < C; ++i) {
    float s = v[0] * m.c[i][0];
    for (int k = 1; k < R; ++k) s = s + v[k] * m.c[i][k];
    r[i] = s;
  }
  return r;
}
template <int K, int R, int C2> WG_HD mat<C2, R> operator*(const mat<K, R>& a, const mat<C2, K>& b) {
  mat<C2, R> m;
  for (int j = 0; j < C2; ++j) m.c[j] = a * b.c[j];
  return m;
}
template <int C, int R> WG_HD mat<C, R> operator*(const mat<C, R>& a, float s) {
  mat<C, R> m;
  for (int j = 0; j < C; ++j) m.c[j] = a.c[j] * s;
  return m;
}
template <int C, int R> WG_HD mat<C, R> operator*(float s, const mat<C, R>& a) {
  mat<C, R> m;
  for (int j = 0; j < C; ++j) m.c[j] = s * a.c[j];
  return m;
}
template <int C, int R> WG_HD mat<C, R> operator+(const mat<C, R>& a, const mat<C, R>& b) {
  mat<C, R> m;
  for (int j = 0; j < C; ++j) m.c[j] = a.c[j] + b.c[j];
  return m;
}
template <int C, int R> WG_HD mat<C, R> operator-(const mat<C, R>& a, const mat<C, R>& b) {
  mat<C, R> m;
  for (int j = 0; j < C; ++j) m.c[j] = a.c[j] - b.c[j];
  return m;
}
template <int C, int R> WG_HD mat<C, R> operator-(const mat<C, R>& a) {
  mat<C, R> m;
  for (int j = 0; j < C; ++j) m.c[j] = -a.c[j];
  return m;
}
template <int C, int R> WG_HD mat<R, C> transpose(const mat<C, R>& a) {
  mat<R, C> m;
  for (int j = 0; j < C; ++j)
    for (int i = 0; i < R; ++i) m.c[i][j] = a.c[j][i];
  return m;
}
WG_HD float determinant(const mat<2, 2>& m) { return m.c[0].x * m.c[1].y - m.c[1].x * m.c[0].y; }
WG_HD float determinant(const mat<3, 3>& m) {
  return m.c[0].x * (m.c[1].y * m.c[2].z - m.c[2].y * m.c[1].z) -
         m.c[1].x * (m.c[0].y * m.c[2].z - m.c[2].y * m.c[0].z) +
         m.c[2].x * (m.c[0].y * m.c[1].z - m.c[1].y * m.c[0].z);
}

// ---------------------------------------------------------------------------
// builtins
// ---------------------------------------------------------------------------
#define WG_UNARY(NAME, EXPR)                                                       \
  WG_HD float NAME(float x) { return EXPR; }                                       \
  template <int N> WG_HD vec<float, N> NAME(const vec<float, N>& v) {              \
    vec<float, N> r;                                                               \
    for (int i = 0; i < N; ++i) r[i] = NAME(v[i]);                                 \
    return r;                                                                      \
  }
WG_UNARY(sin, sin_(x))
WG_UNARY(cos, cos_(x))
WG_UNARY(tan, tanf(x))
WG_UNARY(asin, asinf(x))
WG_UNARY(acos, acosf(x))
WG_UNARY(atan, atanf(x))
WG_UNARY(sinh, sinhf(x))
WG_UNARY(cosh, coshf(x))
WG_UNARY(tanh, tanhf(x))
WG_UNARY(asinh, asinhf(x))
WG_UNARY(acosh, acoshf(x))
WG_UNARY(atanh, atanhf(x))
WG_UNARY(exp, expf(x))
WG_UNARY(exp2, exp2f(x))
WG_UNARY(log, logf(x))
WG_UNARY(log2, log2f(x))
WG_UNARY(sqrt, sqrtf(x))
WG_UNARY(inverseSqrt, rsqrt_(x))
WG_UNARY(floor, floorf(x))
WG_UNARY(ceil, ceilf(x))
WG_UNARY(trunc, truncf(x))
WG_UNARY(round, rintf(x))
WG_UNARY(fract, x - floorf(x))
WG_UNARY(sign, (x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f)))
WG_UNARY(saturate, fmin_(fmax_(x, 0.0f), 1.0f))
WG_UNARY(degrees, x * 57.295779513082323f)
WG_UNARY(radians, x * 0.017453292519943295f)
#undef WG_UNARY

WG_HD float abs(float x) { return fabsf(x); }
WG_HD int abs(int x) { return x < 0 ? -x : x; }
WG_HD unsigned abs(unsigned x) { return x; }
template <class T, int N> WG_HD vec<T, N> abs(const vec<T, N>& v) {
  vec<T, N> r;
  for (int i = 0; i < N; ++i) r[i] = abs(v[i]);
  return r;
}

#define WG_BINARY(NAME, EXPR)                                                          \
  WG_HD float NAME(float a, float b) { return EXPR; }                                  \
  template <int N> WG_HD vec<float, N> NAME(const vec<float, N>& a, const vec<float, N>& b) { \
    vec<float, N> r;                                                                   \
    for (int i = 0; i < N; ++i) r[i] = NAME(a[i], b[i]);                               \
    return r;                                                                          \
  }
WG_BINARY(pow, powf(a, b))
WG_BINARY(atan2, atan2f(a, b))
WG_BINARY(step, (b >= a ? 1.0f : 0.0f))
WG_BINARY(fmod_wgsl, (a - b * truncf(a / b)))
#undef WG_BINARY
// e1 % e2 with a scalar on one side (the scalar applies to every component)
template <int N> WG_HD vec<float, N> fmod_wgsl(const vec<float, N>& a, float b) {
  vec<float, N> r;
  for (int i = 0; i < N; ++i) r[i] = fmod_wgsl(a[i], b);
  return r;
}
template <int N> WG_HD vec<float, N> fmod_wgsl(float a, const vec<float, N>& b) {
  vec<float, N> r;
  for (int i = 0; i < N; ++i) r[i] = fmod_wgsl(a, b[i]);
  return r;
}

// i32 + - * and unary - wrap on overflow (WGSL 8.7), computed in u32
WG_HD int add_i32(int a, int b) { return int(unsigned(a) + unsigned(b)); }
WG_HD int sub_i32(int a, int b) { return int(unsigned(a) - unsigned(b)); }
WG_HD int mul_i32(int a, int b) { return int(unsigned(a) * unsigned(b)); }
WG_HD int neg_i32(int a) { return int(0u - unsigned(a)); }
#define WG_I32_BINARY(NAME)                                                            \
  template <int N> WG_HD vec<int, N> NAME(const vec<int, N>& a, const vec<int, N>& b) { \
    vec<int, N> r;                                                                     \
    for (int i = 0; i < N; ++i) r[i] = NAME(a[i], b[i]);                               \
    return r;                                                                          \
  }                                                                                    \
  template <int N> WG_HD vec<int, N> NAME(const vec<int, N>& a, int b) {               \
    return NAME(a, vec<int, N>(b));                                                    \
  }                                                                                    \
  template <int N> WG_HD vec<int, N> NAME(int a, const vec<int, N>& b) {               \
    return NAME(vec<int, N>(a), b);                                                    \
  }
WG_I32_BINARY(add_i32)
WG_I32_BINARY(sub_i32)
WG_I32_BINARY(mul_i32)
#undef WG_I32_BINARY
template <int N> WG_HD vec<int, N> neg_i32(const vec<int, N>& a) {
  vec<int, N> r;
  for (int i = 0; i < N; ++i) r[i] = neg_i32(a[i]);
  return r;
}

// Integer division and remainder (WGSL 8.7): a / 0 = a, a % 0 = 0, and for
// i32 the most negative value over -1 gives itself / 0 (no trap, no
// undefined behaviour); otherwise truncating.
WG_HD int div_int(int a, int b) { return (b == 0 || (a == -2147483647 - 1 && b == -1)) ? a : a / b; }
WG_HD int mod_int(int a, int b) { return (b == 0 || (a == -2147483647 - 1 && b == -1)) ? 0 : a % b; }
WG_HD unsigned div_int(unsigned a, unsigned b) { return b == 0u ? a : a / b; }
WG_HD unsigned mod_int(unsigned a, unsigned b) { return b == 0u ? 0u : a % b; }
// Shifts by the amount's low 5 bits; left shifts of i32 through u32 (no
// signed overflow), right shifts of i32 arithmetic.
WG_HD int shl(int a, unsigned b) { return int(unsigned(a) << (b & 31u)); }
WG_HD unsigned shl(unsigned a, unsigned b) { return a << (b & 31u); }
WG_HD int shr(int a, unsigned b) { return a >> (b & 31u); }
WG_HD unsigned shr(unsigned a, unsigned b) { return a >> (b & 31u); }
#define WG_INT_BINARY(NAME, BT)                                                              \
  template <class T, int N> WG_HD vec<T, N> NAME(const vec<T, N>& a, const vec<BT, N>& b) { \
    vec<T, N> r;                                                                             \
    for (int i = 0; i < N; ++i) r[i] = NAME(a[i], b[i]);                                     \
    return r;                                                                                \
  }
WG_INT_BINARY(div_int, T)
WG_INT_BINARY(mod_int, T)
WG_INT_BINARY(shl, unsigned)
WG_INT_BINARY(shr, unsigned)
#undef WG_INT_BINARY
template <class T, int N> WG_HD vec<T, N> div_int(const vec<T, N>& a, T b) { return div_int(a, vec<T, N>(b)); }
template <class T, int N> WG_HD vec<T, N> div_int(T a, const vec<T, N>& b) { return div_int(vec<T, N>(a), b); }
template <class T, int N> WG_HD vec<T, N> mod_int(const vec<T, N>& a, T b) { return mod_int(a, vec<T, N>(b)); }
template <class T, int N> WG_HD vec<T, N> mod_int(T a, const vec<T, N>& b) { return mod_int(vec<T, N>(a), b); }

WG_HD float min(float a, float b) { return fmin_(a, b); }
WG_HD float max(float a, float b) { return fmax_(a, b); }
WG_HD int min(int a, int b) { return imin_(a, b); }
WG_HD int max(int a, int b) { return imax_(a, b); }
WG_HD unsigned min(unsigned a, unsigned b) { return umin_(a, b); }
WG_HD unsigned max(unsigned a, unsigned b) { return umax_(a, b); }
template <class T, int N> WG_HD vec<T, N> min(const vec<T, N>& a, const vec<T, N>& b) {
  vec<T, N> r;
  for (int i = 0; i < N; ++i) r[i] = min(a[i], b[i]);
  return r;
}
template <class T, int N> WG_HD vec<T, N> max(const vec<T, N>& a, const vec<T, N>& b) {
  vec<T, N> r;
  for (int i = 0; i < N; ++i) r[i] = max(a[i], b[i]);
  return r;
}
template <class T> WG_HD T clamp(T e, T lo, T hi) { return min(max(e, lo), hi); }
template <class T, int N>
WG_HD vec<T, N> clamp(const vec<T, N>& e, const vec<T, N>& lo, const vec<T, N>& hi) {
  return min(max(e, lo), hi);
}
WG_HD float fma(float a, float b, float c) { return fmaf(a, b, c); }
template <int N>
WG_HD vec<float, N> fma(const vec<float, N>& a, const vec<float, N>& b, const vec<float, N>& c) {
  vec<float, N> r;
  for (int i = 0; i < N; ++i) r[i] = fmaf(a[i], b[i], c[i]);
  return r;
}
// mix(e1, e2, e3) = e1 * (1 - e3) + e2 * e3
WG_HD float mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
template <int N> WG_HD vec<float, N> mix(const vec<float, N>& a, const vec<float, N>& b, float t) {
  return a * (1.0f - t) + b * t;
}
template <int N>
WG_HD vec<float, N> mix(const vec<float, N>& a, const vec<float, N>& b, const vec<float, N>& t) {
  return a * (vec<float, N>(1.0f) - t) + b * t;
}
WG_HD float smoothstep(float lo, float hi, float x) {
  float t = clamp((x - lo) / (hi - lo), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
template <int N>
WG_HD vec<float, N> smoothstep(const vec<float, N>& lo, const vec<float, N>& hi,
                               const vec<float, N>& x) {
  vec<float, N> r;
  for (int i = 0; i < N; ++i) r[i] = smoothstep(lo[i], hi[i], x[i]);
  return r;
}

WG_HD float dot(const vec2f& a, const vec2f& b) { return a.x * b.x + a.y * b.y; }
WG_HD float dot(const vec3f& a, const vec3f& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
WG_HD float dot(const vec4f& a, const vec4f& b) {
  return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w;
}
// dot(a, b) + s (emitted by the front end): precise modules and the host
// add as written; fast modules start the fused multiply-add chain at s
// (one operation and one dependent step fewer)
template <int N> WG_HD float dot_add(const vec<float, N>& a, const vec<float, N>& b, float s) {
#if defined(LINON_PRECISE) || !defined(__CUDA_ARCH__)
  return dot(a, b) + s;
#else
  float r = fmaf(a.x, b.x, s);
  for (int i = 1; i < N; ++i) r = fmaf(a[i], b[i], r);
  return r;
#endif
}
// integer dot products wrap like WGSL's i32 / u32 arithmetic (summed in u32)
template <int N> WG_HD int dot(const vec<int, N>& a, const vec<int, N>& b) {
  unsigned r = 0u;
  for (int i = 0; i < N; ++i) r += unsigned(a[i]) * unsigned(b[i]);
  return int(r);
}
template <int N> WG_HD unsigned dot(const vec<unsigned, N>& a, const vec<unsigned, N>& b) {
  unsigned r = 0u;
  for (int i = 0; i < N; ++i) r += a[i] * b[i];
  return r;
}
WG_HD vec3f cross(const vec3f& a, const vec3f& b) {
  return vec3f(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
WG_HD float length(float x) { return fabsf(x); }
template <int N> WG_HD float length(const vec<float, N>& v) { return sqrtf(dot(v, v)); }
template <int N> WG_HD float distance(const vec<float, N>& a, const vec<float, N>& b) {
  return length(a - b);
}
WG_HD float distance(float a, float b) { return fabsf(a - b); }
// ---------------------------------------------------------------------------
// Fused float3 operations for the march (c + s * a and friends).  Fast
// modules on sm_100 and later issue the x and y components as one packed
// FP32 pair operation (f32x2: two results per issued instruction, each
// rounded exactly like the scalar operation) and z as a scalar one; the
// march is issue-bound, so this removes issue slots without changing any
// rounding.  Precise modules and the host evaluate the shader's separate
// multiply and add.  LINON_NO_F32X2 turns the packing off.
// ---------------------------------------------------------------------------
#if defined(__CUDA_ARCH__) && !defined(LINON_PRECISE) && !defined(LINON_NO_F32X2)
#if __CUDA_ARCH__ >= 1000
#define LINON_F32X2 1
#endif
#endif
#ifdef LINON_F32X2
WG_HD float2 xy2(const vec3f& a) { return make_float2(a.x, a.y); }
#endif
// c + s * a
WG_HD vec3f vmadd(const vec3f& a, float s, const vec3f& c) {
#ifdef LINON_F32X2
  const float2 r = __ffma2_rn(xy2(a), make_float2(s, s), xy2(c));
  return vec3f(r.x, r.y, fmaf(a.z, s, c.z));
#else
  return c + s * a;
#endif
}
// a * s
WG_HD vec3f vscale(const vec3f& a, float s) {
#ifdef LINON_F32X2
  const float2 r = __fmul2_rn(xy2(a), make_float2(s, s));
  return vec3f(r.x, r.y, a.z * s);
#else
  return a * s;
#endif
}
// a + b
WG_HD vec3f vadd(const vec3f& a, const vec3f& b) {
#ifdef LINON_F32X2
  const float2 r = __fadd2_rn(xy2(a), xy2(b));
  return vec3f(r.x, r.y, a.z + b.z);
#else
  return a + b;
#endif
}
// a - b, as a + (-b): there is no packed-subtract builtin, and the
// negation is an operand modifier of the packed add (exact, so the result
// rounds like the subtraction)
WG_HD vec3f vsub(const vec3f& a, const vec3f& b) {
#ifdef LINON_F32X2
  const float2 r = __fadd2_rn(xy2(a), make_float2(-b.x, -b.y));
  return vec3f(r.x, r.y, a.z - b.z);
#else
  return a - b;
#endif
}

template <int N> WG_HD vec<float, N> normalize(const vec<float, N>& v) {
#if defined(LINON_PRECISE) || !defined(__CUDA_ARCH__)
  float l = sqrtf(dot(v, v));
  return v / l;
#else
  return v * rsqrt_ftz(dot(v, v));
#endif
}
// LINON_PACKED_NORMALIZE: fast float3 normalize scales x/y as one packed
// pair (the scale factor has to be paired first; whether that pays depends
// on the kernel's register allocation, so the module that includes this
// file decides).
#if defined(LINON_F32X2) && defined(LINON_PACKED_NORMALIZE)
template <> WG_HD vec3f normalize<3>(const vec3f& v) { return vscale(v, rsqrt_ftz(dot(v, v))); }
#endif
// reflect(e1, e2) = e1 - 2 * dot(e2, e1) * e2
template <int N> WG_HD vec<float, N> reflect(const vec<float, N>& e1, const vec<float, N>& e2) {
  float d = 2.0f * dot(e2, e1);
  return e1 - d * e2;
}
template <int N>
WG_HD vec<float, N> refract(const vec<float, N>& e1, const vec<float, N>& e2, float e3) {
  float d = dot(e2, e1);
  float k = 1.0f - e3 * e3 * (1.0f - d * d);
  if (k < 0.0f) return vec<float, N>(0.0f);
  return e3 * e1 - (e3 * d + sqrtf(k)) * e2;
}
template <int N>
WG_HD vec<float, N> faceForward(const vec<float, N>& e1, const vec<float, N>& e2,
                                const vec<float, N>& e3) {
  return dot(e2, e3) < 0.0f ? e1 : -e1;
}
// select(f, t, cond)
template <class T> WG_HD T select(const T& f, const T& t, bool c) { return c ? t : f; }
template <class T, int N>
WG_HD vec<T, N> select(const vec<T, N>& f, const vec<T, N>& t, const vec<bool, N>& c) {
  vec<T, N> r;
  for (int i = 0; i < N; ++i) r[i] = c[i] ? t[i] : f[i];
  return r;
}
WG_HD bool all(bool b) { return b; }
WG_HD bool any(bool b) { return b; }
template <int N> WG_HD bool all(const vec<bool, N>& v) {
  bool r = true;
  for (int i = 0; i < N; ++i) r = r && v[i];
  return r;
}
template <int N> WG_HD bool any(const vec<bool, N>& v) {
  bool r = false;
  for (int i = 0; i < N; ++i) r = r || v[i];
  return r;
}

// ---------------------------------------------------------------------------
// integer bit builtins (WGSL 17.5: countLeadingZeros ... reverseBits,
// extractBits, insertBits), component-wise on i32 / u32
// ---------------------------------------------------------------------------
WG_HD unsigned clz32_(unsigned x) {
#if defined(__CUDA_ARCH__)
  return unsigned(__clz(int(x)));
#else
  return x ? unsigned(__builtin_clz(x)) : 32u;
#endif
}
WG_HD unsigned ctz32_(unsigned x) {
#if defined(__CUDA_ARCH__)
  return x ? unsigned(__ffs(int(x)) - 1) : 32u;
#else
  return x ? unsigned(__builtin_ctz(x)) : 32u;
#endif
}
WG_HD unsigned popc32_(unsigned x) {
#if defined(__CUDA_ARCH__)
  return unsigned(__popc(x));
#else
  return unsigned(__builtin_popcount(x));
#endif
}
WG_HD unsigned brev32_(unsigned x) {
#if defined(__CUDA_ARCH__)
  return __brev(x);
#else
  unsigned r = 0;
  for (int i = 0; i < 32; ++i) r |= ((x >> i) & 1u) << (31 - i);
  return r;
#endif
}
WG_HD unsigned countLeadingZeros(unsigned x) { return clz32_(x); }
WG_HD int countLeadingZeros(int x) { return int(clz32_(unsigned(x))); }
WG_HD unsigned countTrailingZeros(unsigned x) { return ctz32_(x); }
WG_HD int countTrailingZeros(int x) { return int(ctz32_(unsigned(x))); }
WG_HD unsigned countOneBits(unsigned x) { return popc32_(x); }
WG_HD int countOneBits(int x) { return int(popc32_(unsigned(x))); }
WG_HD unsigned reverseBits(unsigned x) { return brev32_(x); }
WG_HD int reverseBits(int x) { return int(brev32_(unsigned(x))); }
// position of the most significant 1 bit (u32), or of the most significant
// bit that differs from the sign bit (i32); all ones (-1) when there is none
WG_HD unsigned firstLeadingBit(unsigned x) { return x ? 31u - clz32_(x) : 0xffffffffu; }
WG_HD int firstLeadingBit(int x) {
  const unsigned v = x < 0 ? ~unsigned(x) : unsigned(x);
  return v ? int(31u - clz32_(v)) : -1;
}
WG_HD unsigned firstTrailingBit(unsigned x) { return x ? ctz32_(x) : 0xffffffffu; }
WG_HD int firstTrailingBit(int x) { return x ? int(ctz32_(unsigned(x))) : -1; }
// bits [o, o + c) with o = min(offset, 32), c = min(count, 32 - o); zero-
// (u32) or sign-extended (i32); 0 when c = 0
WG_HD unsigned extractBits(unsigned e, unsigned offset, unsigned count) {
  const unsigned o = offset < 32u ? offset : 32u, c = count < 32u - o ? count : 32u - o;
  if (c == 0u) return 0u;
  return (e >> o) & (c == 32u ? 0xffffffffu : ((1u << c) - 1u));
}
WG_HD int extractBits(int e, unsigned offset, unsigned count) {
  const unsigned o = offset < 32u ? offset : 32u, c = count < 32u - o ? count : 32u - o;
  if (c == 0u) return 0;
  return int(unsigned(e) << (32u - o - c)) >> (32u - c);
}
// e with bits [o, o + c) replaced by the low c bits of newbits
WG_HD unsigned insertBits(unsigned e, unsigned newbits, unsigned offset, unsigned count) {
  const unsigned o = offset < 32u ? offset : 32u, c = count < 32u - o ? count : 32u - o;
  if (c == 0u) return e;
  const unsigned mask = (c == 32u ? 0xffffffffu : ((1u << c) - 1u)) << o;
  return (e & ~mask) | ((newbits << o) & mask);
}
WG_HD int insertBits(int e, int newbits, unsigned offset, unsigned count) {
  return int(insertBits(unsigned(e), unsigned(newbits), offset, count));
}
#define WG_BITS1(F)                                                                 \
  template <class T, int N> WG_HD vec<T, N> F(const vec<T, N>& v) {                \
    vec<T, N> r;                                                                    \
    for (int i = 0; i < N; ++i) r[i] = F(v[i]);                                     \
    return r;                                                                       \
  }
WG_BITS1(countLeadingZeros)
WG_BITS1(countTrailingZeros)
WG_BITS1(countOneBits)
WG_BITS1(reverseBits)
WG_BITS1(firstLeadingBit)
WG_BITS1(firstTrailingBit)
#undef WG_BITS1
template <class T, int N> WG_HD vec<T, N> extractBits(const vec<T, N>& v, unsigned o, unsigned c) {
  vec<T, N> r;
  for (int i = 0; i < N; ++i) r[i] = extractBits(v[i], o, c);
  return r;
}
template <class T, int N>
WG_HD vec<T, N> insertBits(const vec<T, N>& v, const vec<T, N>& nb, unsigned o, unsigned c) {
  vec<T, N> r;
  for (int i = 0; i < N; ++i) r[i] = insertBits(v[i], nb[i], o, c);
  return r;
}

// ---------------------------------------------------------------------------
// float decomposition: ldexp, frexp, modf (result structs with the WGSL
// member names), quantizeToF16
// ---------------------------------------------------------------------------
template <class F, class I> struct frexp_result {
  F m_fract;
  I m_exp;
};
template <class F> struct modf_result {
  F m_fract;
  F m_whole;
};
WG_HD float ldexp(float x, int e) { return ldexpf(x, e); }
template <int N> WG_HD vec<float, N> ldexp(const vec<float, N>& x, const vec<int, N>& e) {
  vec<float, N> r;
  for (int i = 0; i < N; ++i) r[i] = ldexpf(x[i], e[i]);
  return r;
}
WG_HD frexp_result<float, int> frexp(float x) {
  frexp_result<float, int> r;
  r.m_fract = frexpf(x, &r.m_exp);
  return r;
}
template <int N> WG_HD frexp_result<vec<float, N>, vec<int, N>> frexp(const vec<float, N>& x) {
  frexp_result<vec<float, N>, vec<int, N>> r;
  for (int i = 0; i < N; ++i) r.m_fract[i] = frexpf(x[i], &r.m_exp[i]);
  return r;
}
WG_HD modf_result<float> modf(float x) {
  modf_result<float> r;
  r.m_fract = modff(x, &r.m_whole);
  return r;
}
template <int N> WG_HD modf_result<vec<float, N>> modf(const vec<float, N>& x) {
  modf_result<vec<float, N>> r;
  for (int i = 0; i < N; ++i) r.m_fract[i] = modff(x[i], &r.m_whole[i]);
  return r;
}
// IEEE binary16 bits of x, rounded to nearest even (overflow to infinity;
// NaN to a quiet NaN)
WG_HD unsigned f32_to_f16_bits(float x) {
  const unsigned u = bitcast_<unsigned>(x);
  const unsigned sign = (u >> 16) & 0x8000u;
  const unsigned a = u & 0x7fffffffu;
  if (a >= 0x7f800000u) return sign | (a > 0x7f800000u ? 0x7e00u : 0x7c00u);
  if (a >= 0x477ff000u) return sign | 0x7c00u;  // >= 65520 rounds to infinity
  if (a < 0x38800000u) {
    // below 2^-14: a binary16 subnormal, the value in units of 2^-24
    if (a < 0x33000000u) return sign;  // below 2^-25 (half the least subnormal)
    const unsigned m = (a & 0x007fffffu) | 0x00800000u;  // 24-bit significand
    const unsigned shift = 126u - (a >> 23);             // to units of 2^-24
    const unsigned q = m >> shift, rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1u);
    return sign | (q + ((rem > half || (rem == half && (q & 1u))) ? 1u : 0u));
  }
  // normal: rebias the exponent (127 -> 15) and round 23 -> 10 bits
  const unsigned q = (a - 0x38000000u) >> 13, rem = a & 0x1fffu;
  return sign | (q + ((rem > 0x1000u || (rem == 0x1000u && (q & 1u))) ? 1u : 0u));
}
WG_HD float f16_bits_to_f32(unsigned h) {
  const unsigned sign = (h & 0x8000u) << 16, e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
  if (e == 0x1fu) return bitcast_<float>(sign | 0x7f800000u | (m << 13));
  if (e == 0u) {
    const float v = float(m) * 5.9604644775390625e-8f;  // m * 2^-24, exact
    return sign ? -v : v;
  }
  return bitcast_<float>(sign | ((e + 112u) << 23) | (m << 13));
}
WG_HD float quantizeToF16(float x) { return f16_bits_to_f32(f32_to_f16_bits(x)); }
template <int N> WG_HD vec<float, N> quantizeToF16(const vec<float, N>& v) {
  vec<float, N> r;
  for (int i = 0; i < N; ++i) r[i] = quantizeToF16(v[i]);
  return r;
}

// ---------------------------------------------------------------------------
// data packing builtins (WGSL 17.9 / 17.10) and packed 8-bit dot products
// ---------------------------------------------------------------------------
WG_HD unsigned pack_snorm_(float x, float s, unsigned mask) {
  const float c = fminf(1.0f, fmaxf(-1.0f, x));
  return unsigned(int(floorf(0.5f + s * c))) & mask;
}
WG_HD unsigned pack_unorm_(float x, float s) {
  return unsigned(floorf(0.5f + s * fminf(1.0f, fmaxf(0.0f, x))));
}
WG_HD unsigned pack4x8snorm(const vec4f& e) {
  unsigned r = 0;
  for (int i = 0; i < 4; ++i) r |= pack_snorm_(e[i], 127.0f, 0xffu) << (8 * i);
  return r;
}
WG_HD unsigned pack4x8unorm(const vec4f& e) {
  unsigned r = 0;
  for (int i = 0; i < 4; ++i) r |= pack_unorm_(e[i], 255.0f) << (8 * i);
  return r;
}
WG_HD unsigned pack2x16snorm(const vec2f& e) {
  return pack_snorm_(e.x, 32767.0f, 0xffffu) | (pack_snorm_(e.y, 32767.0f, 0xffffu) << 16);
}
WG_HD unsigned pack2x16unorm(const vec2f& e) {
  return pack_unorm_(e.x, 65535.0f) | (pack_unorm_(e.y, 65535.0f) << 16);
}
WG_HD unsigned pack2x16float(const vec2f& e) { return f32_to_f16_bits(e.x) | (f32_to_f16_bits(e.y) << 16); }
WG_HD vec4f unpack4x8snorm(unsigned e) {
  vec4f r;
  for (int i = 0; i < 4; ++i) r[i] = fmaxf(float(int(e << (24 - 8 * i)) >> 24) / 127.0f, -1.0f);
  return r;
}
WG_HD vec4f unpack4x8unorm(unsigned e) {
  vec4f r;
  for (int i = 0; i < 4; ++i) r[i] = float((e >> (8 * i)) & 0xffu) / 255.0f;
  return r;
}
WG_HD vec2f unpack2x16snorm(unsigned e) {
  return vec2f(fmaxf(float(int(e << 16) >> 16) / 32767.0f, -1.0f), fmaxf(float(int(e) >> 16) / 32767.0f, -1.0f));
}
WG_HD vec2f unpack2x16unorm(unsigned e) {
  return vec2f(float(e & 0xffffu) / 65535.0f, float(e >> 16) / 65535.0f);
}
WG_HD vec2f unpack2x16float(unsigned e) { return vec2f(f16_bits_to_f32(e & 0xffffu), f16_bits_to_f32(e >> 16)); }
WG_HD unsigned pack4xI8(const vec4i& e) {
  unsigned r = 0;
  for (int i = 0; i < 4; ++i) r |= (unsigned(e[i]) & 0xffu) << (8 * i);
  return r;
}
WG_HD unsigned pack4xU8(const vec4u& e) {
  unsigned r = 0;
  for (int i = 0; i < 4; ++i) r |= (e[i] & 0xffu) << (8 * i);
  return r;
}
WG_HD unsigned pack4xI8Clamp(const vec4i& e) {
  unsigned r = 0;
  for (int i = 0; i < 4; ++i) r |= (unsigned(imin_(127, imax_(-128, e[i]))) & 0xffu) << (8 * i);
  return r;
}
WG_HD unsigned pack4xU8Clamp(const vec4u& e) {
  unsigned r = 0;
  for (int i = 0; i < 4; ++i) r |= umin_(255u, e[i]) << (8 * i);
  return r;
}
WG_HD vec4i unpack4xI8(unsigned e) {
  vec4i r;
  for (int i = 0; i < 4; ++i) r[i] = int(e << (24 - 8 * i)) >> 24;
  return r;
}
WG_HD vec4u unpack4xU8(unsigned e) {
  vec4u r;
  for (int i = 0; i < 4; ++i) r[i] = (e >> (8 * i)) & 0xffu;
  return r;
}
WG_HD unsigned dot4U8Packed(unsigned a, unsigned b) {
  unsigned r = 0;
  for (int i = 0; i < 4; ++i) r += ((a >> (8 * i)) & 0xffu) * ((b >> (8 * i)) & 0xffu);
  return r;
}
WG_HD int dot4I8Packed(unsigned a, unsigned b) {
  int r = 0;
  for (int i = 0; i < 4; ++i) r += (int(a << (24 - 8 * i)) >> 24) * (int(b << (24 - 8 * i)) >> 24);
  return r;
}

// ---------------------------------------------------------------------------
// linon helper functions, src/main_view.wgsl:76-146
// ---------------------------------------------------------------------------
#define LINON_PI 3.14159265358979323846f

// The rotations are the shader's matrix products.  Precise modules (and the
// host build) multiply out the full matrix, zero entries included; fast
// modules drop the products with the structural zeros and ones, which
// changes the result only for non-finite components (0 * inf).
#if defined(LINON_PRECISE) || !defined(__CUDA_ARCH__)
#define LINON_FULL_ROTATIONS 1
#endif
WG_HD vec3f rotateX(const vec3f& v, float phi) {  // main_view.wgsl:78-84
  float s, c;
  sincos_(phi, &s, &c);
#ifdef LINON_FULL_ROTATIONS
  return make_mat(vec3f(1.0f, 0.0f, 0.0f), vec3f(0.0f, c, s), vec3f(0.0f, -s, c)) * v;
#else
  return vec3f(v.x, c * v.y - s * v.z, s * v.y + c * v.z);
#endif
}
WG_HD vec3f rotateY(const vec3f& v, float phi) {  // main_view.wgsl:86-92
  float s, c;
  sincos_(phi, &s, &c);
#ifdef LINON_FULL_ROTATIONS
  return make_mat(vec3f(c, 0.0f, -s), vec3f(0.0f, 1.0f, 0.0f), vec3f(s, 0.0f, c)) * v;
#else
  return vec3f(c * v.x + s * v.z, v.y, c * v.z - s * v.x);
#endif
}
WG_HD vec3f rotateZ(const vec3f& v, float phi) {  // main_view.wgsl:94-100: third column zero
  float s, c;
  sincos_(phi, &s, &c);
#ifdef LINON_FULL_ROTATIONS
  return make_mat(vec3f(c, s, 0.0f), vec3f(-s, c, 0.0f), vec3f(0.0f, 0.0f, 0.0f)) * v;
#else
  return vec3f(c * v.x - s * v.y, s * v.x + c * v.y, 0.0f);
#endif
}
WG_HD vec3f translate(const vec3f& v, float dx, float dy, float dz) {  // main_view.wgsl:102-108
  return vec3f(v.x + dx, v.y + dy, v.z + dz);
}
WG_HD float refraction_index(float t) {  // main_view.wgsl:111-117 (Y. Zhao et al.)
  const float air_pressure = 101325.0f;
  const float c1 = 0.0000104f;
  const float c2 = 0.00366f;
  return c1 * air_pressure * (1.0f + air_pressure * (60.1f - 0.972f * t) * 1e-10f) /
         (1.0f + c2 * t);
}
WG_HD vec3f refraction(float t_in, float t_out, const vec3f& v_in, const vec3f& n) {
  // main_view.wgsl:119-136; clamp(-1.0, 1.0, x) == min(1, x)
  float eta_in = refraction_index(t_in);
  float eta_out = refraction_index(t_out);
  float cosi = clamp(-1.0f, 1.0f, dot(v_in, n));
  vec3f n_ref = n;
  if (cosi < 0.0f) {
    cosi = -cosi;
  } else {
    n_ref = -n;
  }
  float eta = eta_in / eta_out;
  float k = 1.0f - eta * eta * (1.0f - cosi * cosi);
  if (k < 0.0f) return reflect(v_in, n_ref);
  return eta * v_in + (eta * cosi - sqrtf(k)) * n_ref;
}
WG_HD float point_plane_distance(const vec3f& p, const vec3f& n, const vec3f& p0) {
  float d = dot(p0, n);  // main_view.wgsl:138-142
  return fabsf(dot(p, n) - d);
}
WG_HD float sigmoid(float x) { return 1.0f / (1.0f + expf(-x)); }  // main_view.wgsl:144-146

// ---------------------------------------------------------------------------
// Two rays per thread (fast modules that define LINON_PAIRS, sm_100 and
// later).  An f2 is one f32 value of two rays (x: the first, y: the
// second); the front end's pair emission writes a field function over f2,
// and every operation runs lane-wise as one packed FP32 pair instruction
// (f32x2, each lane rounded like the scalar operation) or as two scalar
// ones where there is no packed form (division, square roots, the special
// functions).  a * b is kept unevaluated until it meets + or -, which then
// issue one packed FMA, as the compiler contracts the scalar code.  There is
// deliberately no comparison, no conversion to an integer and no conversion
// back to float: a field that needs one fails to compile in pair form and
// runs one ray per thread.
// ---------------------------------------------------------------------------
#if defined(LINON_PAIRS) && defined(LINON_F32X2)
struct f2 {
  float2 v;
  WG_HD f2() : v(make_float2(0.0f, 0.0f)) {}
  WG_HD f2(float s) : v(make_float2(s, s)) {}
  WG_HD f2(float a, float b) : v(make_float2(a, b)) {}
  WG_HD explicit f2(float2 p) : v(p) {}
};
WG_HD f2 neg(f2 a) { return f2(make_float2(-a.v.x, -a.v.y)); }
WG_HD f2 fma2(f2 a, f2 b, f2 c) { return f2(__ffma2_rn(a.v, b.v, c.v)); }
WG_HD f2 mul2(f2 a, f2 b) { return f2(__fmul2_rn(a.v, b.v)); }
struct f2m {  // a * b, not yet rounded
  f2 a, b;
  WG_HD operator f2() const { return mul2(a, b); }
};
WG_HD f2m operator*(f2 a, f2 b) { return f2m{a, b}; }
WG_HD f2 operator+(f2 a, f2 b) { return f2(__fadd2_rn(a.v, b.v)); }
WG_HD f2 operator-(f2 a, f2 b) { return f2(__fadd2_rn(a.v, neg(b).v)); }
WG_HD f2 operator+(f2m m, f2 c) { return fma2(m.a, m.b, c); }
WG_HD f2 operator+(f2 c, f2m m) { return fma2(m.a, m.b, c); }
WG_HD f2 operator-(f2m m, f2 c) { return fma2(m.a, m.b, neg(c)); }
WG_HD f2 operator-(f2 c, f2m m) { return fma2(neg(m.a), m.b, c); }
WG_HD f2 operator+(f2m m, f2m n) { return fma2(m.a, m.b, f2(n)); }
WG_HD f2 operator-(f2m m, f2m n) { return fma2(m.a, m.b, neg(f2(n))); }
WG_HD f2 operator-(f2 a) { return neg(a); }
WG_HD f2 operator-(f2m m) { return mul2(neg(m.a), m.b); }
WG_HD f2 operator/(f2 a, f2 b) { return f2(a.v.x / b.v.x, a.v.y / b.v.y); }
WG_HD f2& operator+=(f2& a, f2 b) { a = a + b; return a; }
WG_HD f2& operator-=(f2& a, f2 b) { a = a - b; return a; }
WG_HD f2& operator*=(f2& a, f2 b) { a = mul2(a, b); return a; }
WG_HD f2& operator/=(f2& a, f2 b) { a = a / b; return a; }
#define WG_F2_LANES(NAME, EXPR)                                                    \
  WG_HD f2 NAME(f2 a) {                                                            \
    const float x0 = a.v.x, x1 = a.v.y;                                            \
    float r0, r1;                                                                  \
    { const float x = x0; r0 = (EXPR); }                                           \
    { const float x = x1; r1 = (EXPR); }                                           \
    return f2(r0, r1);                                                             \
  }
WG_F2_LANES(sqrt, sqrtf(x))
WG_F2_LANES(inverseSqrt, rsqrt_ftz(x))
WG_F2_LANES(rsqrt_ftz2, rsqrt_ftz(x))
WG_F2_LANES(abs, fabsf(x))
WG_F2_LANES(exp, expf(x))
WG_F2_LANES(sin, sin_(x))
WG_F2_LANES(cos, cos_(x))
WG_F2_LANES(floor, floorf(x))
WG_F2_LANES(length, fabsf(x))
WG_F2_LANES(tan, tanf(x))
WG_F2_LANES(log, logf(x))
WG_F2_LANES(log2, log2f(x))
WG_F2_LANES(exp2, exp2f(x))
WG_F2_LANES(fract, x - floorf(x))
WG_F2_LANES(sign, (x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f)))
#undef WG_F2_LANES
WG_HD f2 atan2(f2 a, f2 b) { return f2(atan2f(a.v.x, b.v.x), atan2f(a.v.y, b.v.y)); }
WG_HD f2 step(f2 e, f2 x) { return f2(x.v.x >= e.v.x ? 1.0f : 0.0f, x.v.y >= e.v.y ? 1.0f : 0.0f); }
// the vector forms, component by component (as the one-ray vec<float, N>
// forms); the three-component one is not a template, so that an unevaluated
// product (vs2, below) converts to it
#define WG_F2_VEC(NAME)                                                            \
  template <int N> WG_HD vec<f2, N> NAME(const vec<f2, N>& v) {                    \
    vec<f2, N> r;                                                                  \
    for (int i = 0; i < N; ++i) r[i] = NAME(v[i]);                                 \
    return r;                                                                      \
  }                                                                                \
  WG_HD vec<f2, 3> NAME(const vec<f2, 3>& v) { return NAME<3>(v); }
WG_F2_VEC(sqrt)
WG_F2_VEC(inverseSqrt)
WG_F2_VEC(exp)
WG_F2_VEC(sin)
WG_F2_VEC(cos)
WG_F2_VEC(floor)
WG_F2_VEC(tan)
WG_F2_VEC(log)
WG_F2_VEC(log2)
WG_F2_VEC(exp2)
WG_F2_VEC(fract)
WG_F2_VEC(sign)
#undef WG_F2_VEC
WG_HD f2 min(f2 a, f2 b) { return f2(fminf(a.v.x, b.v.x), fminf(a.v.y, b.v.y)); }
WG_HD f2 max(f2 a, f2 b) { return f2(fmaxf(a.v.x, b.v.x), fmaxf(a.v.y, b.v.y)); }
WG_HD f2 clamp(f2 e, f2 lo, f2 hi) { return min(max(e, lo), hi); }
WG_HD f2 sigmoid(f2 x) { return f2(1.0f) / (f2(1.0f) + exp(neg(x))); }
WG_HD void sincos2(f2 x, f2* s, f2* c) {
#if !defined(LINON_PRECISE) && !defined(LINON_SINCOS_POLY) && defined(__CUDA_ARCH__)
  // sincos_fast's reduction by 2 pi with the multiply and the two FMAs
  // packed (each lane rounds as the one-ray code does; fma(k, -P, x) is
  // fma(-k, P, x)), then the special-function unit lane by lane
  const f2 y = mul2(x, f2(0x1.45f306p-3f));
  const f2 k(rintf(y.v.x), rintf(y.v.y));
  f2 r = fma2(k, f2(-0x1.921fb6p+2f), x);
  r = fma2(k, f2(0x1.777a5cp-23f), r);
  *s = f2(__sinf(r.v.x), __sinf(r.v.y));
  *c = f2(__cosf(r.v.x), __cosf(r.v.y));
#else
  float s0, c0, s1, c1;
  sincos_(x.v.x, &s0, &c0);
  sincos_(x.v.y, &s1, &c1);
  *s = f2(s0, s1);
  *c = f2(c0, c1);
#endif
}

typedef vec<f2, 3> vec3p;
// s * v (or v * s), not yet rounded: + or - with a vector issues packed FMAs
struct vs2 {
  vec3p v;
  f2 s;
  WG_HD operator vec3p() const { return vec3p(mul2(v.x, s), mul2(v.y, s), mul2(v.z, s)); }
};
WG_HD vs2 operator*(const vec3p& v, f2 s) { return vs2{v, s}; }
WG_HD vs2 operator*(f2 s, const vec3p& v) { return vs2{v, s}; }
WG_HD vs2 operator*(const vec3p& v, float s) { return vs2{v, f2(s)}; }
WG_HD vs2 operator*(float s, const vec3p& v) { return vs2{v, f2(s)}; }
WG_HD vs2 operator*(const vec3p& v, f2m s) { return vs2{v, f2(s)}; }
WG_HD vs2 operator*(f2m s, const vec3p& v) { return vs2{v, f2(s)}; }
WG_HD vec3p operator+(const vec3p& a, const vs2& m) {
  return vec3p(fma2(m.v.x, m.s, a.x), fma2(m.v.y, m.s, a.y), fma2(m.v.z, m.s, a.z));
}
WG_HD vec3p operator+(const vs2& m, const vec3p& a) { return a + m; }
WG_HD vec3p operator-(const vec3p& a, const vs2& m) {
  const f2 ns = neg(m.s);
  return vec3p(fma2(m.v.x, ns, a.x), fma2(m.v.y, ns, a.y), fma2(m.v.z, ns, a.z));
}
WG_HD vec3p operator-(const vs2& m, const vec3p& a) {
  return vec3p(fma2(m.v.x, m.s, neg(a.x)), fma2(m.v.y, m.s, neg(a.y)), fma2(m.v.z, m.s, neg(a.z)));
}
WG_HD vec3p operator+(const vs2& m, const vs2& n) { return vec3p(m) + n; }
WG_HD vec3p operator-(const vs2& m, const vs2& n) { return vec3p(m) - n; }
WG_HD vec3p operator-(const vs2& m) { return vec3p(m.v.x * neg(m.s), m.v.y * neg(m.s), m.v.z * neg(m.s)); }
// every other operation on an unevaluated product rounds the product first,
// as the one-ray code rounds s * v before using it
WG_HD vec3p operator*(const vs2& m, const vec3p& a) { return vec3p(m) * a; }
WG_HD vec3p operator*(const vec3p& a, const vs2& m) { return a * vec3p(m); }
WG_HD vec3p operator*(const vs2& m, const vs2& n) { return vec3p(m) * vec3p(n); }
WG_HD vs2 operator*(const vs2& m, f2 s) { return vec3p(m) * s; }
WG_HD vs2 operator*(f2 s, const vs2& m) { return s * vec3p(m); }
WG_HD vs2 operator*(const vs2& m, float s) { return vec3p(m) * s; }
WG_HD vs2 operator*(float s, const vs2& m) { return s * vec3p(m); }
WG_HD vec3p operator/(const vs2& m, const vec3p& a) { return vec3p(m) / a; }
WG_HD vec3p operator/(const vec3p& a, const vs2& m) { return a / vec3p(m); }
WG_HD vec3p operator/(const vec3p& v, f2 s) { return v * (f2(1.0f) / s); }
WG_HD vec3p operator/(const vec3p& v, float s) { return v * f2(1.0f / s); }
WG_HD vec3p operator+(const vec3p& v, float s) { return v + vec3p(f2(s)); }
WG_HD vec3p operator-(const vec3p& v, float s) { return v - vec3p(f2(s)); }

WG_HD f2 dot(const vec3p& a, const vec3p& b) { return fma2(a.z, b.z, fma2(a.y, b.y, mul2(a.x, b.x))); }
WG_HD f2 dot_add(const vec3p& a, const vec3p& b, f2 s) {
  return fma2(a.z, b.z, fma2(a.y, b.y, fma2(a.x, b.x, s)));
}
WG_HD f2 length(const vec3p& v) { return sqrt(dot(v, v)); }
WG_HD vec3p normalize(const vec3p& v) { return vec3p(v * rsqrt_ftz2(dot(v, v))); }
// component-wise abs / min / max / clamp of three-component values, not
// templates, so that an unevaluated product (vs2) converts to them
WG_HD vec3p abs(const vec3p& v) { return vec3p(abs(v.x), abs(v.y), abs(v.z)); }
WG_HD vec3p min(const vec3p& a, const vec3p& b) { return vec3p(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
WG_HD vec3p max(const vec3p& a, const vec3p& b) { return vec3p(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
WG_HD vec3p clamp(const vec3p& e, const vec3p& lo, const vec3p& hi) { return min(max(e, lo), hi); }
WG_HD vec3p atan2(const vec3p& a, const vec3p& b) { return vec3p(atan2(a.x, b.x), atan2(a.y, b.y), atan2(a.z, b.z)); }
WG_HD vec3p step(const vec3p& e, const vec3p& x) { return vec3p(step(e.x, x.x), step(e.y, x.y), step(e.z, x.z)); }
// mix, smoothstep, distance and reflect with the one-ray runtime's formulas
WG_HD f2 mix(f2 a, f2 b, f2 t) { return fma2(b, t, mul2(a, f2(1.0f) - t)); }
WG_HD vec3p mix(const vec3p& a, const vec3p& b, f2 t) { return vec3p(a * (f2(1.0f) - t)) + b * t; }
WG_HD vec3p mix(const vec3p& a, const vec3p& b, const vec3p& t) {
  return vec3p(mix(a.x, b.x, t.x), mix(a.y, b.y, t.y), mix(a.z, b.z, t.z));
}
WG_HD f2 smoothstep(f2 lo, f2 hi, f2 x) {
  const f2 t = clamp((x - lo) / (hi - lo), f2(0.0f), f2(1.0f));
  return mul2(mul2(t, t), fma2(f2(-2.0f), t, f2(3.0f)));  // 3 - 2 t contracted, as in the one-ray code
}
WG_HD vec3p smoothstep(const vec3p& lo, const vec3p& hi, const vec3p& x) {
  return vec3p(smoothstep(lo.x, hi.x, x.x), smoothstep(lo.y, hi.y, x.y), smoothstep(lo.z, hi.z, x.z));
}
WG_HD f2 distance(const vec3p& a, const vec3p& b) { return length(a - b); }
WG_HD f2 distance(f2 a, f2 b) { return abs(a - b); }
WG_HD vec3p reflect(const vec3p& e1, const vec3p& e2) {
  const f2 d = mul2(f2(2.0f), dot(e2, e1));
  return e1 - e2 * d;
}
WG_HD vec3p cross(const vec3p& a, const vec3p& b) {
  return vec3p(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
WG_HD f2 pow_k(f2 x, float k) {
  if (k == 1.0f) return x;
  if (k == 2.0f) return mul2(x, x);
  if (k == 3.0f) return mul2(mul2(x, x), x);
  if (k == 4.0f) { const f2 y = mul2(x, x); return mul2(y, y); }
  if (k == 0.5f) return sqrt(x);
  if (k == 1.5f) return mul2(x, sqrt(x));
  if (k == -0.5f) return rsqrt_ftz2(x);
  if (k == -1.0f) return f2(1.0f) / x;
  if (k == -1.5f) { const f2 r = rsqrt_ftz2(x); return mul2(mul2(r, r), r); }
  if (k == -2.0f) { const f2 r = f2(1.0f) / x; return mul2(r, r); }
  if (k == -3.0f) { const f2 r = f2(1.0f) / x; return mul2(mul2(r, r), r); }
  return f2(powf(x.v.x, k), powf(x.v.y, k));
}
WG_HD f2 scaled_pow_neg_k(f2 s, f2 x, float k) {
  if (k == 1.5f) {
    const f2 r = rsqrt_ftz2(x);
    return mul2(mul2(s, r), mul2(r, r));
  }
  return mul2(s, pow_k(x, -k));
}
WG_HD vs2 div_pow_k_sv(f2 s, const vec3p& v, f2 x, float k) { return vs2{v, scaled_pow_neg_k(s, x, k)}; }
WG_HD vs2 div_pow_k_vs(const vec3p& v, f2 s, f2 x, float k) { return vs2{v, scaled_pow_neg_k(s, x, k)}; }
WG_HD vs2 div_pow_k(const vec3p& a, f2 x, float k) { return vs2{a, pow_k(x, -k)}; }
WG_HD f2 div_pow_k(f2 a, f2 x, float k) { return mul2(a, pow_k(x, -k)); }
// the linon helpers (main_view.wgsl:78-108), lane-wise, structural zeros
// left out as in the one-ray fast modules
WG_HD vec3p rotateX(const vec3p& v, f2 phi) {
  f2 s, c;
  sincos2(phi, &s, &c);
  return vec3p(v.x, c * v.y - s * v.z, s * v.y + c * v.z);
}
WG_HD vec3p rotateY(const vec3p& v, f2 phi) {
  f2 s, c;
  sincos2(phi, &s, &c);
  return vec3p(c * v.x + s * v.z, v.y, c * v.z - s * v.x);
}
WG_HD vec3p rotateZ(const vec3p& v, f2 phi) {
  f2 s, c;
  sincos2(phi, &s, &c);
  return vec3p(c * v.x - s * v.y, s * v.x + c * v.y, f2(0.0f));
}
WG_HD vec3p translate(const vec3p& v, f2 dx, f2 dy, f2 dz) { return vec3p(v.x + dx, v.y + dy, v.z + dz); }
#endif  // LINON_PAIRS

}  // namespace wgsl
