// Vector types and builtins for WGSL translated to C++ by wgsl_transpile.py
// (test infrastructure only: it runs the reference shader's compute passes
// on the host to pin the oracle).
//
// Definitions follow the WGSL specification; where WGSL leaves a result to
// the implementation, this header fixes one definition, the same one the
// oracle and the CUDA kernels use:
//   * binary32 round-to-nearest, no contraction (compile -ffp-contract=off);
//   * dot(a, b) sums left to right: (a.x*b.x + a.y*b.y) + a.z*b.z ...;
//     length(v) = sqrt(dot(v, v)); normalize(v) = v / length(v);
//   * inverseSqrt(x) = 1 / sqrt(x), both correctly rounded;
//   * round() ties to even; f32 -> i32/u32 truncates and saturates, NaN -> 0;
//   * min/max on f32 are fminf/fmaxf; clamp(e, lo, hi) = min(max(e, lo), hi);
//     mix(a, b, t) = a*(1-t) + b*t; smoothstep = t*t*(3-2t) with
//     t = clamp((x-lo)/(hi-lo), 0, 1); fract(x) = x - floor(x);
//   * exp, pow, sin, cos, atan2 are the binary32 functions of rfmm_math.h;
//   * atomic read-modify-writes are host atomics (relaxed; integer sums
//     commute, so the order of invocations does not change results).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>

#include "rfmm_math.h"

namespace wgsl {

template <class T, int N>
struct vec {
  T v[4];  // four slots for every width; only vec4 appears in buffers
  T &operator[](uint32_t i) { return v[i]; }
  const T &operator[](uint32_t i) const { return v[i]; }
};

template <class T, uint32_t Size>
struct arr {
  T v[Size];
  T &operator[](uint32_t i) { return v[i]; }
  const T &operator[](uint32_t i) const { return v[i]; }
};

template <class T>
struct is_vec : std::false_type {};
template <class T, int N>
struct is_vec<vec<T, N>> : std::true_type {};

// Scalar and vector conversions (WGSL T(e)).
template <class T, class U>
inline T convert(U x) {
  if constexpr (std::is_same_v<T, U>) {
    return x;
  } else if constexpr (is_vec<T>::value) {
    T r{};
    for (int i = 0; i < 4; i++) r.v[i] = convert<std::remove_reference_t<decltype(r.v[0])>>(x.v[i]);
    return r;
  } else if constexpr (std::is_floating_point_v<U> && std::is_same_v<T, int32_t>) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483648.0f) return INT32_MIN;
    return (int32_t)x;
  } else if constexpr (std::is_floating_point_v<U> && std::is_same_v<T, uint32_t>) {
    if (x != x || x <= 0.0f) return 0u;
    if (x >= 4294967296.0f) return UINT32_MAX;
    return (uint32_t)x;
  } else {
    return static_cast<T>(x);
  }
}

// Vector constructors: one argument splats (scalar) or converts (vector);
// several arguments concatenate scalars and vectors.
template <class T>
struct vec_width;
template <class T, int N>
struct vec_width<vec<T, N>> {
  static constexpr int value = N;
};

template <class T, int N, class A>
inline void append(vec<T, N> &r, int &k, const A &a) {
  if constexpr (is_vec<A>::value) {
    for (int i = 0; i < vec_width<A>::value; i++) r.v[k++] = static_cast<T>(a.v[i]);
  } else {
    r.v[k++] = static_cast<T>(a);
  }
}

template <class T, int N, class A>
inline vec<T, N> make(A a) {
  vec<T, N> r{};
  if constexpr (is_vec<A>::value) {
    for (int i = 0; i < N; i++) r.v[i] = convert<T>(a.v[i]);
  } else {
    for (int i = 0; i < N; i++) r.v[i] = convert<T>(a);
  }
  return r;
}
template <class T, int N, class A, class B, class... R>
inline vec<T, N> make(A a, B b, R... rest) {
  vec<T, N> r{};
  int k = 0;
  append(r, k, a);
  append(r, k, b);
  (append(r, k, rest), ...);
  return r;
}

template <int... I, class T, int N>
inline vec<T, (int)sizeof...(I)> swizzle(const vec<T, N> &a) {
  vec<T, (int)sizeof...(I)> r{};
  int k = 0;
  ((r.v[k++] = a.v[I]), ...);
  return r;
}

// Component-wise operators.
#define WGSL_VEC_BINOP(OP)                                                        \
  template <class T, int N>                                                       \
  inline vec<T, N> operator OP(const vec<T, N> &a, const vec<T, N> &b) {          \
    vec<T, N> r{};                                                                \
    for (int i = 0; i < N; i++) r.v[i] = static_cast<T>(a.v[i] OP b.v[i]);       \
    return r;                                                                     \
  }                                                                               \
  template <class T, int N, class S, class = std::enable_if_t<std::is_arithmetic_v<S>>> \
  inline vec<T, N> operator OP(const vec<T, N> &a, S s) {                         \
    vec<T, N> r{};                                                                \
    for (int i = 0; i < N; i++) r.v[i] = static_cast<T>(a.v[i] OP static_cast<T>(s)); \
    return r;                                                                     \
  }                                                                               \
  template <class T, int N, class S, class = std::enable_if_t<std::is_arithmetic_v<S>>> \
  inline vec<T, N> operator OP(S s, const vec<T, N> &a) {                         \
    vec<T, N> r{};                                                                \
    for (int i = 0; i < N; i++) r.v[i] = static_cast<T>(static_cast<T>(s) OP a.v[i]); \
    return r;                                                                     \
  }                                                                               \
  template <class T, int N, class S>                                              \
  inline vec<T, N> &operator OP##=(vec<T, N> &a, const S &b) {                    \
    a = a OP b;                                                                   \
    return a;                                                                     \
  }
WGSL_VEC_BINOP(+)
WGSL_VEC_BINOP(-)
WGSL_VEC_BINOP(*)
WGSL_VEC_BINOP(/)
#undef WGSL_VEC_BINOP

template <class T, int N>
inline vec<T, N> operator-(const vec<T, N> &a) {
  vec<T, N> r{};
  for (int i = 0; i < N; i++) r.v[i] = static_cast<T>(-a.v[i]);
  return r;
}

#define WGSL_VEC_CMP(OP)                                                          \
  template <class T, int N>                                                       \
  inline vec<bool, N> operator OP(const vec<T, N> &a, const vec<T, N> &b) {       \
    vec<bool, N> r{};                                                             \
    for (int i = 0; i < N; i++) r.v[i] = a.v[i] OP b.v[i];                        \
    return r;                                                                     \
  }
WGSL_VEC_CMP(<)
WGSL_VEC_CMP(<=)
WGSL_VEC_CMP(>)
WGSL_VEC_CMP(>=)
WGSL_VEC_CMP(==)
WGSL_VEC_CMP(!=)
#undef WGSL_VEC_CMP

template <int N>
inline bool any(const vec<bool, N> &a) {
  bool r = false;
  for (int i = 0; i < N; i++) r = r || a.v[i];
  return r;
}
template <int N>
inline bool all(const vec<bool, N> &a) {
  bool r = true;
  for (int i = 0; i < N; i++) r = r && a.v[i];
  return r;
}

// Scalar builtins, lifted component-wise below.
inline float s_abs(float x) { return fabsf(x); }
inline int32_t s_abs(int32_t x) { return x < 0 ? (int32_t)(0u - (uint32_t)x) : x; }
inline uint32_t s_abs(uint32_t x) { return x; }
inline float s_min(float a, float b) { return fminf(a, b); }
inline float s_max(float a, float b) { return fmaxf(a, b); }
template <class T>
inline T s_min(T a, T b) { return b < a ? b : a; }
template <class T>
inline T s_max(T a, T b) { return a < b ? b : a; }

template <class T>
inline auto abs(const T &x) {
  if constexpr (is_vec<T>::value) {
    T r{};
    for (int i = 0; i < 4; i++) r.v[i] = s_abs(x.v[i]);
    return r;
  } else {
    return s_abs(x);
  }
}
template <class T, class U>
inline auto min(const T &a, const U &b) {
  if constexpr (is_vec<T>::value) {
    T r{};
    for (int i = 0; i < 4; i++) r.v[i] = s_min(a.v[i], b.v[i]);
    return r;
  } else {
    return s_min(a, static_cast<T>(b));
  }
}
template <class T, class U>
inline auto max(const T &a, const U &b) {
  if constexpr (is_vec<T>::value) {
    T r{};
    for (int i = 0; i < 4; i++) r.v[i] = s_max(a.v[i], b.v[i]);
    return r;
  } else {
    return s_max(a, static_cast<T>(b));
  }
}
template <class T, class U, class V>
inline auto clamp(const T &e, const U &lo, const V &hi) {
  return min(max(e, lo), hi);
}

template <class F, class T>
inline T lift(F f, const T &x) {
  if constexpr (is_vec<T>::value) {
    T r{};
    for (int i = 0; i < 4; i++) r.v[i] = f(x.v[i]);
    return r;
  } else {
    return f(x);
  }
}
template <class T>
inline T floor(const T &x) { return lift([](float a) { return floorf(a); }, x); }
template <class T>
inline T ceil(const T &x) { return lift([](float a) { return ceilf(a); }, x); }
template <class T>
inline T round(const T &x) { return lift([](float a) { return rintf(a); }, x); }
template <class T>
inline T trunc(const T &x) { return lift([](float a) { return truncf(a); }, x); }
template <class T>
inline T fract(const T &x) { return lift([](float a) { return a - floorf(a); }, x); }
template <class T>
inline T sqrt(const T &x) { return lift([](float a) { return sqrtf(a); }, x); }
template <class T>
inline T inverseSqrt(const T &x) { return lift([](float a) { return 1.0f / sqrtf(a); }, x); }
template <class T>
inline T exp(const T &x) { return lift([](float a) { return rf_expf(a); }, x); }
template <class T>
inline T sin(const T &x) { return lift([](float a) { return rf_sinf(a); }, x); }
template <class T>
inline T cos(const T &x) { return lift([](float a) { return rf_cosf(a); }, x); }
inline float pow(float a, float b) { return rf_powf(a, b); }
inline float atan2(float y, float x) { return rf_atan2f(y, x); }

template <class T, int N>
inline T dot(const vec<T, N> &a, const vec<T, N> &b) {
  T s = a.v[0] * b.v[0];
  for (int i = 1; i < N; i++) s = s + a.v[i] * b.v[i];
  return s;
}
template <int N>
inline float length(const vec<float, N> &a) { return sqrtf(dot(a, a)); }
inline float length(float a) { return fabsf(a); }
template <int N>
inline vec<float, N> normalize(const vec<float, N> &a) { return a / length(a); }
template <int N>
inline float distance(const vec<float, N> &a, const vec<float, N> &b) { return length(a - b); }
inline vec<float, 3> cross(const vec<float, 3> &a, const vec<float, 3> &b) {
  return vec<float, 3>{{a.v[1] * b.v[2] - a.v[2] * b.v[1], a.v[2] * b.v[0] - a.v[0] * b.v[2],
                        a.v[0] * b.v[1] - a.v[1] * b.v[0], 0.0f}};
}
template <class T>
inline T mix(const T &a, const T &b, float t) { return a * (1.0f - t) + b * t; }
inline float smoothstep(float lo, float hi, float x) {
  const float t = fminf(fmaxf((x - lo) / (hi - lo), 0.0f), 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
template <class T>
inline T select(const T &f, const T &t, bool c) { return c ? t : f; }

template <class T>
inline T mod(T a, T b) {
  if constexpr (std::is_floating_point_v<T>) {
    return a - b * truncf(a / b);
  } else {
    return b == 0 ? a : a % b;
  }
}

// Atomics: the harness may run a dispatch's invocations on several host
// threads, so the read-modify-write forms are real atomic operations.
// Integer sums wrap modulo 2^32 like the device's.
template <class T, class U>
inline T atomicAdd(T *p, U v) {
  static_assert(sizeof(T) == 4, "32-bit atomics only");
  return (T)__atomic_fetch_add(reinterpret_cast<uint32_t *>(p), (uint32_t)(T)v, __ATOMIC_RELAXED);
}
template <class T, class U>
inline T atomicSub(T *p, U v) {
  static_assert(sizeof(T) == 4, "32-bit atomics only");
  return (T)__atomic_fetch_sub(reinterpret_cast<uint32_t *>(p), (uint32_t)(T)v, __ATOMIC_RELAXED);
}
template <class T>
inline T atomicLoad(T *p) { return *p; }
template <class T, class U>
inline void atomicStore(T *p, U v) { *p = (T)v; }

}  // namespace wgsl
