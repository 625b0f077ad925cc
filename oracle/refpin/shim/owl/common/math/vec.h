// vec.h -- TEST INFRASTRUCTURE ONLY: owl::common small vectors, restated
// for the reference pin harness (see owl-common.h for the semantics).
#pragma once
#include "../owl-common.h"

namespace owl {
namespace common {

template <typename T, int N> struct vec_t;

template <typename T> struct vec_t<T, 2> {
  T x, y;
  vec_t() = default;
  vec_t(T s) : x(s), y(s) {}
  vec_t(T a, T b) : x(a), y(b) {}
  template <typename U> explicit vec_t(const vec_t<U, 2> &o) : x(T(o.x)), y(T(o.y)) {}
  T &operator[](int i) { return i == 0 ? x : y; }
  T operator[](int i) const { return i == 0 ? x : y; }
};
template <typename T> struct vec_t<T, 3> {
  T x, y, z;
  vec_t() = default;
  vec_t(T s) : x(s), y(s), z(s) {}
  vec_t(T a, T b, T c) : x(a), y(b), z(c) {}
  template <typename U> explicit vec_t(const vec_t<U, 3> &o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
  // the xyz of a 4-vector
  template <typename U> explicit vec_t(const vec_t<U, 4> &o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
  // a plain struct of x, y, z (the backends' float3 records)
  template <typename S, typename = decltype(S::x), typename = decltype(S::z)>
  explicit vec_t(const S &o, ...) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
  T &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <typename T> struct vec_t<T, 4> {
  T x, y, z, w;
  vec_t() = default;
  vec_t(T s) : x(s), y(s), z(s), w(s) {}
  vec_t(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
  vec_t(const vec_t<T, 3> &v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
  template <typename U> explicit vec_t(const vec_t<U, 4> &o) : x(T(o.x)), y(T(o.y)), z(T(o.z)), w(T(o.w)) {}
  T &operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

typedef vec_t<float, 2> vec2f;
typedef vec_t<float, 3> vec3f;
typedef vec_t<float, 4> vec4f;
typedef vec_t<double, 3> vec3d;
typedef vec_t<int, 2> vec2i;
typedef vec_t<int, 3> vec3i;
typedef vec_t<int, 4> vec4i;
typedef vec_t<uint32_t, 2> vec2ui;
typedef vec_t<uint32_t, 3> vec3ui;
typedef vec_t<uint32_t, 4> vec4ui;
typedef vec_t<int64_t, 3> vec3l;
typedef vec_t<uint8_t, 4> vec4uc;
typedef vec_t<uint8_t, 3> vec3uc;

// componentwise application
template <typename T, typename F> inline vec_t<T, 2> cw(const vec_t<T, 2> &a, F f) { return {f(a.x), f(a.y)}; }
template <typename T, typename F> inline vec_t<T, 3> cw(const vec_t<T, 3> &a, F f) {
  return {f(a.x), f(a.y), f(a.z)};
}
template <typename T, typename F> inline vec_t<T, 4> cw(const vec_t<T, 4> &a, F f) {
  return {f(a.x), f(a.y), f(a.z), f(a.w)};
}
template <typename T, typename F> inline vec_t<T, 2> cw2(const vec_t<T, 2> &a, const vec_t<T, 2> &b, F f) {
  return {f(a.x, b.x), f(a.y, b.y)};
}
template <typename T, typename F> inline vec_t<T, 3> cw2(const vec_t<T, 3> &a, const vec_t<T, 3> &b, F f) {
  return {f(a.x, b.x), f(a.y, b.y), f(a.z, b.z)};
}
template <typename T, typename F> inline vec_t<T, 4> cw2(const vec_t<T, 4> &a, const vec_t<T, 4> &b, F f) {
  return {f(a.x, b.x), f(a.y, b.y), f(a.z, b.z), f(a.w, b.w)};
}

#define OWL_SHIM_BINOP(OP)                                                                                   \
  template <typename T, int N> inline vec_t<T, N> operator OP(const vec_t<T, N> &a, const vec_t<T, N> &b) {  \
    return cw2(a, b, [](T p, T q) { return p OP q; });                                                       \
  }                                                                                                          \
  template <typename T, int N> inline vec_t<T, N> operator OP(const vec_t<T, N> &a, T s) {                   \
    return cw(a, [s](T p) { return p OP s; });                                                               \
  }                                                                                                          \
  template <typename T, int N> inline vec_t<T, N> operator OP(T s, const vec_t<T, N> &a) {                   \
    return cw(a, [s](T p) { return s OP p; });                                                               \
  }                                                                                                          \
  template <typename T, int N> inline vec_t<T, N> &operator OP##=(vec_t<T, N> &a, const vec_t<T, N> &b) {    \
    return a = a OP b;                                                                                       \
  }                                                                                                          \
  template <typename T, int N> inline vec_t<T, N> &operator OP##=(vec_t<T, N> &a, T s) { return a = a OP s; }
OWL_SHIM_BINOP(+)
OWL_SHIM_BINOP(-)
OWL_SHIM_BINOP(*)
OWL_SHIM_BINOP(/)
#undef OWL_SHIM_BINOP

template <typename T, int N> inline vec_t<T, N> operator-(const vec_t<T, N> &a) {
  return cw(a, [](T p) { return -p; });
}
template <typename T> inline bool operator==(const vec_t<T, 3> &a, const vec_t<T, 3> &b) {
  return a.x == b.x && a.y == b.y && a.z == b.z;
}
template <typename T> inline bool operator!=(const vec_t<T, 3> &a, const vec_t<T, 3> &b) { return !(a == b); }

template <typename T, int N> inline vec_t<T, N> min(const vec_t<T, N> &a, const vec_t<T, N> &b) {
  return cw2(a, b, [](T p, T q) { return std::min(p, q); });
}
template <typename T, int N> inline vec_t<T, N> max(const vec_t<T, N> &a, const vec_t<T, N> &b) {
  return cw2(a, b, [](T p, T q) { return std::max(p, q); });
}
template <typename T, int N> inline vec_t<T, N> abs(const vec_t<T, N> &a) {
  return cw(a, [](T p) { return std::abs(p); });
}
template <typename T, int N> inline vec_t<T, N> rcp(const vec_t<T, N> &a) {
  return cw(a, [](T p) { return T(1) / p; });
}
template <typename T> inline T reduce_min(const vec_t<T, 3> &a) { return std::min(std::min(a.x, a.y), a.z); }
template <typename T> inline T reduce_max(const vec_t<T, 3> &a) { return std::max(std::max(a.x, a.y), a.z); }
template <typename T> inline T reduce_min(const vec_t<T, 4> &a) {
  return std::min(std::min(std::min(a.x, a.y), a.z), a.w);
}
template <typename T> inline T reduce_max(const vec_t<T, 4> &a) {
  return std::max(std::max(std::max(a.x, a.y), a.z), a.w);
}
template <typename T> inline int arg_min(const vec_t<T, 3> &a) {
  return a.x <= a.y ? (a.x <= a.z ? 0 : 2) : (a.y <= a.z ? 1 : 2);
}
template <typename T> inline int arg_max(const vec_t<T, 3> &a) {
  return a.x >= a.y ? (a.x >= a.z ? 0 : 2) : (a.y >= a.z ? 1 : 2);
}
template <typename T> inline T dot(const vec_t<T, 3> &a, const vec_t<T, 3> &b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename T> inline vec_t<T, 3> cross(const vec_t<T, 3> &a, const vec_t<T, 3> &b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename T> inline T length(const vec_t<T, 3> &a) { return std::sqrt(dot(a, a)); }
template <typename T> inline vec_t<T, 3> normalize(const vec_t<T, 3> &a) {
  return a * (T(1) / std::sqrt(dot(a, a)));
}
template <typename T, int N> inline vec_t<T, N> divRoundUp(const vec_t<T, N> &a, const vec_t<T, N> &b) {
  return (a + b - vec_t<T, N>(T(1))) / b;
}
template <typename T, int N> inline vec_t<T, N> clamp(const vec_t<T, N> &v, const vec_t<T, N> &lo,
                                                      const vec_t<T, N> &hi) {
  return min(hi, max(lo, v));
}

}  // namespace common
}  // namespace owl
