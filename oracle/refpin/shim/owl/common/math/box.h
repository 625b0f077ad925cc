// box.h -- TEST INFRASTRUCTURE ONLY: owl::common intervals and boxes,
// restated for the reference pin harness (see owl-common.h).
#pragma once
#include "vec.h"

namespace owl {
namespace common {

template <typename T> struct interval {
  T lower, upper;
  interval() : lower(std::numeric_limits<T>::infinity()), upper(-std::numeric_limits<T>::infinity()) {}
  interval(T lo, T hi) : lower(lo), upper(hi) {}
  T span() const { return upper - lower; }
  T center() const { return (lower + upper) / T(2); }
  bool empty() const { return upper < lower; }
  void extend(T v) {
    lower = min(lower, v);
    upper = max(upper, v);
  }
  void extend(const interval &o) {
    lower = min(lower, o.lower);
    upper = max(upper, o.upper);
  }
};
typedef interval<float> range1f;

template <typename V> struct box_t {
  V lower, upper;
  box_t() = default;
  box_t(const V &lo, const V &hi) : lower(lo), upper(hi) {}
  V size() const { return upper - lower; }
  V span() const { return upper - lower; }
  V center() const { return (lower + upper) * typename std::remove_reference<decltype(lower.x)>::type(.5); }
};
typedef box_t<vec3f> box3f;
typedef box_t<vec4f> box4f;
typedef box_t<vec3i> box3i;
typedef box_t<vec2f> box2f;
typedef box_t<vec2i> box2i;

}  // namespace common
}  // namespace owl
