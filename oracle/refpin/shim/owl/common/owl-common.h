// owl-common.h -- TEST INFRASTRUCTURE ONLY: a restatement of the parts of
// the owl math library (owl::common, >= 1.2.9) that the reference's
// structured-volume headers use, written for this project because the owl
// submodule is empty in the reference checkout.  The semantics are the ones
// the CPU oracle states (oracle/gbv_oracle.cpp header):
//   min/max as std::min/std::max ((b<a)?b:a, (a<b)?b:a), clamp(v,lo,hi) =
//   min(hi,max(lo,v)), rcp(x) = 1.f/x, reduce_min/max = min(min(x,y),z),
//   dot = (x*x'+y*y')+z*z', normalize(v) = v*(1/sqrt(dot(v,v))),
//   interval<float> default-constructs empty (+inf,-inf), span = upper-lower.
// Compiled only into the reference pin harness (oracle/_ref/).
#pragma once
#include <algorithm>
#include <cassert>
#include <cmath>
#include <math.h>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <sstream>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#define __both__ /* host only */
#define OWL_ALIGN(a) alignas(a)
// debug-print macros of owl
#define PING std::cout << __FILE__ << "::" << __LINE__ << ": " << __FUNCTION__ << std::endl
#define PRINT(var) std::cout << #var << "=" << (var) << std::endl
#define OWL_TERMINAL_RED ""
#define OWL_TERMINAL_GREEN ""
#define OWL_TERMINAL_YELLOW ""
#define OWL_TERMINAL_BLUE ""
#define OWL_TERMINAL_LIGHT_RED ""
#define OWL_TERMINAL_DEFAULT ""
#define OWL_TERMINAL_RESET ""

namespace owl {
namespace common {

using std::max;
using std::min;

inline float rcp(float f) { return 1.f / f; }
inline double rcp(double f) { return 1. / f; }

template <typename T> inline T clamp(T v, T lo, T hi) { return min(hi, max(lo, v)); }
inline int divRoundUp(int a, int b) { return (a + b - 1) / b; }
inline size_t divRoundUp(size_t a, size_t b) { return (a + b - 1) / b; }

}  // namespace common
}  // namespace owl
