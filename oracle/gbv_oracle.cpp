// gbv_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU oracle for the structured-volume path: a restatement, in plain C++, of
// what the reference renderer (Barney 1.1.8) computes on its embree (CPU)
// backend.  It is the checker for the CUDA product and is never shipped or
// measured as the product.  Only tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py may load it.
//
// Pinned by the reference's own code: the reference holds no golden vectors
// for this path (its unitTests/ cover umesh iso-surfaces and an omni camera
// only) and cannot be built as a whole here (submodules owl/embree/cuBQL/
// optix are empty), but its sources for the path compile unchanged against a
// restated owl and a stubbed embree API (oracle/refpin); the scalar kernels,
// the sampler, the per-ray isProg, the sRGB packing and the NanoVDB field
// code agree with this file bit for bit (tests/test_oracle_refpin.py).  The
// rest is pinned by known-answer tests and by an independent pure-Python
// restatement of the scalar kernels.
//
// Every function names the reference file:line it follows.  The third-party
// owl math library (owl::common, >= 1.2.9, submodule commit unrecorded) is
// absent; its semantics are restated in the small vector section below:
//   rcp(x) = 1.f/x componentwise; min/max as std::min/std::max
//   ((b<a)?b:a and (a<b)?b:a); clamp(v,lo,hi) = min(hi,max(lo,v));
//   reduce_min/max = min(min(x,y),z); dot = (x*x'+y*y')+z*z';
//   normalize(v) = v*(1/sqrt(dot(v,v))); length = sqrt(dot);
//   interval<float> default-constructs empty (+inf,-inf), extend = min/max,
//   span() = upper-lower.
//
// Build with -ffp-contract=off so that x86-64 and aarch64 hosts give
// identical FP32 results (no fused multiply-add).

#include "gbv_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace orc {

// ---------------------------------------------------------------------------
// owl-equivalent vector math (restated; see header comment)
// ---------------------------------------------------------------------------
template <typename T> inline T mn(T a, T b) { return (b < a) ? b : a; }
template <typename T> inline T mx(T a, T b) { return (a < b) ? b : a; }
template <typename T> inline T clampv(T v, T lo, T hi) { return mn(hi, mx(lo, v)); }

template <typename R> struct V3 {
  R x, y, z;
  V3() : x(0), y(0), z(0) {}
  V3(R a, R b, R c) : x(a), y(b), z(c) {}
  explicit V3(R a) : x(a), y(a), z(a) {}
  R &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <typename R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename R> inline V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <typename R> inline V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <typename R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <typename R> inline V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <typename R> inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <typename R> inline bool operator==(V3<R> a, V3<R> b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
template <typename R> inline V3<R> vmin(V3<R> a, V3<R> b) { return {mn(a.x, b.x), mn(a.y, b.y), mn(a.z, b.z)}; }
template <typename R> inline V3<R> vmax(V3<R> a, V3<R> b) { return {mx(a.x, b.x), mx(a.y, b.y), mx(a.z, b.z)}; }
template <typename R> inline V3<R> vabs(V3<R> a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
template <typename R> inline V3<R> rcp(V3<R> a) { return {R(1) / a.x, R(1) / a.y, R(1) / a.z}; }
template <typename R> inline V3<R> vfloor(V3<R> a) { return {std::floor(a.x), std::floor(a.y), std::floor(a.z)}; }
template <typename R> inline R reduce_min(V3<R> a) { return mn(mn(a.x, a.y), a.z); }
template <typename R> inline R reduce_max(V3<R> a) { return mx(mx(a.x, a.y), a.z); }
template <typename R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename R> inline V3<R> cross(V3<R> a, V3<R> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename R> inline V3<R> normalize(V3<R> v) { return v * (R(1) / std::sqrt(dot(v, v))); }
template <typename R> inline R length(V3<R> v) { return std::sqrt(dot(v, v)); }
template <typename R> inline V3<R> vmin_s(V3<R> a, R s) { return vmin(a, V3<R>(s)); }
template <typename R, typename S> inline V3<R> cvt(V3<S> a) { return {R(a.x), R(a.y), R(a.z)}; }

template <typename R> struct V4 { R x, y, z, w; };

static const float INF = INFINITY;
static const float ONE_PI = 3.14159265358979323846f;
static const float TWO_PI = 2.f * 3.14159265358979323846f;
static const float FOUR_PI = 4.f * 3.14159265358979323846f;
static const float ONE_OVER_PI = 1.f / 3.14159265358979323846f;
static const float ONE_OVER_TWO_PI = 1.f / (2.f * 3.14159265358979323846f);
static const float ONE_OVER_FOUR_PI = 1.f / (4.f * 3.14159265358979323846f);

// Sine and cosine of an angle x in [-pi/4, 2 pi + pi/4], the bounded method
// of the library's device code (orc_scene.bounded_math; the reference uses
// libm): Cody-Waite reduction r = x - k pi/2, k = rint(x 2/pi), with pi/2
// split into three floats (201/128, the next 21 bits, the rest rounded), so
// r is exact near multiples of pi/2; then Taylor polynomials of sin (to r^9)
// and cos (to r^10) on |r| <= pi/4 in Horner form, and the quadrant k mod 4
// picks signs and roles.  Built without contraction, like the device code.
static void bounded_sincos(float x, float &sn, float &cs) {
  const float k = rintf(x * 0.636619772f);
  const float r = ((x - k * 0x1.92p+0f) - k * 0x1.fb544p-12f) - k * 0x1.0b4612p-34f;
  const float r2 = r * r;
  const float ps = r + (r * r2) * (-1.f / 6.f + r2 * (1.f / 120.f + r2 * (-1.f / 5040.f + r2 * (1.f / 362880.f))));
  const float pc =
      1.f - .5f * r2 + (r2 * r2) * (1.f / 24.f + r2 * (-1.f / 720.f + r2 * (1.f / 40320.f + r2 * (-1.f / 3628800.f))));
  const int q = (int)k & 3;
  if (q == 0) { sn = ps; cs = pc; }
  else if (q == 1) { sn = pc; cs = -ps; }
  else if (q == 2) { sn = -ps; cs = -pc; }
  else { sn = -pc; cs = ps; }
}
// the path's sine and cosine: libm (the reference) or the bounded method
inline void path_sincos(bool bounded, float x, float &sn, float &cs) {
  if (bounded) bounded_sincos(x, sn, cs);
  else { sn = sinf(x); cs = cosf(x); }
}
// Arc cosine and two-argument arc tangent by the library's series
// (orc_scene.bounded_math; the reference uses libm): asin s = s + s t P(t)
// with t = s^2 on [0, 1/2], acos from it by pi/2 - asin z or
// 2 asin(sqrt((1 -+ z)/2)) (pi minus that for z < -1/2); atan u = u + u w Q(w)
// with w = u^2 on |u| <= tan(pi/8), atan2 by the pi/4 reduction of the
// magnitude ratio, then pi/2 - a, pi - a and the sign of y.  P, Q are the
// library's fitted coefficients; pi/2, pi, pi/4 as two-float sums.
static const float PIO2_HI = 0x1.921fb6p+0f, PIO2_LO = -0x1.777a5cp-25f;
static const float PI_HI = 0x1.921fb6p+1f, PI_LO = -0x1.777a5cp-24f;
static const float PIO4_HI = 0x1.921fb6p-1f, PIO4_LO = -0x1.777a5cp-26f;
static float series_asin(float s, float t) {
  float p = 0x1.06a85p-5f;
  p = p * t + 0x1.28e096p-6f;
  p = p * t + 0x1.fa3d84p-6f;
  p = p * t + 0x1.6d7fd6p-5f;
  p = p * t + 0x1.3333a6p-4f;
  p = p * t + 0x1.555556p-3f;
  return s + (s * t) * p;
}
static float bounded_acos(float z) {
  const float a = fabsf(z);
  if (a <= 0.5f) {
    const float s = copysignf(series_asin(a, a * a), z);
    return (PIO2_LO - s) + PIO2_HI;
  }
  const float t = (1.f - a) * 0.5f;
  const float w = 2.f * series_asin(sqrtf(t), t);
  if (z > 0.f) return w;
  return (PI_LO - w) + PI_HI;
}
static float series_atan(float u) {
  const float w = u * u;
  float q = -0x1.4b32d6p-5f;
  q = q * w + 0x1.2441d2p-4f;
  q = q * w - 0x1.71d376p-4f;
  q = q * w + 0x1.c6f68p-4f;
  q = q * w - 0x1.2491cp-3f;
  q = q * w + 0x1.999998p-3f;
  q = q * w - 0x1.555556p-2f;
  return u + (u * w) * q;
}
static float bounded_atan2(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float big = ax < ay ? ay : ax, small = ax < ay ? ax : ay;
  float a;
  if (big == 0.f) a = 0.f;
  else if (small > 0x1.a8279ap-2f * big) a = (PIO4_LO + series_atan((small - big) / (small + big))) + PIO4_HI;
  else a = series_atan(small / big);
  if (ay > ax) a = (PIO2_LO - a) + PIO2_HI;
  if (std::signbit(x)) a = (PI_LO - a) + PI_HI;
  return copysignf(a, y);
}

// ---------------------------------------------------------------------------
// half precision with the embree backend's rounding (rtcore/embree/Float16.cpp
// float32ToFloat16: round to nearest, ties away from zero; subnormals kept)
// ---------------------------------------------------------------------------
inline uint16_t f2h(float value) {
  uint32_t bits;
  std::memcpy(&bits, &value, 4);
  int i = (int)bits;
  int s = (i >> 16) & 0x00008000;
  int e = ((i >> 23) & 0x000000ff) - (127 - 15);
  int m = i & 0x007fffff;
  if (e <= 0) {
    if (e < -10) return uint16_t(s);
    m = (m | 0x00800000) >> (1 - e);
    if (m & 0x00001000) m += 0x00002000;
    return uint16_t(s | (m >> 13));
  } else if (e == 0xff - (127 - 15)) {
    if (m == 0) return uint16_t(s | 0x7c00);
    m >>= 13;
    return uint16_t(s | 0x7c00 | m | (m == 0));
  } else {
    if (m & 0x00001000) {
      m += 0x00002000;
      if (m & 0x00800000) { m = 0; e += 1; }
    }
    if (e > 30) return uint16_t(s | 0x7c00);
    return uint16_t(s | (e << 10) | (m >> 13));
  }
}
// rtcore/embree/Float16.cpp float16ToFloat32 (exact widening)
inline float h2f(uint16_t h) {
  uint32_t s = (h >> 15) & 1, e = (h >> 10) & 0x1f, m = h & 0x3ff, out;
  if (e == 0) {
    if (m == 0) out = s << 31;
    else {
      while (!(m & 0x400)) { m <<= 1; e -= 1; }
      e += 1; m &= ~0x400u;
      out = (s << 31) | ((e + (127 - 15)) << 23) | (m << 13);
    }
  } else if (e == 31) {
    out = (s << 31) | 0x7f800000u | (m << 13);
  } else {
    out = (s << 31) | ((e + (127 - 15)) << 23) | (m << 13);
  }
  float f;
  std::memcpy(&f, &out, 4);
  return f;
}
// vec3h <-> vec3f (barney/common/half.h:47-71)
struct V3h { uint16_t x, y, z; };
inline V3h toh(V3<float> v) { return {f2h(v.x), f2h(v.y), f2h(v.z)}; }
inline V3<float> fromh(V3h v) { return {h2f(v.x), h2f(v.y), h2f(v.z)}; }

// ---------------------------------------------------------------------------
// RNG (barney/common/barney-common.h:65-152)
// ---------------------------------------------------------------------------
struct RNGSeed {
  uint64_t state = 0xcafef00dd15ea5e5ull;
  uint32_t next() {                              // :74-82
    uint64_t x = state;
    const uint64_t multiplier = 6364136223846793005ull;
    unsigned count = (unsigned)(x >> 61);
    state = x * multiplier;
    x ^= x >> 22;
    return (uint32_t)(x >> (22 + count));
  }
  uint32_t next_h(uint64_t hash) {               // :87-93
    state ^= (hash << 1);
    return next();
  }
};
// RNGSeed::seed's arguments are uint32_t: 2*a+1 wraps in 32 bits before the
// xor with the 64-bit state.  Keep that exact behaviour.
inline void rng_seed(RNGSeed &r, uint32_t a, uint32_t b) {
  r.state ^= (uint64_t)(uint32_t)(2u * a + 1u);
  r.next();
  r.state ^= (uint64_t)(uint32_t)(2u * b);
  r.next();
}
struct Random2 : RNGSeed {                       // :97-111
  Random2(uint32_t a, uint32_t b) { rng_seed(*this, a, b); }
  // Random2(RNGSeed &seed, uint32_t b) and (RNGSeed &seed, uint64_t b): both
  // end in next((uint64_t)b) after the widening, so one form covers both.
  Random2(RNGSeed &seed, uint64_t b) {
    state = seed.state;
    seed.next();
    next_h(b ? b : 290374ull);
  }
  // a stream resumed from a saved state
  struct Resume {};
  Random2(Resume, uint64_t st) { state = st; }
  float operator()() { return (next() & 0x00FFFFFF) * (1.f / (float)0x01000000); }
};
inline uint64_t fnv_hash1(uint32_t v) {          // :132-137
  const uint64_t off = 0xcbf29ce484222325ull, prime = 0x100000001b3ull;
  return off ^ (prime * (uint64_t)v);
}
inline uint64_t fnv_hash2(uint64_t h, uint32_t v) { return (h * 0x100000001b3ull) ^ (uint64_t)v; }
inline uint64_t fnv_hash3(uint32_t a, uint32_t b, uint32_t c) { return fnv_hash2(fnv_hash2(fnv_hash1(a), b), c); }
inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
// The shading step's `(const uint32_t&)ray.tMax` (shadeRays.cu:610, 722): a
// C-style cast to a const reference of another type is a static_cast that
// converts the value into a temporary -- the hit distance truncated to an
// integer, not its bits.
inline uint32_t hit_hash(float t) { return static_cast<uint32_t>(t); }

// Volume.h:174-184
inline float fastLog(float f) {
  f = (f - 1.f) / (f + 1.f);
  float f2 = f * f;
  float s = f;
  f *= f2;
  s += (1.f / 3.f) * f;
  f *= f2;
  s += (1.f / 5.f) * f;
  return s + s;
}
inline double fastLog(double f) {
  f = (f - 1.0) / (f + 1.0);
  double f2 = f * f;
  double s = f;
  f *= f2;
  s += (1.0 / 3.0) * f;
  f *= f2;
  s += (1.0 / 5.0) * f;
  return s + s;
}

// ---------------------------------------------------------------------------
// Field and transfer function
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// NanoVDB grids (orc_scene.nanovdb): the reference's NanoVDB field
// (barney/volume/NanoVDB.{h,cu}) over the NanoVDB 32 buffer layout -- grid
// header (672 B, value type at 636), tree header (64 B), root (64 B +
// 32-byte tiles keyed by the 4096^3 region), upper nodes (32^3 entries,
// child mask at 4128, table at 8256), lower nodes (16^3, 544, 1088), leaves
// (8^3 values at 96: floats, or for the quantized types Fp4/Fp8/Fp16/FpN
// codes c with value float(c) * quantum (at 84) + minimum (at 80), FpN's bit
// width 1 << (flags (at 15) >> 5)); child offsets are signed and relative to
// the parent (the root for root tiles).
// ---------------------------------------------------------------------------
struct Nvdb {
  const unsigned char *b = nullptr;
  uint32_t type = 1;  // nanovdb::GridType: Float 1, Fp4 13, Fp8 14, Fp16 15, FpN 16
  int64_t root = 0;
  uint32_t tiles = 0;
  float background = 0.f;
  float inv[9] = {0}, vec[3] = {0};
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  V3<float> wlo, whi;  // world bounds as floats (NanoVDBData::commit)
  int M[3] = {0, 0, 0};  // macrocells: divRoundUp(index size, 16) (NanoVDBData::buildMCs)
};
template <typename T> inline T nv_get(const unsigned char *p) {
  T v;
  std::memcpy(&v, p, sizeof(T));
  return v;
}
inline Nvdb nv_parse(const unsigned char *b) {
  Nvdb g;
  g.b = b;
  g.type = nv_get<uint32_t>(b + 636);
  g.root = 672 + nv_get<int64_t>(b + 672 + 24);
  g.tiles = nv_get<uint32_t>(b + g.root + 24);
  g.background = nv_get<float>(b + g.root + 28);
  for (int i = 0; i < 9; i++) g.inv[i] = nv_get<float>(b + 296 + 36 + 4 * i);
  for (int i = 0; i < 3; i++) {
    g.vec[i] = nv_get<float>(b + 296 + 72 + 4 * i);
    g.lo[i] = nv_get<int32_t>(b + g.root + 4 * i);
    g.hi[i] = nv_get<int32_t>(b + g.root + 12 + 4 * i);
    g.wlo[i] = (float)nv_get<double>(b + 560 + 8 * i);
    g.whi[i] = (float)nv_get<double>(b + 560 + 24 + 8 * i);
    g.M[i] = (g.hi[i] - g.lo[i] + 1 + 15) / 16;
  }
  return g;
}
// LeafData<BuildType>::getValue (NanoVDB.h: LeafData<float>, <Fp4>, <Fp8>,
// <Fp16>, <FpN>) for voxel n of the leaf at lf
inline float nv_leaf_value(uint32_t type, const unsigned char *lf, uint32_t n) {
  const unsigned char *codes = lf + 96;
  uint32_t c = 0;
  switch (type) {
  case 1: return nv_get<float>(codes + 4 * (size_t)n);
  case 13: c = (codes[n / 2] >> (4 * (n % 2))) & 0xfu; break;
  case 14: c = codes[n]; break;
  case 15: c = nv_get<uint16_t>(codes + 2 * (size_t)n); break;
  default: {  // FpN: the branched form of getValue
    switch (lf[15] >> 5) {
    case 0: c = (codes[n / 8] >> (n % 8)) & 1u; break;
    case 1: c = (codes[n / 4] >> (2 * (n % 4))) & 3u; break;
    case 2: c = (codes[n / 2] >> (4 * (n % 2))) & 15u; break;
    case 3: c = codes[n]; break;
    default: c = nv_get<uint16_t>(codes + 2 * (size_t)n); break;
    }
  }
  }
  const float q = nv_get<float>(lf + 84), m = nv_get<float>(lf + 80);
  return float(c) * q + m;
}
// ReadAccessor::getValue
inline float nv_value(const Nvdb &g, int x, int y, int z) {
  const unsigned char *root = g.b + g.root;
  const uint64_t key = uint64_t(uint32_t(z) >> 12) | (uint64_t(uint32_t(y) >> 12) << 21) |
                       (uint64_t(uint32_t(x) >> 12) << 42);
  for (uint32_t t = 0; t < g.tiles; t++) {
    const unsigned char *tile = root + 64 + 32 * (size_t)t;
    if (nv_get<uint64_t>(tile) != key) continue;
    const int64_t child = nv_get<int64_t>(tile + 8);
    if (!child) return nv_get<float>(tile + 20);
    const unsigned char *up = root + child;
    const uint32_t n2 = ((uint32_t(x) & 4095u) >> 7) * 1024u + ((uint32_t(y) & 4095u) >> 7) * 32u +
                        ((uint32_t(z) & 4095u) >> 7);
    if (!(nv_get<uint64_t>(up + 4128 + 8 * (n2 / 64)) & (1ull << (n2 % 64))))
      return nv_get<float>(up + 8256 + 8 * (size_t)n2);
    const unsigned char *lw = up + nv_get<int64_t>(up + 8256 + 8 * (size_t)n2);
    const uint32_t n1 = ((uint32_t(x) & 127u) >> 3) * 256u + ((uint32_t(y) & 127u) >> 3) * 16u +
                        ((uint32_t(z) & 127u) >> 3);
    if (!(nv_get<uint64_t>(lw + 544 + 8 * (n1 / 64)) & (1ull << (n1 % 64))))
      return nv_get<float>(lw + 1088 + 8 * (size_t)n1);
    const unsigned char *lf = lw + nv_get<int64_t>(lw + 1088 + 8 * (size_t)n1);
    const uint32_t n0 = (uint32_t(x) & 7u) * 64u + (uint32_t(y) & 7u) * 8u + (uint32_t(z) & 7u);
    return nv_leaf_value(g.type, lf, n0);
  }
  return g.background;
}
// NanoVDBDataSampler::DD::sample (NanoVDB.h:100-129): worldToIndexF (the
// translation in double, the 3x3 product in float with fmaf), -0.5,
// Clamp = fmax(fmin(x, hi), lo) to the index bbox, then the trilinear
// SampleFromVoxels<acc, 1>: floor, fractions, 8 values, lerp a + float(w) (b - a)
// along z, y, x.
inline float nv_sample(const Nvdb &g, V3<float> P) {
  const double d[3] = {(double)P.x - (double)g.vec[0], (double)P.y - (double)g.vec[1], (double)P.z - (double)g.vec[2]};
  const float f[3] = {(float)d[0], (float)d[1], (float)d[2]};
  double ip[3];
  for (int r = 0; r < 3; r++) {
    ip[r] = (double)std::fmaf(f[0], g.inv[3 * r], std::fmaf(f[1], g.inv[3 * r + 1], f[2] * g.inv[3 * r + 2]));
    ip[r] -= 0.5;
    ip[r] = std::fmax(std::fmin(ip[r], (double)g.hi[r]), (double)g.lo[r]);
  }
  int c[3];
  float w[3];
  for (int r = 0; r < 3; r++) {
    const double fl = std::floor(ip[r]);
    c[r] = (int32_t)fl;
    w[r] = (float)(ip[r] - fl);
  }
  auto L = [](float a, float b, float t) { return a + t * (b - a); };
  float v[2][2][2];
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++)
      for (int k = 0; k < 2; k++) v[i][j][k] = nv_value(g, c[0] + i, c[1] + j, c[2] + k);
  return L(L(L(v[0][0][0], v[0][0][1], w[2]), L(v[0][1][0], v[0][1][1], w[2]), w[1]),
           L(L(v[1][0][0], v[1][0][1], w[2]), L(v[1][1][0], v[1][1][1], w[2]), w[1]), w[0]);
}
// NanoVDBData_computeMCs (NanoVDB.cu:28-60): macrocell m spans index
// coordinates lo + (m*size)/M .. lo + ((m+1)*size)/M + 1, inclusive
inline void nv_mc_ranges(const Nvdb &g, float *out) {
  const int64_t n = (int64_t)g.M[0] * g.M[1] * g.M[2];
  int size[3];
  for (int r = 0; r < 3; r++) size[r] = g.hi[r] - g.lo[r] + 1;
  for (int64_t t = 0; t < n; t++) {
    const int m[3] = {int(t % g.M[0]), int((t / g.M[0]) % g.M[1]), int(t / ((int64_t)g.M[0] * g.M[1]))};
    int a[3], e[3];
    for (int r = 0; r < 3; r++) {
      a[r] = g.lo[r] + (m[r] * size[r]) / g.M[r];
      e[r] = g.lo[r] + ((m[r] + 1) * size[r]) / g.M[r] + 1;
    }
    float lo = INFINITY, hi = -INFINITY;
    for (int x = a[0]; x <= e[0]; x++)
      for (int y = a[1]; y <= e[1]; y++)
        for (int z = a[2]; z <= e[2]; z++) {
          const float v = nv_value(g, x, y, z);
          lo = mn(lo, v);
          hi = mx(hi, v);
        }
    out[2 * t] = lo;
    out[2 * t + 1] = hi;
  }
}

struct Field {
  bool isNvdb = false;
  Nvdb nv;
  const float *data;
  int N[3];          // numScalars
  int C[3];          // numCells = dims-1 (StructuredData.cu:142-151)
  V3<float> origin, spacing, rcpSpacing;
  V3<float> boundsLo, boundsHi;  // StructuredData.cu:176-180
  // U8 storage form (orc_scene.u8_scaled): (min, max) per 8^3-cell scale brick
  const float *u8lohi = nullptr;
  int ns[3] = {0, 0, 0};
};

// The library's U8 store: the corner voxel v of a cell in scale brick
// (min, max) reads back as min + (span/255) * round(255 (v - min) / span).
inline float u8_dequant(float v, float lo, float hi) {
  const float span = hi - lo;
  int q = 0;
  if (span > 0.f) q = (int)std::floor((v - lo) * (255.f / span) + .5f);
  q = std::min(255, std::max(0, q));
  const float scale = span > 0.f ? span / 255.f : 0.f;
  return lo + scale * (float)q;
}
// The 8 dequantized corners of cell (cx, cy, cz), in the store's order.
inline void u8_cell_corners(const Field &F, int cx, int cy, int cz, float c[8]) {
  const size_t sb = (size_t)(cx >> 3) + (size_t)F.ns[0] * ((size_t)(cy >> 3) + (size_t)F.ns[1] * (size_t)(cz >> 3));
  const float lo = F.u8lohi[2 * sb], hi = F.u8lohi[2 * sb + 1];
  const size_t Nx = F.N[0], Ny = F.N[1];
  for (int k = 0; k < 8; k++) {
    const int x = cx + (k & 1), y = cy + ((k >> 1) & 1), z = cz + (k >> 2);
    c[k] = u8_dequant(F.data[x + Nx * (y + Ny * (size_t)z)], lo, hi);
  }
}

inline Field make_field(const orc_scene *s) {
  Field f;
  if (s->nanovdb) {
    f.isNvdb = true;
    f.nv = nv_parse(s->nanovdb);
    f.data = nullptr;
    for (int i = 0; i < 3; i++) { f.N[i] = 0; f.C[i] = 0; }
    f.boundsLo = f.nv.wlo;
    f.boundsHi = f.nv.whi;
    f.origin = f.boundsLo;
    return f;
  }
  f.data = s->scalars;
  for (int i = 0; i < 3; i++) { f.N[i] = s->dims[i]; f.C[i] = s->dims[i] - 1; }
  f.origin = {s->origin[0], s->origin[1], s->origin[2]};
  f.spacing = {s->spacing[0], s->spacing[1], s->spacing[2]};
  f.rcpSpacing = rcp(f.spacing);
  f.boundsLo = f.origin;
  f.boundsHi = f.origin + f.spacing * V3<float>((float)f.C[0], (float)f.C[1], (float)f.C[2]);
  return f;
}

// rtcore/embree/Texture.cpp:324-336 lerpCoords_notNormalized
template <typename R> inline void lerpCoords(int N, R tc, int &i0, int &i1, R &f) {
  if (tc - R(.5) <= R(0)) { i0 = i1 = 0; f = R(0); return; }
  if (tc - R(.5) >= R(N - 1)) { i0 = i1 = N - 1; f = R(0); return; }
  f = (tc - R(.5)) - R(int(tc - R(.5)));
  i0 = int(tc - R(.5));
  i1 = i0 + 1;
}
template <typename R> inline R lerp_l(R f, R a, R b) { return (R(1) - f) * a + f * b; }

struct Tri {  // trilinear stencil, for the adjoint
  int ix[2], iy[2], iz[2];
  double fx, fy, fz;
};

// StructuredData.h:104-115 + rtcore/embree/Texture.cpp:339-411 (LINEAR, CLAMP,
// unnormalised).  Returns NaN outside [0,numCells).
template <typename R> inline R sample_field(const Field &F, V3<R> P, Tri *tri = nullptr);
// sample_field of the U8 storage form: the cell holding the stencil (a
// clamped axis uses cell 0 with weight 0 or cell N-2 with weight 1, as a
// cell store must) and its dequantized corners
inline float sample_field_u8(const Field &F, V3<float> P) {
  V3<float> rel = (P - F.origin) * F.rcpSpacing;
  if (rel.x < 0.f || rel.y < 0.f || rel.z < 0.f) return NAN;
  if (rel.x >= (float)F.C[0] || rel.y >= (float)F.C[1] || rel.z >= (float)F.C[2]) return NAN;
  V3<float> tc = rel + V3<float>(.5f);
  int x0, x1, y0, y1, z0, z1;
  float fx, fy, fz;
  lerpCoords<float>(F.N[0], tc.x, x0, x1, fx);
  lerpCoords<float>(F.N[1], tc.y, y0, y1, fy);
  lerpCoords<float>(F.N[2], tc.z, z0, z1, fz);
  if (x0 == x1 && x0 > 0) { x0 -= 1; fx = 1.f; }
  if (y0 == y1 && y0 > 0) { y0 -= 1; fy = 1.f; }
  if (z0 == z1 && z0 > 0) { z0 -= 1; fz = 1.f; }
  float c[8];
  u8_cell_corners(F, x0, y0, z0, c);
  float v00 = lerp_l(fx, c[0], c[1]), v01 = lerp_l(fx, c[2], c[3]);
  float v10 = lerp_l(fx, c[4], c[5]), v11 = lerp_l(fx, c[6], c[7]);
  float v0 = lerp_l(fy, v00, v01), v1 = lerp_l(fy, v10, v11);
  return lerp_l(fz, v0, v1);
}

template <typename R> inline R sample_field(const Field &F, V3<R> P, Tri *tri) {
  if (F.isNvdb) return R(nv_sample(F.nv, V3<float>((float)P.x, (float)P.y, (float)P.z)));
  if constexpr (std::is_same<R, float>::value) {
    if (F.u8lohi) return sample_field_u8(F, P);
  }
  V3<R> rel = (P - cvt<R>(F.origin)) * cvt<R>(F.rcpSpacing);
  if (rel.x < R(0) || rel.y < R(0) || rel.z < R(0)) return R(NAN);
  if (rel.x >= R(F.C[0]) || rel.y >= R(F.C[1]) || rel.z >= R(F.C[2])) return R(NAN);
  V3<R> tc = rel + V3<R>(R(.5));
  int x0, x1, y0, y1, z0, z1;
  R fx, fy, fz;
  lerpCoords<R>(F.N[0], tc.x, x0, x1, fx);
  lerpCoords<R>(F.N[1], tc.y, y0, y1, fy);
  lerpCoords<R>(F.N[2], tc.z, z0, z1, fz);
  const size_t Nx = F.N[0], Ny = F.N[1];
  auto at = [&](int i, int j, int k) { return R(F.data[i + Nx * (j + Ny * (size_t)k)]); };
  R v000 = at(x0, y0, z0), v001 = at(x1, y0, z0), v010 = at(x0, y1, z0), v011 = at(x1, y1, z0);
  R v100 = at(x0, y0, z1), v101 = at(x1, y0, z1), v110 = at(x0, y1, z1), v111 = at(x1, y1, z1);
  R v00 = lerp_l(fx, v000, v001), v01 = lerp_l(fx, v010, v011);
  R v10 = lerp_l(fx, v100, v101), v11 = lerp_l(fx, v110, v111);
  R v0 = lerp_l(fy, v00, v01), v1 = lerp_l(fy, v10, v11);
  if (tri) {
    tri->ix[0] = x0; tri->ix[1] = x1; tri->iy[0] = y0; tri->iy[1] = y1;
    tri->iz[0] = z0; tri->iz[1] = z1;
    tri->fx = fx; tri->fy = fy; tri->fz = fz;
  }
  return lerp_l(fz, v0, v1);
}

// rtcore/embree/Texture.cpp:249-271 (POINT filter, unnormalised): clamp, then
// truncate.  Used by the macrocell build at integer coordinates.
inline float point_field(const float *data, const int N[3], float x, float y, float z) {
  auto cl = [](float f, float lo, float hi) { return mx(mn(f, hi), lo); };  // Texture.cpp:15-18
  uint32_t lx = (uint32_t)cl(x, 0.f, N[0] - 1.f);
  uint32_t ly = (uint32_t)cl(y, 0.f, N[1] - 1.f);
  uint32_t lz = (uint32_t)cl(z, 0.f, N[2] - 1.f);
  return data[lx + size_t(N[0]) * (ly + size_t(N[1]) * lz)];
}

struct XF {
  const float *v;  // RGBA
  int n;
  float lo, hi, span, baseDensity;
};
inline XF make_xf(const float *tf, int n, float lo, float hi, float bd) {
  return XF{tf, n, lo, hi, hi - lo, bd};
}

// TransferFunction.h:66-86
template <typename R> inline V4<R> xf_map(const XF &xf, R s, int *idx_out = nullptr, R *f_out = nullptr,
                                          bool *clamped = nullptr) {
  R f = (s - R(xf.lo)) / R(xf.span);
  if (clamped) *clamped = !(f > R(0) && f < R(1));
  f = clampv(f, R(0), R(1));
  f *= R(xf.n - 1);
  int idx = clampv(int(f), 0, xf.n - 2);
  f -= R(idx);
  const float *v0 = xf.v + 4 * idx, *v1 = xf.v + 4 * (idx + 1);
  V4<R> r;
  r.x = (R(1) - f) * R(v0[0]) + f * R(v1[0]);
  r.y = (R(1) - f) * R(v0[1]) + f * R(v1[1]);
  r.z = (R(1) - f) * R(v0[2]) + f * R(v1[2]);
  r.w = (R(1) - f) * R(v0[3]) + f * R(v1[3]);
  r.w *= R(xf.baseDensity);
  if (idx_out) *idx_out = idx;
  if (f_out) *f_out = f;
  return r;
}

// TransferFunction.h:91-116
inline float xf_majorant(const XF &xf, float lower, float upper) {
  if (lower > upper) return 0.f;
  float f_lo = (lower - xf.lo) / xf.span;
  float f_hi = (upper - xf.lo) / xf.span;
  f_lo = clampv(f_lo, 0.f, 1.f);
  f_hi = clampv(f_hi, 0.f, 1.f);
  f_lo *= (xf.n - 1);
  f_hi *= (xf.n - 1);
  int idx0_lo = clampv(int(f_lo), 0, xf.n - 2);
  int idx0_hi = clampv(int(f_hi), 0, xf.n - 2);
  f_lo -= idx0_lo;
  f_hi -= idx0_hi;
  float lerp_lo = (1.f - f_lo) * xf.v[4 * idx0_lo + 3] + f_lo * xf.v[4 * (idx0_lo + 1) + 3];
  float lerp_hi = (1.f - f_hi) * xf.v[4 * idx0_hi + 3] + f_hi * xf.v[4 * (idx0_hi + 1) + 3];
  float m = 0.f;
  m = mx(m, lerp_lo);
  m = mx(m, lerp_hi);
  for (int i = idx0_lo + 1; i <= idx0_hi; i++) m = mx(m, xf.v[4 * i + 3]);
  return m * xf.baseDensity;
}

// Volume.h:66-80 (non-principled): NaN -> 0, else TF map
template <typename R> inline V4<R> sample_and_map(const Field &F, const XF &xf, V3<R> P) {
  R f = sample_field<R>(F, P);
  if (std::isnan(f)) return V4<R>{0, 0, 0, 0};
  return xf_map<R>(xf, f);
}

// ---------------------------------------------------------------------------
// Macrocells (StructuredData.cu:29-95, MCGrid.cu:63-116)
// ---------------------------------------------------------------------------
inline void mc_dims_of(const int N[3], int cpm, int M[3]) {
  for (int i = 0; i < 3; i++) {
    int cells = N[i] - 1;
    M[i] = cells <= 0 ? 0 : (cells + cpm - 1) / cpm;  // divRoundUp(numCells, cellsPerMC)
  }
}

inline void mc_range_one(const float *data, const int N[3], int cpm, int mx_, int my_, int mz_,
                         float &lo, float &hi) {
  lo = +INF;
  hi = -INF;
  for (int iiz = 0; iiz <= cpm; iiz++)
    for (int iiy = 0; iiy <= cpm; iiy++)
      for (int iix = 0; iix <= cpm; iix++) {
        int sx = mx_ * cpm + iix, sy = my_ * cpm + iiy, sz = mz_ * cpm + iiz;
        if (sx >= N[0] || sy >= N[1] || sz >= N[2]) continue;
        float f = point_field(data, N, (float)sx, (float)sy, (float)sz);
        lo = mn(lo, f);  // interval::extend
        hi = mx(hi, f);
      }
}

// ---------------------------------------------------------------------------
// Thread pool parallel_for (mirrors rtcore/embree/Compute.cpp:17-25: one
// worker per hardware thread, dynamic chunks)
// ---------------------------------------------------------------------------
template <typename F> void parallel_for(int64_t n, int nthreads, F &&fn, int64_t chunk = 1) {
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  if (nthreads == 1 || n <= chunk) {
    for (int64_t i = 0; i < n; i++) fn(i);
    return;
  }
  std::atomic<int64_t> next{0};
  std::vector<std::thread> pool;
  for (int t = 0; t < nthreads; t++)
    pool.emplace_back([&]() {
      while (true) {
        int64_t b = next.fetch_add(chunk);
        if (b >= n) break;
        int64_t e = std::min(n, b + chunk);
        for (int64_t i = b; i < e; i++) fn(i);
      }
    });
  for (auto &th : pool) th.join();
}

// ---------------------------------------------------------------------------
// Scene (host-side commits of camera, lights, env map)
// ---------------------------------------------------------------------------
struct Camera {  // Camera.cu:83-97
  V3<float> lens00, dir00, du, dv;
};
inline Camera commit_camera(const float pos[3], const float dir[3], const float up[3], float fovy) {
  Camera c;
  V3<float> from(pos[0], pos[1], pos[2]);
  V3<float> direction = normalize(V3<float>(dir[0], dir[1], dir[2]));  // set3f("direction") normalizes
  V3<float> vup(up[0], up[1], up[2]);
  V3<float> dir_00 = normalize(direction);
  V3<float> dir_du = normalize(cross(dir_00, vup));
  V3<float> dir_dv = normalize(cross(dir_du, dir_00));
  dir_00 = dir_00 * (float)(1.f / (2.0f * tanf((0.5f * fovy) * (float)M_PI / 180.0f)));
  c.lens00 = from;
  c.dir00 = dir_00;
  c.du = dir_du;
  c.dv = dir_dv;
  return c;
}

struct M3 { V3<float> vx, vy, vz; };  // owl linear3f, columns
inline V3<float> xfmVector(const M3 &m, V3<float> v) { return m.vx * v.x + m.vy * v.y + m.vz * v.z; }
// owl linear3f rcp(): inverse = adjoint^T / det
inline M3 inverse(const M3 &m) {
  V3<float> a = cross(m.vy, m.vz), b = cross(m.vz, m.vx), c = cross(m.vx, m.vy);
  float det = dot(m.vx, a);
  float r = 1.f / det;
  M3 t;  // rows of the inverse are a,b,c scaled; store as columns
  t.vx = V3<float>(a.x, b.x, c.x) * r;
  t.vy = V3<float>(a.y, b.y, c.y) * r;
  t.vz = V3<float>(a.z, b.z, c.z) * r;
  return t;
}

struct Env {
  bool present = false;
  bool boundedMath = false;  // orc_scene.bounded_math
  const float *tex = nullptr;
  int W = 0, H = 0;
  int addr[2] = {0, 0};
  M3 toWorld, toLocal;
  float scale = 1.f;
  std::vector<float> cdf_y, cdf_x;
};

// rtcore/embree/Texture.cpp:25-93 computeAddress for normalized coordinates
struct LerpAddr { int idx0, idx1; float f; };
inline LerpAddr compute_address(int mode, float tc, int N) {
  LerpAddr out{0, 0, 0.f};
  switch (mode) {
    case 0: {  // WRAP
      tc = tc * (float)N - .5f;
      tc = fmodf(tc, (float)N);
      if (tc < 0.f) tc += (float)N;
      float fc = floorf(tc);
      int ic = int(fc);
      out.f = tc - ic;
      out.idx0 = ic;
      out.idx1 = int(fmodf(tc + 1.f, (float)N));
    } break;
    case 3: {  // MIRROR
      tc = tc * N + .5f;
      float fc = floorf(tc);
      int ic = int(fc);
      out.f = tc - ic;
      int i0 = ic - 1, i1 = ic + 0;
      if (i0 < 0) i0 = -i0;
      if (i1 < 0) i1 = -i1;
      i0 = i0 % (2 * N);
      i1 = i1 % (2 * N);
      if (i0 >= N) i0 = 2 * N - 1 - i0;
      if (i1 >= N) i1 = 2 * N - 1 - i1;
      out.idx0 = i0;
      out.idx1 = i1;
    } break;
    case 2:  // BORDER: the embree backend leaves the address zeroed
      break;
    case 1:
    default: {  // CLAMP
      tc = tc * N;
      if (tc - .5f <= 0.f) { out.idx0 = out.idx1 = 0; out.f = 0.f; }
      else if (tc - .5f >= N - 1) { out.idx0 = out.idx1 = N - 1; out.f = 0.f; }
      else {
        out.f = (tc - .5f) - int(tc - .5f);
        out.idx0 = int(tc - .5f);
        out.idx1 = out.idx0 + 1;
      }
    } break;
  }
  return out;
}
// rtcore/embree/Texture.cpp:295-321 tex2D LINEAR, normalized coordinates
inline V4<float> tex2D(const float *tex, int W, int H, const int addr[2], float u, float v) {
  LerpAddr lx = compute_address(addr[0], u, W), ly = compute_address(addr[1], v, H);
  auto px = [&](int ix, int iy) -> V4<float> {
    const float *p = tex + 4 * ((size_t)ix + (size_t)iy * W);
    return {p[0], p[1], p[2], p[3]};
  };
  V4<float> v00 = px(lx.idx0, ly.idx0), v01 = px(lx.idx1, ly.idx0);
  V4<float> v10 = px(lx.idx0, ly.idx1), v11 = px(lx.idx1, ly.idx1);
  auto lrp = [](float f, V4<float> a, V4<float> b) -> V4<float> {
    return {(1.f - f) * a.x + f * b.x, (1.f - f) * a.y + f * b.y, (1.f - f) * a.z + f * b.z,
            (1.f - f) * a.w + f * b.w};
  };
  V4<float> v0 = lrp(lx.f, v00, v01), v1 = lrp(lx.f, v10, v11);
  return lrp(ly.f, v0, v1);
}

// EnvMap.cu:61-137 (ComputeWeights_xy, ComputeCDFs_doLine, Normalize_cdf_y)
inline void env_cdfs(const float *tex, int W, int H, const int addr[2], float *cdf_y, float *cdf_x,
                     bool boundedMath = false) {
  for (int iy = 0; iy < H; iy++)
    for (int ix = 0; ix < W; ix++) {
      float weight = 0.f;
      for (int iiy = 0; iiy <= 2; iiy++)
        for (int iix = 0; iix <= 2; iix++) {
          V4<float> t = tex2D(tex, W, H, addr, (ix + iix * .5f) / (W), (iy + iiy * .5f) / (H));
          weight = mx(weight, mx(mx(t.x, t.y), t.z));
        }
      cdf_x[ix + W * iy] = weight;
    }
  for (int y = 0; y < H; y++) {
    float *line = cdf_x + (size_t)y * W;
    float sum = 0.f;
    for (int ix = 0; ix < W; ix++) sum += line[ix];
    float rcp_sum = 1.f / sum;
    sum = 0.f;
    for (int ix = 0; ix < W; ix++) {
      sum += line[ix];
      line[ix] = sum * rcp_sum;
    }
    line[W - 1] = 1.f;
    float rel_y = (y + .5f) / H;
    const float theta = ONE_PI * rel_y;
    float sinTheta, cosTheta;
    path_sincos(boundedMath, theta, sinTheta, cosTheta);
    cdf_y[y] = sum * sinTheta;
  }
  float sum = 0.f;
  for (int i = 0; i < H; i++) sum += cdf_y[i];
  float rcp_sum = 1.f / sum;
  sum = 0.f;
  for (int i = 0; i < H; i++) {
    sum += cdf_y[i];
    cdf_y[i] = sum * rcp_sum;
  }
  cdf_y[H - 1] = 1.f;
}

struct DirLightDD { V3<float> direction; float radiance; V3<float> color; };

// U8 storage form: the (min, max) of each 8^3-cell scale brick over its 9^3
// voxels (the 8-cell macrocell range), and macrocell ranges bounding the
// dequantized corners of the macrocell's cells.
inline void u8_build(Field &F, std::vector<float> &lohi) {
  for (int i = 0; i < 3; i++) F.ns[i] = (F.C[i] + 7) >> 3;
  const size_t n = (size_t)F.ns[0] * F.ns[1] * F.ns[2];
  lohi.resize(2 * n);
  for (size_t b = 0; b < n; b++) {
    const int bx = (int)(b % F.ns[0]), by = (int)((b / F.ns[0]) % F.ns[1]), bz = (int)(b / ((size_t)F.ns[0] * F.ns[1]));
    mc_range_one(F.data, F.N, 8, bx, by, bz, lohi[2 * b], lohi[2 * b + 1]);
  }
  F.u8lohi = lohi.data();
}
inline void u8_mc_ranges(const Field &F, int cpm, const int M[3], float *out) {
  const size_t nmc = (size_t)M[0] * M[1] * M[2];
  for (size_t m = 0; m < nmc; m++) {
    const int x0 = (int)(m % M[0]) * cpm, y0 = (int)((m / M[0]) % M[1]) * cpm,
              z0 = (int)(m / ((size_t)M[0] * M[1])) * cpm;
    float lo = INF, hi = -INF;
    for (int z = z0; z < std::min(z0 + cpm, F.C[2]); z++)
      for (int y = y0; y < std::min(y0 + cpm, F.C[1]); y++)
        for (int x = x0; x < std::min(x0 + cpm, F.C[0]); x++) {
          float c[8];
          u8_cell_corners(F, x, y, z, c);
          for (int k = 0; k < 8; k++) { lo = mn(lo, c[k]); hi = mx(hi, c[k]); }
        }
    out[2 * m] = lo;
    out[2 * m + 1] = hi;
  }
}

struct Scene {
  Field F;
  XF xf;
  std::vector<float> majorants_own;
  std::vector<float> u8lohi;  // U8 storage form: (min, max) per scale brick
  const float *maj;
  int M[3];
  V3<float> mcOrigin, mcSpacing, mcRcpSpacing;
  Camera cam;
  int W, H;
  int numDir;
  DirLightDD dir[4];
  Env env;
  V4<float> bg;
  float ambient;
  int multi, volMS, maxVB;
  float aniso, scatAlb;
  // RTC instance hashes of the volume and the iso-surface (hash(instance,
  // 0, 0), MCAccelerator.h:389-392 and :614-615)
  uint64_t volHash = 0, isoHash = 0;
  // hit IDs (instance index and userID of the volume and the iso-surface)
  // and the auxiliary channels to write (orc_scene.aux_*)
  int volInst = 0, isoInst = -1, volUser = 0, isoUser = -1;
  float *auxDepth = nullptr;
  int *auxPrim = nullptr, *auxInst = nullptr, *auxObj = nullptr;
  // iso-surface geometry with its AnariMatte material
  bool iso = false, noVolume = false, isoFirst = false;
  float isoValue = 0.f, isoAlpha = 1.f, isoDelta = 0.f;
  V3<float> isoAlbedo{0.f, 0.f, 0.f};
  std::vector<float> isoRanges;  // the field's macrocell scalar ranges
};

inline void build_scene(const orc_scene *s, Scene &S) {
  S.F = make_field(s);
  S.xf = make_xf(s->tf, s->tf_n, s->domain[0], s->domain[1], s->base_density);
  int cpm = s->cells_per_mc;
  if (S.F.isNvdb) {
    // NanoVDBData::buildMCs (NanoVDB.cu:70-92): origin = worldBounds.lower,
    // spacing = worldBounds.size() * rcp(mcDims)
    for (int i = 0; i < 3; i++) S.M[i] = S.F.nv.M[i];
    S.mcOrigin = S.F.boundsLo;
    S.mcSpacing = (S.F.boundsHi - S.F.boundsLo) * rcp(V3<float>((float)S.M[0], (float)S.M[1], (float)S.M[2]));
  } else {
    mc_dims_of(S.F.N, cpm, S.M);
    // StructuredData.cu:70-76: mc origin = worldBounds.lower, spacing = cpm*gridSpacing
    S.mcOrigin = S.F.boundsLo;
    S.mcSpacing = V3<float>((float)cpm) * S.F.spacing;
  }
  S.mcRcpSpacing = rcp(S.mcSpacing);
  size_t nmc = (size_t)S.M[0] * S.M[1] * S.M[2];
  if (s->u8_scaled && !S.F.isNvdb) u8_build(S.F, S.u8lohi);
  std::vector<float> r;
  if (!s->majorants || s->iso_enabled) {
    r.resize(2 * nmc);
    if (S.F.isNvdb) nv_mc_ranges(S.F.nv, r.data());
    else if (s->u8_scaled) u8_mc_ranges(S.F, cpm, S.M, r.data());
    else orc_mc_ranges(s->scalars, s->dims, cpm, r.data());
  }
  if (s->majorants) S.maj = s->majorants;
  else {
    S.majorants_own.resize(nmc);
    if (s->iso_enabled && s->no_volume) std::fill(S.majorants_own.begin(), S.majorants_own.end(), 0.f);
    else
      orc_majorants(r.data(), (int)nmc, s->tf, s->tf_n, s->domain[0], s->domain[1], s->base_density,
                    S.majorants_own.data());
    S.maj = S.majorants_own.data();
  }
  S.volHash = fnv_hash3((uint32_t)s->volume_instance, 0, 0);
  S.volInst = s->volume_instance;
  S.volUser = s->volume_user_id;
  S.auxDepth = s->aux_depth;
  S.auxPrim = s->aux_prim_id;
  S.auxInst = s->aux_inst_id;
  S.auxObj = s->aux_obj_id;
  if (s->iso_enabled) {
    S.isoInst = s->iso_instance;
    S.isoUser = s->iso_user_id;
    S.iso = true;
    S.noVolume = s->no_volume != 0;
    S.isoFirst = S.noVolume || s->iso_instance < s->volume_instance;
    S.isoHash = fnv_hash3((uint32_t)s->iso_instance, 0, 0);
    S.isoValue = s->iso_value;
    S.isoRanges = std::move(r);
    // MCAccelerator.h:476-479
    S.isoDelta = length(S.F.boundsHi - S.F.boundsLo) * .1f / float(S.M[0] + S.M[1] + S.M[2]);
    // AnariMatte::DD::createBSDF (AnariMatte.h:50-62) with VALUE parameters
    // (PossiblyMappedParameter::DD::eval, Material.h:101-106): a NaN value
    // reads as (0, 0, 0, 1); opacity is (opacity, 0, 0, 1)
    V4<float> base{s->iso_color[0], s->iso_color[1], s->iso_color[2], s->iso_color[3]};
    if (std::isnan(base.x)) base = {0.f, 0.f, 0.f, 1.f};
    const float opacity = std::isnan(s->iso_opacity) ? 0.f : s->iso_opacity;
    const float reflectance = .85f;
    S.isoAlbedo = reflectance * V3<float>(base.x, base.y, base.z) * ONE_OVER_PI;
    S.isoAlpha = base.w * opacity;
  }
  S.cam = commit_camera(s->cam_pos, s->cam_dir, s->cam_up, s->fovy);
  S.W = s->width;
  S.H = s->height;
  S.numDir = std::min(4, std::max(0, s->num_dir_lights));
  for (int i = 0; i < S.numDir; i++) {
    // DirLight.cu:10-20 with the identity instance transform
    S.dir[i].direction = normalize(V3<float>(s->dir_light_dir[i][0], s->dir_light_dir[i][1], s->dir_light_dir[i][2]));
    S.dir[i].color = V3<float>(s->dir_light_color[i][0], s->dir_light_color[i][1], s->dir_light_color[i][2]);
    S.dir[i].radiance = s->dir_light_radiance[i];
  }
  S.env.boundedMath = s->bounded_math != 0;
  if (s->env_texels) {
    Env &e = S.env;
    e.present = true;
    e.tex = s->env_texels;
    e.W = s->env_dims[0];
    e.H = s->env_dims[1];
    e.addr[0] = s->env_addr[0];
    e.addr[1] = s->env_addr[1];
    e.scale = s->env_scale;
    // EnvMap.cu:164-179
    V3<float> up(s->env_up[0], s->env_up[1], s->env_up[2]);
    V3<float> dir(s->env_dir[0], s->env_dir[1], s->env_dir[2]);
    e.toWorld.vz = -normalize(up);
    e.toWorld.vy = -normalize(cross(e.toWorld.vz, dir));
    e.toWorld.vx = normalize(cross(e.toWorld.vy, e.toWorld.vz));
    e.toLocal = inverse(e.toWorld);
    e.cdf_y.resize(e.H);
    e.cdf_x.resize((size_t)e.W * e.H);
    env_cdfs(e.tex, e.W, e.H, e.addr, e.cdf_y.data(), e.cdf_x.data(), e.boundedMath);
  }
  S.bg = {s->bg_color[0], s->bg_color[1], s->bg_color[2], s->bg_color[3]};
  S.ambient = s->ambient_radiance;
  S.multi = s->multi_scatter;
  S.volMS = s->volume_multi_scatter;
  S.maxVB = s->max_volume_bounces;
  S.aniso = s->anisotropy;
  S.scatAlb = s->scattering_albedo;
}

// DG.h:97-106
inline float sphericalTheta(V3<float> v, bool boundedMath) {
  const float z = clampv(v.z, -1.f, 1.f);
  return boundedMath ? bounded_acos(z) : acosf(z);
}
inline float sphericalPhi(V3<float> v, bool boundedMath) {
  float p = boundedMath ? bounded_atan2(v.y, v.x) : atan2f(v.y, v.x);
  return (p < 0.f) ? (p + float(2.f * M_PI)) : p;
}
// EnvMap.h:98-134
inline float cdfGetPDF(int position, const float *cdf, int N) {
  float f_at = cdf[position];
  float f_before = position ? cdf[position - 1] : 0.f;
  return N * (f_at - f_before);
}
inline int sampleCDF(const float *cdf, int N, float v, float &pdf) {
  int begin = 0, end = N;
  while ((end - begin) > 1) {
    int mid = (begin + end) / 2;
    float f_mid = cdf[mid - 1];
    if (v < f_mid) end = mid;
    else begin = mid;
  }
  float f_at = cdf[begin];
  float f_before = begin ? cdf[begin - 1] : 0.f;
  pdf = N * (f_at - f_before);
  return begin;
}
// EnvMap.h:165-180
inline void env_worldToPixel(const Env &e, V3<float> worldDir, int &ix, int &iy) {
  V3<float> localDir = xfmVector(e.toLocal, worldDir);
  float theta = sphericalTheta(localDir, e.boundedMath);
  float phi = sphericalPhi(localDir, e.boundedMath);
  float u = phi * ONE_OVER_TWO_PI, v = theta * ONE_OVER_PI;
  ix = (int)clampv(u * (float)e.W, 0.f, e.W - 1.f);
  iy = (int)clampv(v * (float)e.H, 0.f, e.H - 1.f);
}
// EnvMap.h:136-163
inline float env_pdf(const Env &e, V3<float> dir) {
  if (!e.present) return ONE_OVER_FOUR_PI;
  int px, py;
  env_worldToPixel(e, dir, px, py);
  float pdf_y = cdfGetPDF(py, e.cdf_y.data(), e.H);
  float pdf_x = cdfGetPDF(px, e.cdf_x.data() + (size_t)py * e.W, e.W);
  float rel_y = (py + .5f) / e.H;
  const float theta = ONE_PI * rel_y;
  float sinTheta, cosTheta;
  path_sincos(e.boundedMath, theta, sinTheta, cosTheta);
  return pdf_x * pdf_y * 1.f / (TWO_PI * ONE_PI * sinTheta);
}
// EnvMap.h:198-210
inline V3<float> env_uvToWorld(const Env &e, float fx, float fy) {
  const float phi = TWO_PI * fx;
  const float theta = ONE_PI * fy;
  float sinTheta, cosTheta, sinPhi, cosPhi;
  path_sincos(e.boundedMath, theta, sinTheta, cosTheta);
  path_sincos(e.boundedMath, phi, sinPhi, cosPhi);
  V3<float> d;
  d.z = cosTheta;
  d.x = cosPhi * sinTheta;
  d.y = sinPhi * sinTheta;
  return xfmVector(e.toWorld, d);
}

struct LightSample {  // light/Light.h Light::Sample
  V3<float> radiance{0.f, 0.f, 0.f};
  V3<float> direction{0.f, 0.f, 0.f};
  float distance = 0.f;
  float pdf = 0.f;
};

// EnvMap.h:212-250
inline LightSample env_sample(const Env &e, Random2 &r) {
  LightSample sample;
  float r_y = r();
  float r_x = r();
  float pdf_y, pdf_x;
  int iy = sampleCDF(e.cdf_y.data(), e.H, r_y, pdf_y);
  int ix = sampleCDF(e.cdf_x.data() + (size_t)e.W * iy, e.W, r_x, pdf_x);
  float sx = (ix + r()) / e.W;
  float sy = (iy + r()) / e.H;
  V4<float> t = tex2D(e.tex, e.W, e.H, e.addr, sx, sy);
  sample.radiance = e.scale * V3<float>(t.x, t.y, t.z);
  sample.direction = env_uvToWorld(e, sx, sy);
  float rel_y = sy;
  const float theta = ONE_PI * rel_y;
  float sinTheta, cosTheta;
  path_sincos(e.boundedMath, theta, sinTheta, cosTheta);
  sample.pdf = pdf_x * pdf_y * 1.f / (TWO_PI * ONE_PI * sinTheta);
  sample.distance = INF;
  return sample;
}

// DG.h:183-193
inline V3<float> randomDirection(Random2 &rng) {
  V3<float> v;
  while (true) {
    v.x = 1.f - 2.f * rng();
    v.y = 1.f - 2.f * rng();
    v.z = 1.f - 2.f * rng();
    if (dot(v, v) <= 1.f) return normalize(v);
  }
}

// ---------------------------------------------------------------------------
// Ray record (render/Ray.h:49-99); only the fields this path reads
// ---------------------------------------------------------------------------
struct Ray {
  V3<float> org, dir;
  float tMax;
  RNGSeed rngSeed;
  V3<float> P;
  bool hit;          // bsdfType != NONE
  bool surf;         // the hit is on the iso-surface (Lambertian), else a volume hit (Phase)
  bool isShadowRay;
  V3<float> albedo;  // Phase data
  float g;
  V3h N;             // Ray::N, the surface hit's normal in half precision (Ray.h:84)
  V4<float> missColor;
};
struct PathState {   // render/Ray.h:18-26
  V3h throughput;
  float misWeight;
  int numDiffuseBounces;
  int numVolumeBounces;
};

struct Counters {
  uint64_t samples = 0, mcs = 0, rays = 0;
};

// Woodcock::sampleRange (Volume.h:188-223), templated on the arithmetic type
// of everything downstream of the 24-bit random numbers.
template <typename R>
inline bool woodcock(const Scene &S, V3<R> org, V3<R> dir, R t0, R &t1, R majorant, Random2 &rand,
                     V4<R> &sample, Counters &cnt) {
  R t = t0;
  while (true) {
    R r = R(rand());
    R dt = -fastLog(R(1) - r) / majorant;
    t += dt;
    if (t >= t1) return false;
    V3<R> P = org + t * dir;
    sample = sample_and_map<R>(S.F, S.xf, P);
    cnt.samples++;
    if (sample.w >= R(rand()) * majorant) {
      t1 = t;
      return true;
    }
  }
}

// Ray.h:175-187 boxTest
template <typename R> inline bool boxTest(V3<R> org, V3<R> dir, R &t0, R &t1, V3<R> lo, V3<R> hi) {
  V3<R> t_lo = (lo - org) * rcp(dir);
  V3<R> t_hi = (hi - org) * rcp(dir);
  V3<R> t_nr = vmin(t_lo, t_hi), t_fr = vmax(t_lo, t_hi);
  t0 = mx(t0, reduce_max(t_nr));
  t1 = mn(t1, reduce_min(t_fr));
  return t0 <= t1;
}

// MCVolumeAccel::isProg (MCAccelerator.h:569-708) + dda::dda3 (DDA.h:65-206)
// as dispatched by the embree backend (tmin 0, tmax ray.tMax, identity
// instance transform, geometry 0 of the volume's instance: S.volHash =
// hash(instance, 0, 0), instance 0 unless an iso-surface precedes it).
// The trace direction has zero components replaced by 1e-6
// (traceRays.dev.cu:41-44).  On a hit, fills t/rgb/P and returns true.
template <typename R>
inline bool trace(const Scene &S, Ray &ray, Counters &cnt, R &t_hit, V3<R> &rgb_hit) {
  cnt.rays++;
  V3<float> dirf = ray.dir;
  if (dirf.x == 0.f) dirf.x = 1e-6f;
  if (dirf.y == 0.f) dirf.y = 1e-6f;
  if (dirf.z == 0.f) dirf.z = 1e-6f;
  if (S.M[0] <= 0 || S.M[1] <= 0 || S.M[2] <= 0) return false;
  const V3<R> org = cvt<R>(ray.org), dir = cvt<R>(dirf);
  R tLo = R(0), tHi = R(ray.tMax);
  if (!boxTest<R>(org, dir, tLo, tHi, cvt<R>(S.F.boundsLo), cvt<R>(S.F.boundsHi))) return false;

  V3<R> dda_org = (org - cvt<R>(S.mcOrigin)) * rcp(cvt<R>(S.mcSpacing));
  V3<R> dda_dir = dir * rcp(cvt<R>(S.mcSpacing));
  Random2 rng(ray.rngSeed, S.volHash);
  const R tMaxRay = R(ray.tMax);
  const R tMax = tHi;

  // ---- dda3 ----
  const V3<R> f_size((R)S.M[0], (R)S.M[1], (R)S.M[2]);
  const V3<R> rcp_dir = rcp(dda_dir);
  V3<R> t_lo = (V3<R>(R(0)) - dda_org) * rcp(dda_dir);
  V3<R> t_hi = (f_size - dda_org) * rcp(dda_dir);
  V3<R> t_nr = vmin(t_lo, t_hi), t_fr = vmax(t_lo, t_hi);
  for (int a = 0; a < 3; a++) {
    if (dda_dir[a] == R(0)) {
      if (dda_org[a] < R(0) || dda_org[a] > f_size[a]) return false;
      t_nr[a] = -R(INFINITY);
      t_fr[a] = +R(INFINITY);
    }
  }
  R ray_t0 = mx(R(0), reduce_max(t_nr));
  R ray_t1 = mn(tMax, reduce_min(t_fr));
  if (ray_t0 > ray_t1) return false;
  V3<R> org_in_volume = dda_org + ray_t0 * dda_dir;
  V3<R> f_cell = vmax(V3<R>(R(0)), vmin(f_size - V3<R>(R(1)), vfloor(org_in_volume)));
  V3<R> f_cell_end(dda_dir.x > R(0) ? f_cell.x + R(1) : f_cell.x, dda_dir.y > R(0) ? f_cell.y + R(1) : f_cell.y,
                   dda_dir.z > R(0) ? f_cell.z + R(1) : f_cell.z);
  V3<R> t_step = vabs(rcp_dir);
  V3<R> t_next;
  for (int a = 0; a < 3; a++)
    t_next[a] = (dda_dir[a] == R(0)) ? R(INFINITY) : (std::fabs(f_cell_end[a] - org_in_volume[a]) * t_step[a]);
  int stop[3], delta[3], cell[3];
  for (int a = 0; a < 3; a++) {
    stop[a] = dda_dir[a] > R(0) ? S.M[a] : -1;
    delta[a] = dda_dir[a] > R(0) ? +1 : -1;
    cell[a] = int(f_cell[a]);
  }
  R next_cell_begin = R(0);
  const int maxIter = S.M[0] + S.M[1] + S.M[2] + 8;
  for (int it = 0; it < maxIter; it++) {
    R t_closest = reduce_min(t_next);
    const R cell_t0 = ray_t0 + next_cell_begin;
    const R cell_t1 = ray_t0 + mn(t_closest, tMax);
    // ---- lambda (MCAccelerator.h:56-146) ----
    const float majorant = S.maj[cell[0] + S.M[0] * (cell[1] + S.M[1] * cell[2])];
    if (majorant != 0.f) {
      cnt.mcs++;
      R segLo = cell_t0, segHi = mn(cell_t1, tMaxRay);
      V4<R> sample{0, 0, 0, 0};
      if (woodcock<R>(S, org, dir, segLo, segHi, R(majorant), rng, sample, cnt)) {
        t_hit = segHi;
        rgb_hit = V3<R>(sample.x, sample.y, sample.z);
        return true;
      }
    }
    next_cell_begin = t_closest;
    for (int a = 0; a < 3; a++) {
      if (t_next[a] == t_closest) {
        t_next[a] += t_step[a];
        cell[a] += delta[a];
        if (cell[a] == stop[a]) return false;
      }
    }
  }
  return false;
}

// MCIsoSurfaceAccel::isProg (barney/volume/MCAccelerator.h:338-567) up to
// the hit record: dda::dda3 (DDA.h:65-206) over the macrocell grid; per
// macrocell whose scalar range holds the iso value, the cell's t range is
// cut into 10 sub-steps, and the first sub-step whose end values bracket the
// iso value gives t by linear interpolation.  The normal is the central
// difference of the field at +-d per axis (one-sided where a sample falls
// outside the field), normalized.  `dir` is the trace direction (zero
// components already replaced by 1e-6, traceRays.dev.cu:41-44); the box test
// runs on [0, tmax].  `onBox` runs once the box test passes, where the
// reference constructs the geometry's random stream from ray.rngSeed.
template <class OnBox>
inline bool iso_isprog(const Field &F, const int M[3], V3<float> mcOrigin, V3<float> mcSpacing, const float *ranges,
                       float iso, float d, V3<float> org, V3<float> dir, float tmax, float &tOut, V3<float> &P,
                       V3<float> &N, OnBox onBox) {
  if (M[0] <= 0 || M[1] <= 0 || M[2] <= 0) return false;
  float tLo = 0.f, tHi = tmax;
  if (!boxTest<float>(org, dir, tLo, tHi, F.boundsLo, F.boundsHi)) return false;
  onBox();
  const V3<float> dda_org = (org - mcOrigin) * rcp(mcSpacing);
  const V3<float> dda_dir = dir * rcp(mcSpacing);
  const float tMax = tHi;
  // ---- dda3 ----
  const V3<float> f_size((float)M[0], (float)M[1], (float)M[2]);
  const V3<float> rcp_dir = rcp(dda_dir);
  V3<float> t_lo = (V3<float>(0.f) - dda_org) * rcp(dda_dir);
  V3<float> t_hi = (f_size - dda_org) * rcp(dda_dir);
  V3<float> t_nr = vmin(t_lo, t_hi), t_fr = vmax(t_lo, t_hi);
  for (int a = 0; a < 3; a++) {
    if (dda_dir[a] == 0.f) {
      if (dda_org[a] < 0.f || dda_org[a] > f_size[a]) return false;
      t_nr[a] = -INF;
      t_fr[a] = +INF;
    }
  }
  const float ray_t0 = mx(0.f, reduce_max(t_nr));
  const float ray_t1 = mn(tMax, reduce_min(t_fr));
  if (ray_t0 > ray_t1) return false;
  const V3<float> oiv = dda_org + ray_t0 * dda_dir;
  const V3<float> f_cell = vmax(V3<float>(0.f), vmin(f_size - V3<float>(1.f), vfloor(oiv)));
  const V3<float> f_end(dda_dir.x > 0.f ? f_cell.x + 1.f : f_cell.x, dda_dir.y > 0.f ? f_cell.y + 1.f : f_cell.y,
                        dda_dir.z > 0.f ? f_cell.z + 1.f : f_cell.z);
  const V3<float> t_step = vabs(rcp_dir);
  V3<float> t_next;
  for (int a = 0; a < 3; a++)
    t_next[a] = (dda_dir[a] == 0.f) ? INF : (std::fabs(f_end[a] - oiv[a]) * t_step[a]);
  int stop[3], delta[3], cell[3];
  for (int a = 0; a < 3; a++) {
    stop[a] = dda_dir[a] > 0.f ? M[a] : -1;
    delta[a] = dda_dir[a] > 0.f ? +1 : -1;
    cell[a] = int(f_cell[a]);
  }
  float tHit = tmax;
  float next_cell_begin = 0.f;
  const int maxIter = M[0] + M[1] + M[2] + 8;
  bool stopped = false;
  for (int it = 0; it < maxIter && !stopped; it++) {
    const float t_closest = reduce_min(t_next);
    const float t0 = ray_t0 + next_cell_begin;
    const float t1 = ray_t0 + mn(t_closest, tMax);
    // ---- the iso lambda (MCAccelerator.h:405-471) ----
    [&]() {
      if (t0 >= mn(t1, tmax)) return;
      const size_t ci = (size_t)cell[0] + (size_t)M[0] * ((size_t)cell[1] + (size_t)M[1] * cell[2]);
      const float vlo = ranges[2 * ci], vhi = ranges[2 * ci + 1];
      if (!(iso >= vlo && iso <= vhi)) return;
      float tt1 = t0;
      float ff1 = sample_field<float>(F, org + tt1 * dir);
      for (int i = 1; i <= 10; i++) {
        const float tt0 = tt1;
        const float ff0 = ff1;
        tt1 = lerp_l((float)i / 10.f, t0, t1);
        ff1 = sample_field<float>(F, org + tt1 * dir);
        if (std::isnan(ff0) || std::isnan(ff1)) continue;
        const float lo = mn(ff0, ff1), hi = mx(ff0, ff1);
        if (iso >= lo && iso <= hi) {
          float t = (iso - ff0) / (ff1 - ff0);
          t = lerp_l(t, tt0, tt1);
          tHit = mn(tHit, t);
          if (tHit < tmax) {
            stopped = true;
            return;
          }
        }
      }
    }();
    if (stopped) break;
    next_cell_begin = t_closest;
    bool done = false;
    for (int a = 0; a < 3 && !done; a++) {
      if (t_next[a] == t_closest) {
        t_next[a] += t_step[a];
        cell[a] += delta[a];
        if (cell[a] == stop[a]) done = true;
      }
    }
    if (done) break;
  }
  if (!(tHit < tmax)) return false;
  // ---- normal (MCAccelerator.h:476-503) ----
  P = org + tHit * dir;
  const float fP = sample_field<float>(F, P);
  float fx0 = sample_field<float>(F, P + V3<float>(-d, 0.f, 0.f));
  float fx1 = sample_field<float>(F, P + V3<float>(+d, 0.f, 0.f));
  float fy0 = sample_field<float>(F, P + V3<float>(0.f, -d, 0.f));
  float fy1 = sample_field<float>(F, P + V3<float>(0.f, +d, 0.f));
  float fz0 = sample_field<float>(F, P + V3<float>(0.f, 0.f, -d));
  float fz1 = sample_field<float>(F, P + V3<float>(0.f, 0.f, +d));
  float dx = 2.f, dy = 2.f, dz = 2.f;
  if (std::isnan(fx0)) { dx -= 1.f; fx0 = fP; }
  if (std::isnan(fx1)) { dx -= 1.f; fx1 = fP; }
  if (std::isnan(fy0)) { dy -= 1.f; fy0 = fP; }
  if (std::isnan(fy1)) { dy -= 1.f; fy1 = fP; }
  if (std::isnan(fz0)) { dz -= 1.f; fz0 = fP; }
  if (std::isnan(fz1)) { dz -= 1.f; fz1 = fP; }
  N = V3<float>(dx == 0.f ? 0.f : (fx1 - fx0) / dx, dy == 0.f ? 0.f : (fy1 - fy0) / dy,
                dz == 0.f ? 0.f : (fz1 - fz0) / dz);
  if (N == V3<float>(0.f)) N = -normalize(dir);
  N = normalize(N);
  tOut = tHit;
  return true;
}


// ---------------------------------------------------------------------------
// Shading (kernels/shadeRays.cu), volume-only world
// ---------------------------------------------------------------------------
// shadeRays.cu:141-191
inline bool sampleDirLights(const Scene &S, V3<float> N, Random2 &random, LightSample &ls) {
  if (S.numDir == 0) return false;
  const int RES = 2;
  int lID[RES];
  float weights[RES];
  float sumWeights = 0.f;
  for (int i = 0; i < RES; i++) {
    lID[i] = mn(int(random() * S.numDir), S.numDir - 1);
    weights[i] = 0.f;
    const DirLightDD &light = S.dir[lID[i]];
    V3<float> light_radiance = light.color * light.radiance;
    V3<float> lightDir = -light.direction;
    float weight = (N == V3<float>(0.f)) ? 1.f : dot(lightDir, N);
    if (weight <= 1e-3f) continue;
    weight *= reduce_max(light_radiance);
    if (weight <= 1e-3f) continue;
    weights[i] = weight;
    sumWeights += weight;
  }
  if (sumWeights == 0.f) return false;
  float r = random() * sumWeights;
  int i = 0;
  while (i < RES && r >= weights[i]) { r -= weights[i]; ++i; }
  if (i == RES) return false;
  const DirLightDD &light = S.dir[lID[i]];
  ls.direction = -light.direction;
  ls.distance = INF;
  ls.radiance = light.color * light.radiance * 1.f / (weights[i] / sumWeights * (float(RES) / float(S.numDir)));
  ls.pdf = INF;
  return weights[i] != 0.f;
}

// shadeRays.cu:268-293
inline bool sampleEnvLight(const Scene &S, V3<float> N, Random2 &random, LightSample &ls) {
  if (S.env.present) {
    ls = env_sample(S.env, random);
  } else {
    ls.direction = randomDirection(random);
    ls.distance = INF;
    if (!(N == V3<float>(0.f))) {
      ls.radiance = V3<float>(TWO_PI * S.ambient);
      if (dot(ls.direction, N) < 0.f) ls.direction = -ls.direction;
      ls.pdf = ONE_OVER_TWO_PI;
    } else {
      ls.radiance = V3<float>(FOUR_PI * S.ambient);
      ls.pdf = ONE_OVER_FOUR_PI;
    }
  }
  return true;
}

// shadeRays.cu:295-404 (no area or point lights in this world)
inline bool sampleLights(const Scene &S, V3<float> Ng, Random2 &random, LightSample &ls, bool &needsMIS,
                         bool &isDir) {
  needsMIS = false;
  LightSample els;
  float elsWeight = sampleEnvLight(S, Ng, random, els) ? reduce_max(els.radiance) : 0.f;
  LightSample als;  // no quad lights: sampleAreaLights returns false
  float alsWeight = 0.f;
  LightSample dls;
  float dlsWeight = sampleDirLights(S, Ng, random, dls) ? reduce_max(dls.radiance) : 0.f;
  float plsWeight = 0.f;
  float sumWeights = alsWeight + dlsWeight + elsWeight + plsWeight;
  if (sumWeights == 0.f) return false;
  elsWeight *= 1.f / sumWeights;
  alsWeight *= 1.f / sumWeights;
  dlsWeight *= 1.f / sumWeights;
  plsWeight *= 1.f / sumWeights;
  float r = random();
  if (r <= alsWeight) {
    // only reachable with r == 0 exactly; the reference then reads an
    // unfilled sample.  Here that sample is zero, so the pdf test rejects it.
    ls = als;
    ls.radiance = ls.radiance * (1.f / alsWeight);
  } else if (r <= alsWeight + elsWeight) {
    ls = els;
    ls.radiance = ls.radiance * (1.f / elsWeight);
    needsMIS = true;
  } else if (r <= alsWeight + elsWeight + plsWeight) {
    return false;  // unreachable: no point lights
  } else {
    ls = dls;
    ls.radiance = ls.radiance * (1.f / dlsWeight);
    isDir = true;
  }
  if (std::isnan(ls.pdf) || (ls.pdf <= 0.f)) return false;
  return true;
}

// shadeRays.cu:437-456
inline V3<float> radianceFromEnv(const Scene &S, const Ray &ray) {
  const Env &env = S.env;
  if (env.present) {
    V3<float> d = xfmVector(env.toLocal, normalize(ray.dir));
    float theta = sphericalTheta(d, S.env.boundedMath);
    float phi = sphericalPhi(d, S.env.boundedMath);
    const float invPi = 1.f / (float)M_PI;
    const float inv2Pi = 1.f / (2.f * (float)M_PI);
    float u = phi * inv2Pi, v = theta * invPi;
    V4<float> c = tex2D(env.tex, env.W, env.H, env.addr, u, v);
    return env.scale * V3<float>(c.x, c.y, c.z);
  }
  return V3<float>(S.ambient);
}

// Phase.h:49-57 / 145-146
inline float phase_pdf(const Scene &S, const Ray &ray, V3<float> wo, V3<float> wi) {
  if (!S.multi) return ONE_OVER_FOUR_PI;
  V3<float> wi_in = normalize(-wo);
  float cosTheta = dot(wi_in, normalize(wi));
  float g = ray.g;
  if (fabsf(g) < 1e-3f) return ONE_OVER_FOUR_PI;
  float g2 = g * g;
  float denom = 1.f + g2 - 2.f * g * cosTheta;
  return ONE_OVER_FOUR_PI * (1.f - g2) / (denom * sqrtf(denom));
}
inline float hgPhase(float g, float cosTheta) {
  if (fabsf(g) < 1e-3f) return ONE_OVER_FOUR_PI;
  float g2 = g * g;
  float denom = 1.f + g2 - 2.f * g * cosTheta;
  return ONE_OVER_FOUR_PI * (1.f - g2) / (denom * sqrtf(denom));
}
// Phase.h:74-99
inline V3<float> sampleHGDirection(V3<float> wi_in, float g, Random2 &random, bool boundedMath) {
  float u0 = random();
  float u1 = random();
  float cosTheta;
  if (fabsf(g) < 1e-3f) cosTheta = 1.f - 2.f * u0;
  else {
    float sqrTerm = (1.f - g * g) / (1.f + g - 2.f * g * u0);
    cosTheta = (1.f + g * g - sqrTerm * sqrTerm) / (2.f * g);
  }
  float sinTheta = sqrtf(mx(0.f, 1.f - cosTheta * cosTheta));
  float phi = TWO_PI * u1;
  float sinPhi, cosPhi;
  path_sincos(boundedMath, phi, sinPhi, cosPhi);
  V3<float> local(cosPhi * sinTheta, sinPhi * sinTheta, cosTheta);
  V3<float> w = normalize(wi_in);
  V3<float> u, v;
  if (fabsf(w.x) > 0.1f) u = normalize(cross(V3<float>(0.f, 1.f, 0.f), w));
  else u = normalize(cross(V3<float>(1.f, 0.f, 0.f), w));
  v = cross(w, u);
  return normalize(local.x * u + local.y * v + local.z * w);
}

struct Fragment { V3<float> rgb; };

// owl::common::frame, the orthonormal frame around a unit normal N that
// xfmVector(frame(N), v) uses: dx is the longer of (1,0,0) x N and
// (0,1,0) x N, normalized, and dy = normalize(N x dx).  (owl's source is
// absent from the reference checkout; this restates it.)
inline void frame_of(V3<float> N, V3<float> &dx, V3<float> &dy) {
  const V3<float> dx0 = cross(V3<float>(1.f, 0.f, 0.f), N), dx1 = cross(V3<float>(0.f, 1.f, 0.f), N);
  dx = normalize(dot(dx0, dx0) > dot(dx1, dx1) ? dx0 : dx1);
  dy = normalize(cross(N, dx));
}

// Lambertian::pdf (packedBSDF/Lambertian.h:46-55): cosine-hemisphere pdf
// about the normal turned toward wi
inline float lambert_pdf(V3<float> Ng, V3<float> wi) {
  V3<float> N = Ng;
  if (dot(wi, N) < 0.f) N = -N;
  const float cosThetaI = mx(dot(wi, N), 0.f);
  return cosThetaI * ONE_OVER_PI;  // cosineSampleHemispherePDF (DG.h:177-180)
}

// bounce() for an iso-surface hit (shadeRays.cu:541-878 with isVolumeHit
// false): Ng = normalize(ray.N), offsets along the front-facing normal Ngff,
// light sampling with Ngff (sampleDirLights weights by dot(lightDir, N), the
// ambient sample turns into N's hemisphere), the Lambertian of the
// AnariMatte material (Lambertian.h:57-90) with the cosine factors of the
// surface branches, and a diffuse scatter, at most MAX_DIFFUSE_BOUNCES = 1
// per path (shadeRays.cu:18, 795-808).  No fragment of its own.
inline V3<float> bounce_surface(const Scene &S, Ray &ray, PathState &state, Ray &shadowRay, PathState &shadowState,
                                bool &shadowValid, int pathDepth) {
  const float EPS = 1e-4f;
  const V3<float> fragment(0.f);
  const V3<float> incomingThroughput = fromh(state.throughput);
  const V3<float> Ng = normalize(fromh(ray.N));
  const bool hitWasOnFront = dot(ray.dir, Ng) < 0.f;
  const V3<float> Ngff = hitWasOnFront ? Ng : -Ng;
  Random2 random(ray.rngSeed, (uint64_t)hit_hash(ray.tMax));
  // DG (shadeRays.cu:625-629): Ng = Ns = the unflipped normal
  const V3<float> P = ray.P;
  const V3<float> wo = -normalize(ray.dir);
  const float offsetEpsilon = mx(EPS, 1e-6f * reduce_max(vabs(P)));  // safe_eps :39-43
  LightSample ls;
  bool needsMIS = false, isDir = false;
  if (sampleLights(S, Ngff, random, ls, needsMIS, isDir)) {
    // Lambertian::eval: cosine against Ns, unflipped
    const float cosThetaI = mx(dot(ls.direction, Ng), 0.f);
    V3<float> fr_value = S.isoAlbedo * ONE_OVER_PI * cosThetaI;
    const float fr_pdf = cosThetaI * ONE_OVER_PI;
    if (!(fr_pdf > 0.f) || reduce_max(fr_value) < 1e-4f) {
      shadowValid = false;
    } else {
      fr_value = vmin(fr_value, V3<float>(13.f));  // CLAMP_F_R
      V3<float> tp_sr = incomingThroughput * (std::isinf(ls.pdf) ? 1.f : 1.f / ls.pdf) * fr_value * ls.radiance *
                        (ONE_OVER_PI * std::fabs(dot(Ng, ls.direction)));
      shadowRay.hit = false;
      shadowRay.surf = false;
      shadowRay.isShadowRay = true;
      shadowRay.dir = ls.direction;
      shadowRay.org = P + offsetEpsilon * Ngff;
      shadowRay.tMax = ls.distance * (1.f - 2.f * offsetEpsilon);
      shadowState.throughput = toh(tp_sr);
      shadowRay.rngSeed = ray.rngSeed;
      ray.rngSeed.next_h((uint64_t)hit_hash(ray.tMax));
      shadowState.misWeight = 1.f;
      shadowValid = true;
      if (!isDir && needsMIS) {
        const float pdf_l = env_pdf(S.env, ls.direction);
        const float pdf_s = lambert_pdf(Ng, ls.direction);
        shadowState.misWeight = pdf_l / (pdf_l + pdf_s + 1e-10f);
        if (shadowState.misWeight < 1e-5f) shadowValid = false;
      }
    }
  }
  if (pathDepth >= 10) {  // MAX_PATH_DEPTH
    ray.tMax = -1.f;
    return fragment;
  }
  ray.hit = false;
  ray.surf = false;
  ray.tMax = INF;
  // Lambertian::scatter: a cosine-weighted direction about the normal
  // turned toward wo.  Its vec2f s(random(), random()) takes the second
  // argument's draw first: the reference's CPU backend is built with gcc,
  // which evaluates the arguments right to left.
  V3<float> N = Ng;
  if (dot(wo, N) < 0.f) N = -N;
  const float r0 = random();
  const float r1 = random();
  const float sx = r1, sy = r0;
  // cosineSampleHemisphere / cartesian (DG.h:135-168)
  const float phi = TWO_PI * sx;
  const float cosTheta = std::sqrt(sy);
  const float sinTheta = std::sqrt(1.0f - sy);
  float sinPhi, cosPhi;
  path_sincos(S.env.boundedMath, phi, sinPhi, cosPhi);
  const V3<float> local(cosPhi * sinTheta, sinPhi * sinTheta, cosTheta);
  V3<float> dx, dy;
  frame_of(N, dx, dy);
  const V3<float> sdir = dx * local.x + dy * local.y + N * local.z;
  const float spdf = local.z * ONE_OVER_PI;
  if (!(spdf > 0.f) || spdf <= 1e-6f) return fragment;  // ray stays alive unchanged
  // DIFFUSE scatter
  if (state.numDiffuseBounces >= 1) {
    ray.tMax = -1.f;
    return fragment;
  }
  state.numDiffuseBounces = state.numDiffuseBounces + 1;
  ray.org = P + (1.f * offsetEpsilon) * Ngff;
  ray.dir = normalize(sdir);
  V3<float> scatterFactor =
      S.isoAlbedo * std::fabs(dot(Ng, normalize(ray.dir))) / (std::isinf(spdf) ? 1.f : (spdf + 1e-10f));
  scatterFactor = vmin(scatterFactor, V3<float>(2.5f));
  state.throughput = toh(fromh(state.throughput) * scatterFactor);
  if (needsMIS && !std::isinf(spdf)) {
    const float pdf_s = lambert_pdf(Ng, ray.dir);
    const float pdf_l = env_pdf(S.env, ray.dir);
    state.misWeight = pdf_s / (pdf_s + pdf_l);
  } else {
    state.misWeight = 1.f;
  }
  return fragment;
}

// bounce() (shadeRays.cu:477-878): miss, volume-hit and (bounce_surface)
// iso-surface branches.  Returns the fragment; updates ray/state; fills the
// shadow ray.
inline V3<float> bounce(const Scene &S, Ray &ray, PathState &state, Ray &shadowRay, PathState &shadowState,
                        bool &shadowValid, int pathDepth) {
  const float EPS = 1e-4f;
  V3<float> fragment(0.f);
  shadowValid = false;
  const bool hadNoIntersection = !ray.hit;
  const V3<float> incomingThroughput = fromh(state.throughput);
  if (ray.isShadowRay) {
    if (hadNoIntersection) fragment = state.misWeight * fromh(state.throughput);
    ray.tMax = -1.f;
    return fragment;
  }
  // Ng = 0 for volume hits (N is never set for this world's hits)
  if (hadNoIntersection) {
    if (pathDepth == 0) {
      fragment = S.env.present ? radianceFromEnv(S, ray) : V3<float>(ray.missColor.x, ray.missColor.y, ray.missColor.z);
    } else {
      const V3<float> fromEnv = radianceFromEnv(S, ray);
      fragment = fromh(state.throughput) * fromEnv * state.misWeight;
    }
    ray.tMax = -1.f;
    return fragment;
  }
  if (ray.surf) return bounce_surface(S, ray, state, shadowRay, shadowState, shadowValid, pathDepth);
  // volume hit: isVolumeHit, hitWasOnFront false, Ngff = -Ng = -0
  const V3<float> Ngff(-0.f, -0.f, -0.f);
  Random2 random(ray.rngSeed, (uint64_t)hit_hash(ray.tMax));
  // DG (shadeRays.cu:625-639)
  const V3<float> P = ray.P;
  const V3<float> wo = -normalize(ray.dir);
  const float offsetEpsilon = mx(EPS, 1e-6f * reduce_max(vabs(P)));  // safe_eps :39-43
  const V3<float> frontFacingSurfaceOffset = wo;

  LightSample ls;
  bool needsMIS = false, isDir = false;
  if (sampleLights(S, Ngff, random, ls, needsMIS, isDir)) {
    // Phase::eval
    float density = S.multi ? phase_pdf(S, ray, wo, ls.direction) : ONE_OVER_FOUR_PI;
    V3<float> fr_value = density * ray.albedo;
    float fr_pdf = density;
    if (!(fr_pdf > 0.f) || reduce_max(fr_value) < 1e-4f) {
      shadowValid = false;
    } else {
      fr_value = vmin(fr_value, V3<float>(13.f));  // CLAMP_F_R
      V3<float> tp_sr = incomingThroughput * (std::isinf(ls.pdf) ? 1.f : 1.f / ls.pdf) * fr_value *
                        ls.radiance * 1.f;
      // makeShadowRay (Ray.h:152-163)
      shadowRay.hit = false;
      shadowRay.surf = false;
      shadowRay.isShadowRay = true;
      shadowRay.dir = ls.direction;
      shadowRay.org = P + offsetEpsilon * frontFacingSurfaceOffset;
      shadowRay.tMax = ls.distance * (1.f - 2.f * offsetEpsilon);
      shadowState.throughput = toh(tp_sr);
      shadowRay.rngSeed = ray.rngSeed;
      ray.rngSeed.next_h((uint64_t)hit_hash(ray.tMax));
      shadowState.misWeight = 1.f;
      shadowValid = true;
      if (!isDir && needsMIS) {
        float pdf_l = env_pdf(S.env, ls.direction);
        float pdf_s = S.multi ? phase_pdf(S, ray, wo, ls.direction) : ONE_OVER_FOUR_PI;
        shadowState.misWeight = pdf_l / (pdf_l + pdf_s + 1e-10f);
        if (shadowState.misWeight < 1e-5f) shadowValid = false;
      }
    }
  }
  if (pathDepth >= 10) {  // MAX_PATH_DEPTH
    ray.tMax = -1.f;
    return fragment;
  }
  ray.hit = false;
  ray.tMax = INF;
  // Phase::scatter
  V3<float> sdir;
  float spdf;
  V3<float> sf_r;
  if (S.multi) {
    V3<float> wi_in = normalize(-wo);
    sdir = sampleHGDirection(wi_in, ray.g, random, S.env.boundedMath);
    float density = hgPhase(ray.g, dot(wi_in, sdir));
    spdf = density;
    sf_r = ray.albedo * density;
  } else {
    float r1 = random();
    float r2 = random();
    float x = cosf(TWO_PI * r1) * sqrtf(r2 * (1.f - r2));
    float y = sinf(TWO_PI * r1) * sqrtf(r2 * (1.f - r2));
    float z = (1.f - 2.f * r2);
    spdf = ONE_OVER_FOUR_PI;
    sf_r = ray.albedo * spdf;
    sdir = V3<float>(x, y, z);
  }
  if (!(spdf > 0.f) || spdf <= 1e-6f) return fragment;  // ray stays alive unchanged
  // VOLUME scatter
  if (S.multi) {
    if (!S.volMS || state.numVolumeBounces >= S.maxVB) {
      ray.tMax = -1.f;
      return fragment;
    }
    state.numVolumeBounces = state.numVolumeBounces + 1;
  } else {
    ray.tMax = -1.f;  // SCI_VIS_MODE: volumes shadow, nothing more
    return fragment;
  }
  ray.org = P + (1.f * offsetEpsilon) * frontFacingSurfaceOffset;
  ray.dir = normalize(sdir);
  V3<float> scatterFactor = sf_r * 1.f / (std::isinf(spdf) ? 1.f : (spdf + 1e-10f));
  scatterFactor = vmin(scatterFactor, V3<float>(2.5f));
  state.throughput = toh(fromh(state.throughput) * scatterFactor);
  if (needsMIS && !std::isinf(spdf)) {
    float pdf_s = S.multi ? phase_pdf(S, ray, wo, ray.dir) : ONE_OVER_FOUR_PI;
    float pdf_l = env_pdf(S.env, ray.dir);
    state.misWeight = pdf_s / (pdf_s + pdf_l);
  } else {
    state.misWeight = 1.f;
  }
  return fragment;
}

// _generateRays (generateRays.cu:72-243), perspective camera without aperture
inline void generate(const Scene &S, int ix, int iy, int accumID, Ray &ray, PathState &state) {
  state.misWeight = 0.f;
  Random2 rand(unsigned(ix + S.W * accumID), unsigned(iy + S.H * accumID));
  ray.rngSeed = RNGSeed();
  rng_seed(ray.rngSeed, (uint32_t)(ix + accumID * S.W), (uint32_t)iy);
  float pixel_u = ((accumID == 0) ? .5f : rand());
  float pixel_v = ((accumID == 0) ? .5f : rand());
  float image_u = ((ix + pixel_u) / float(S.W));
  float image_v = ((iy + pixel_v) / float(S.H));
  float aspect = S.W / float(S.H);
  ray.org = S.cam.lens00;
  V3<float> ray_dir = S.cam.dir00 + (1.f * aspect * (image_u - .5f)) * S.cam.du + (1.f * (image_v - .5f)) * S.cam.dv;
  ray.dir = normalize(ray_dir);
  ray.hit = false;
  ray.surf = false;
  ray.isShadowRay = false;
  ray.tMax = 1e30f;
  state.numDiffuseBounces = 0;
  state.numVolumeBounces = 0;
  const float t = (iy + .5f) / float(S.H);
  V4<float> bg = S.bg;
  if (!(S.bg.w >= 0.f)) {
    bg.x = (1.0f - t) * 0.9f + t * 0.15f;
    bg.y = (1.0f - t) * 0.9f + t * 0.25f;
    bg.z = (1.0f - t) * 0.9f + t * .8f;
    bg.w = (1.0f - t) * 1.f + t * 1.f;
  }
  ray.missColor = bg;
  state.throughput = toh(V3<float>(1.f));
}

// The iso-surface's isProg (MCAccelerator.h:338-567) from the box test on:
// its random stream Random2(ray.rngSeed, hash(instance, 0, 0)) -- which
// advances ray.rngSeed -- the hit search on [0, ray.tMax], the opacity test
// (a material of opacity < 1 lets the ray through when rng() > opacity) and
// DeviceMaterial::setHit (DeviceMaterial.h:70-78): Ray::setHit stores P, the
// unit normal in half precision, t and the Lambertian.
inline void iso_hit_record(const Field &F, const int M[3], V3<float> mcOrigin, V3<float> mcSpacing,
                           const float *ranges, float iso, float delta, uint64_t isoHash, float alpha, Ray &ray) {
  V3<float> dirf = ray.dir;
  if (dirf.x == 0.f) dirf.x = 1e-6f;
  if (dirf.y == 0.f) dirf.y = 1e-6f;
  if (dirf.z == 0.f) dirf.z = 1e-6f;
  uint64_t isoRng = 0;  // the geometry's Random2, made at the box test
  float t;
  V3<float> P, N;
  if (!iso_isprog(F, M, mcOrigin, mcSpacing, ranges, iso, delta, ray.org, dirf, ray.tMax, t, P, N,
                  [&]() { isoRng = Random2(ray.rngSeed, isoHash).state; }))
    return;
  if (alpha < 1.f) {
    Random2 rng(Random2::Resume{}, isoRng);
    if (rng() > alpha) return;
  }
  ray.hit = true;
  ray.surf = true;
  ray.tMax = t;
  ray.P = P;
  ray.N = toh(N);
}
inline void trace_iso(const Scene &S, Ray &ray) {
  iso_hit_record(S.F, S.M, S.mcOrigin, S.mcSpacing, S.isoRanges.data(), S.isoValue, S.isoDelta, S.isoHash,
                 S.isoAlpha, ray);
}

// trace + setVolumeHit (Ray.h:118-149): albedo = 0.7*rgb (default build) or
// scatteringAlbedo*rgb with the volume's anisotropy (multi-scatter build).
// With an iso-surface the world's two instances run in ascending instance
// order, each bounded by the other's hit (ray.tMax), so the closest hit
// stays; the order decides which one's random stream comes from the seed
// first.  (The reference leaves the order of two instances with the same
// bounds to embree's traversal.)
template <typename R> inline void trace_volume(const Scene &S, Ray &ray, Counters &cnt);
template <typename R> inline void trace_and_record(const Scene &S, Ray &ray, Counters &cnt) {
  if (!S.iso) {
    trace_volume<R>(S, ray, cnt);
    return;
  }
  if (S.noVolume) {
    cnt.rays++;
    trace_iso(S, ray);
  } else if (S.isoFirst) {
    trace_iso(S, ray);
    trace_volume<R>(S, ray, cnt);
  } else {
    trace_volume<R>(S, ray, cnt);
    trace_iso(S, ray);
  }
}
template <typename R> inline void trace_volume(const Scene &S, Ray &ray, Counters &cnt) {
  R t;
  V3<R> rgb;
  if (trace<R>(S, ray, cnt, t, rgb)) {
    V3<float> dirf = ray.dir;
    if (dirf.x == 0.f) dirf.x = 1e-6f;
    if (dirf.y == 0.f) dirf.y = 1e-6f;
    if (dirf.z == 0.f) dirf.z = 1e-6f;
    float tf = (float)t;
    V3<float> rgbf((float)rgb.x, (float)rgb.y, (float)rgb.z);
    ray.P = cvt<float>(cvt<R>(ray.org) + t * cvt<R>(dirf));
    ray.tMax = tf;
    ray.hit = true;
    ray.surf = false;
    if (S.multi) {
      ray.albedo = S.scatAlb * rgbf;
      ray.g = S.aniso;
    } else {
      ray.albedo = .7f * rgbf;
      ray.g = 0.f;
    }
  }
}

// One accumulation pass (one value of accumID) for one pixel, following
// Context::renderTiles (Context.cpp:142-185) and _shadeRays' accumulation
// (shadeRays.cu:970-1038).  Within a generation the pixel's shadow ray is
// accumulated before its bounce ray.
template <typename R> inline void render_pixel(const Scene &S, int ix, int iy, int accumID, float *acc,
                                               Counters &cnt) {
  Ray ray;
  PathState state;
  generate(S, ix, iy, accumID, ray, state);
  bool rayAlive = true;
  Ray sray;
  PathState sstate;
  bool sValid = false;
  const float clampMax = 10.f * (1 + accumID);
  for (int gen = 0; rayAlive || sValid; gen++) {
    Ray nsray;
    PathState nsstate;
    bool nsValid = false;
    if (sValid) {
      trace_and_record<R>(S, sray, cnt);
      Ray dummy;
      PathState dstate;
      bool dv;
      V3<float> frag = bounce(S, sray, sstate, dummy, dstate, dv, gen);
      frag = vmin(frag, V3<float>(clampMax));
      if (frag.x > 0.f) acc[0] += frag.x;
      if (frag.y > 0.f) acc[1] += frag.y;
      if (frag.z > 0.f) acc[2] += frag.z;
      sValid = false;
    }
    if (rayAlive) {
      trace_and_record<R>(S, ray, cnt);
      float alpha = (gen == 0) ? (ray.hit ? 1.f : ray.missColor.w) : 0.f;
      if (gen == 0) {
        // the aux tiles (shadeRays.cu:923, 1003-1023): incomingZ = ray.tMax;
        // the closest hit's IDs, primID 0 of the one-primitive user geometry
        const size_t px = (size_t)iy * S.W + ix;
        const float z = ray.tMax;
        if (accumID == 0) {
          if (S.auxDepth) S.auxDepth[px] = z;
          if (S.auxPrim) S.auxPrim[px] = ray.hit ? 0 : -1;
          if (S.auxInst) S.auxInst[px] = !ray.hit ? -1 : ray.surf ? S.isoInst : S.volInst;
          if (S.auxObj) S.auxObj[px] = !ray.hit ? -1 : ray.surf ? S.isoUser : S.volUser;
        } else if (S.auxDepth && z < S.auxDepth[px]) {
          S.auxDepth[px] = z;
        }
      }
      V3<float> frag = bounce(S, ray, state, nsray, nsstate, nsValid, gen);
      frag = vmin(frag, V3<float>(clampMax));
      if (accumID == 0 && gen == 0) {
        acc[0] = frag.x;
        acc[1] = frag.y;
        acc[2] = frag.z;
        acc[3] = alpha;
      } else {
        if (gen == 0 && alpha > 0.f) acc[3] += alpha;
        if (frag.x > 0.f) acc[0] += frag.x;
        if (frag.y > 0.f) acc[1] += frag.y;
        if (frag.z > 0.f) acc[2] += frag.z;
      }
      rayAlive = ray.tMax > 0.f;
    }
    if (nsValid && nsray.tMax > 0.f) {
      sray = nsray;
      sstate = nsstate;
      sValid = true;
    }
  }
}

}  // namespace orc

using namespace orc;

// ===========================================================================
// C interface
// ===========================================================================
extern "C" {

void orc_rng_sequence(uint32_t a, uint32_t b, int n, float *out) {
  Random2 r(a, b);
  for (int i = 0; i < n; i++) out[i] = r();
}

void orc_rng_from_seed(uint64_t seed_state, uint64_t hash, int use_u64, int n, float *out,
                       uint64_t *new_seed_state) {
  // the 32-bit constructor takes the hash's low 32 bits
  RNGSeed s;
  s.state = seed_state;
  Random2 r(s, use_u64 ? hash : (uint64_t)(uint32_t)hash);
  for (int i = 0; i < n; i++) out[i] = r();
  if (new_seed_state) *new_seed_state = s.state;
}

uint64_t orc_rng_seed_state(uint32_t a, uint32_t b) {
  RNGSeed s;
  rng_seed(s, a, b);
  return s.state;
}
uint64_t orc_hash3(uint32_t a, uint32_t b, uint32_t c) { return fnv_hash3(a, b, c); }

float orc_fast_log(float f) { return fastLog(f); }
uint16_t orc_float_to_half(float f) { return f2h(f); }
float orc_half_to_float(uint16_t h) { return h2f(h); }

void orc_sample_points(const orc_scene *s, const float *P, int n, float *out) {
  Field F = make_field(s);
  std::vector<float> lohi;
  if (s->u8_scaled) u8_build(F, lohi);
  for (int i = 0; i < n; i++)
    out[i] = sample_field<float>(F, V3<float>(P[3 * i], P[3 * i + 1], P[3 * i + 2]));
}

void orc_tf_map(const orc_scene *s, const float *scalars, int n, float *rgba) {
  XF xf = make_xf(s->tf, s->tf_n, s->domain[0], s->domain[1], s->base_density);
  for (int i = 0; i < n; i++) {
    V4<float> r = xf_map<float>(xf, scalars[i]);
    rgba[4 * i + 0] = r.x;
    rgba[4 * i + 1] = r.y;
    rgba[4 * i + 2] = r.z;
    rgba[4 * i + 3] = r.w;
  }
}

extern "C" void orc_bounded_sincos(const float *x, long long n, float *sn, float *cs) {
  for (long long i = 0; i < n; i++) bounded_sincos(x[i], sn[i], cs[i]);
}
extern "C" void orc_bounded_angles(const float *y, const float *x, long long n, float *acos_x, float *atan2_yx) {
  for (long long i = 0; i < n; i++) {
    acos_x[i] = bounded_acos(x[i]);
    atan2_yx[i] = bounded_atan2(y[i], x[i]);
  }
}

void orc_mc_dims(const int dims[3], int cells_per_mc, int mc_dims[3]) { mc_dims_of(dims, cells_per_mc, mc_dims); }

void orc_mc_ranges(const float *scalars, const int dims[3], int cpm, float *ranges) {
  int M[3];
  mc_dims_of(dims, cpm, M);
  int64_t n = (int64_t)M[0] * M[1] * M[2];
  parallel_for(n, 0, [&](int64_t tid) {
    int x = int(tid % M[0]), y = int((tid / M[0]) % M[1]), z = int(tid / ((int64_t)M[0] * M[1]));
    float lo, hi;
    mc_range_one(scalars, dims, cpm, x, y, z, lo, hi);
    ranges[2 * tid] = lo;
    ranges[2 * tid + 1] = hi;
  }, 64);
}

void orc_scene_mc_grid(const orc_scene *s, int mc_dims[3], float world[6]) {
  Field F = make_field(s);
  if (F.isNvdb) {
    for (int i = 0; i < 3; i++) {
      mc_dims[i] = F.nv.M[i];
      world[i] = F.boundsLo[i];
      world[3 + i] = F.boundsHi[i];
    }
    return;
  }
  mc_dims_of(F.N, s->cells_per_mc, mc_dims);
  for (int i = 0; i < 3; i++) {
    world[i] = F.boundsLo[i];
    world[3 + i] = F.boundsHi[i];
  }
}

void orc_scene_mc_ranges(const orc_scene *s, float *ranges) {
  Field F = make_field(s);
  if (F.isNvdb) {
    nv_mc_ranges(F.nv, ranges);
    return;
  }
  int M[3];
  mc_dims_of(F.N, s->cells_per_mc, M);
  if (!s->u8_scaled) {
    orc_mc_ranges(s->scalars, s->dims, s->cells_per_mc, ranges);
    return;
  }
  std::vector<float> lohi;
  u8_build(F, lohi);
  u8_mc_ranges(F, s->cells_per_mc, M, ranges);
}

void orc_majorants(const float *ranges, int num_mc, const float *tf, int tf_n, float lo, float hi,
                   float base_density, float *out) {
  XF xf = make_xf(tf, tf_n, lo, hi, base_density);
  for (int i = 0; i < num_mc; i++) out[i] = xf_majorant(xf, ranges[2 * i], ranges[2 * i + 1]);
}

int orc_trace_ray(const orc_scene *s, const float org[3], const float dir[3], float tmax, uint64_t *seed_state,
                  float *t_hit, float rgb[3]) {
  Scene S;
  build_scene(s, S);
  Ray ray;
  ray.org = V3<float>(org[0], org[1], org[2]);
  ray.dir = V3<float>(dir[0], dir[1], dir[2]);
  ray.tMax = tmax;
  ray.rngSeed.state = *seed_state;
  Counters c;
  float t = 0.f;
  V3<float> c3;
  bool h = trace<float>(S, ray, c, t, c3);
  *seed_state = ray.rngSeed.state;
  if (h) {
    *t_hit = t;
    rgb[0] = c3.x;
    rgb[1] = c3.y;
    rgb[2] = c3.z;
  }
  return h ? 1 : 0;
}

// MCIsoSurfaceAccel::isProg (barney/volume/MCAccelerator.h:338-567) over
// dda::dda3 (DDA.h:65-206), as the embree backend dispatches it (tmin 0,
// tmax ray.tMax, identity instance).  The trace direction has zero
// components replaced by 1e-6 (traceRays.dev.cu:41-44).  Per macrocell whose
// scalar range holds the iso value, the cell's t range is cut into 10
// sub-steps; the first sub-step whose end values bracket the iso value gives
// t by linear interpolation.  The normal is the central difference of the
// field at +-delta per axis (a one-sided difference where a sample falls
// outside the field).  out: t, P[3], N[3] (N normalized).
int orc_iso_intersect(const orc_scene *s, const float *ranges, float iso, const float org_[3], const float dir_[3],
                      float tmax, float out[7]) {
  Field F = make_field(s);
  std::vector<float> lohi;
  if (s->u8_scaled) u8_build(F, lohi);
  int M[3];
  mc_dims_of(F.N, s->cells_per_mc, M);
  std::vector<float> own;
  if (!ranges && M[0] > 0 && M[1] > 0 && M[2] > 0) {
    own.resize((size_t)2 * M[0] * M[1] * M[2]);
    orc_scene_mc_ranges(s, own.data());
    ranges = own.data();
  }
  V3<float> dir(dir_[0], dir_[1], dir_[2]);
  if (dir.x == 0.f) dir.x = 1e-6f;
  if (dir.y == 0.f) dir.y = 1e-6f;
  if (dir.z == 0.f) dir.z = 1e-6f;
  const V3<float> mcSpacing = V3<float>((float)s->cells_per_mc) * F.spacing;
  const float delta = length(F.boundsHi - F.boundsLo) * .1f / float(M[0] + M[1] + M[2]);
  float t;
  V3<float> P, N;
  if (!iso_isprog(F, M, F.boundsLo, mcSpacing, ranges, iso, delta, V3<float>(org_[0], org_[1], org_[2]), dir, tmax,
                  t, P, N, []() {}))
    return 0;
  out[0] = t;
  out[1] = P.x; out[2] = P.y; out[3] = P.z;
  out[4] = N.x; out[5] = N.y; out[6] = N.z;
  return 1;
}

// The iso-surface isProg with an AnariMatte material of constant color and
// opacity, as ref_iso_hit exposes the reference's: returns 1 on a hit with t,
// P, the normal's three halfs and the Lambertian's albedo (xyz) and alpha
// (w); *seed_state carries the ray's seed in and out.
int orc_iso_hit(const orc_scene *s, const float *ranges, float iso, const float color[4], float opacity, int inst,
                const float org[3], const float dir[3], float tmax, uint64_t *seed_state, float *t_hit, float P[3],
                uint16_t N[3], float albedo[4]) {
  Field F = make_field(s);
  std::vector<float> lohi;
  if (s->u8_scaled) u8_build(F, lohi);
  int M[3];
  mc_dims_of(F.N, s->cells_per_mc, M);
  const V3<float> mcSpacing = V3<float>((float)s->cells_per_mc) * F.spacing;
  const float delta = length(F.boundsHi - F.boundsLo) * .1f / float(M[0] + M[1] + M[2]);
  V4<float> base{color[0], color[1], color[2], color[3]};
  if (std::isnan(base.x)) base = {0.f, 0.f, 0.f, 1.f};
  const float op = std::isnan(opacity) ? 0.f : opacity;
  Ray ray;
  ray.org = V3<float>(org[0], org[1], org[2]);
  ray.dir = V3<float>(dir[0], dir[1], dir[2]);
  ray.tMax = tmax;
  ray.rngSeed.state = *seed_state;
  ray.hit = ray.surf = false;
  iso_hit_record(F, M, F.boundsLo, mcSpacing, ranges, iso, delta, fnv_hash3((uint32_t)inst, 0, 0), base.w * op, ray);
  *seed_state = ray.rngSeed.state;
  if (!ray.hit) return 0;
  const V3<float> alb = .85f * V3<float>(base.x, base.y, base.z) * ONE_OVER_PI;
  *t_hit = ray.tMax;
  P[0] = ray.P.x; P[1] = ray.P.y; P[2] = ray.P.z;
  N[0] = ray.N.x; N[1] = ray.N.y; N[2] = ray.N.z;
  albedo[0] = alb.x; albedo[1] = alb.y; albedo[2] = alb.z;
  albedo[3] = base.w * op;
  return 1;
}

// The AnariMatte Lambertian at a surface of normal Ng seen from wo, as
// ref_lambertian exposes the reference's: eval and pdf toward wi, then one
// scatter drawing from Random2(a, b) (libm sine and cosine).  out: eval
// value[3], eval pdf, pdf(wi), scatter dir[3], scatter pdf, f_r[3].
void orc_lambertian(const float color[4], const float Ng_[3], const float wo_[3], const float wi_[3], uint32_t a,
                    uint32_t b, float out[12]) {
  V4<float> base{color[0], color[1], color[2], color[3]};
  if (std::isnan(base.x)) base = {0.f, 0.f, 0.f, 1.f};
  const V3<float> albedo = .85f * V3<float>(base.x, base.y, base.z) * ONE_OVER_PI;
  const V3<float> Ng(Ng_[0], Ng_[1], Ng_[2]), wo(wo_[0], wo_[1], wo_[2]), wi(wi_[0], wi_[1], wi_[2]);
  const float cosThetaI = mx(dot(wi, Ng), 0.f);
  const V3<float> v = albedo * ONE_OVER_PI * cosThetaI;
  out[0] = v.x; out[1] = v.y; out[2] = v.z;
  out[3] = cosThetaI * ONE_OVER_PI;
  out[4] = lambert_pdf(Ng, wi);
  Random2 random(a, b);
  V3<float> N = Ng;
  if (dot(wo, N) < 0.f) N = -N;
  const float r0 = random();
  const float r1 = random();
  const float sx = r1, sy = r0;
  const float phi = TWO_PI * sx;
  const float cosTheta = std::sqrt(sy);
  const float sinTheta = std::sqrt(1.0f - sy);
  float sinPhi, cosPhi;
  path_sincos(false, phi, sinPhi, cosPhi);
  const V3<float> local(cosPhi * sinTheta, sinPhi * sinTheta, cosTheta);
  V3<float> dx, dy;
  frame_of(N, dx, dy);
  const V3<float> d = dx * local.x + dy * local.y + N * local.z;
  out[5] = d.x; out[6] = d.y; out[7] = d.z;
  out[8] = local.z * ONE_OVER_PI;
  out[9] = albedo.x; out[10] = albedo.y; out[11] = albedo.z;
}

// bounce() on a world and path given as DD-level records (the reference
// pin's ref_bounce takes the same), for the shading pin tests.
void orc_bounce(const orc_shade_world *w, int multi, int depth, orc_shade_path *io, orc_shade_path *sh,
                float fragment[3]) {
  Scene S;
  S.numDir = std::min(4, std::max(0, w->num_dir_lights));
  for (int i = 0; i < S.numDir; i++) {
    S.dir[i].direction = V3<float>(w->dir_light_dir[i][0], w->dir_light_dir[i][1], w->dir_light_dir[i][2]);
    S.dir[i].color = V3<float>(w->dir_light_color[i][0], w->dir_light_color[i][1], w->dir_light_color[i][2]);
    S.dir[i].radiance = w->dir_light_radiance[i];
  }
  S.env.boundedMath = false;
  if (w->env_texels) {
    Env &e = S.env;
    e.present = true;
    e.tex = w->env_texels;
    e.W = w->env_dims[0];
    e.H = w->env_dims[1];
    e.addr[0] = w->env_addr[0];
    e.addr[1] = w->env_addr[1];
    e.scale = w->env_scale;
    const float *a = w->env_to_world, *b = w->env_to_local;
    e.toWorld.vx = V3<float>(a[0], a[1], a[2]);
    e.toWorld.vy = V3<float>(a[3], a[4], a[5]);
    e.toWorld.vz = V3<float>(a[6], a[7], a[8]);
    e.toLocal.vx = V3<float>(b[0], b[1], b[2]);
    e.toLocal.vy = V3<float>(b[3], b[4], b[5]);
    e.toLocal.vz = V3<float>(b[6], b[7], b[8]);
    e.cdf_y.assign(w->env_cdf_y, w->env_cdf_y + e.H);
    e.cdf_x.assign(w->env_cdf_x, w->env_cdf_x + (size_t)e.W * e.H);
  }
  S.ambient = w->ambient_radiance;
  S.multi = multi;
  S.volMS = w->volume_multi_scatter;
  S.maxVB = w->max_volume_bounces;
  Ray ray;
  ray.org = V3<float>(io->org[0], io->org[1], io->org[2]);
  ray.dir = V3<float>(io->dir[0], io->dir[1], io->dir[2]);
  ray.tMax = io->tmax;
  ray.rngSeed.state = io->seed;
  ray.P = V3<float>(io->P[0], io->P[1], io->P[2]);
  ray.hit = io->hit != 0;
  ray.surf = io->hit == 2;
  ray.isShadowRay = io->shadow != 0;
  ray.missColor = {io->miss_color[0], io->miss_color[1], io->miss_color[2], io->miss_color[3]};
  ray.g = 0.f;
  const V3<float> rgb(io->rgb[0], io->rgb[1], io->rgb[2]);
  if (io->hit == 1) {
    ray.albedo = multi ? io->scattering_albedo * rgb : .7f * rgb;  // Phase(color) (Phase.h:40-46, 121-129)
    ray.g = multi ? io->g : 0.f;
  } else if (io->hit == 2) {
    V4<float> base{io->color[0], io->color[1], io->color[2], io->color[3]};
    if (std::isnan(base.x)) base = {0.f, 0.f, 0.f, 1.f};
    S.isoAlbedo = .85f * V3<float>(base.x, base.y, base.z) * ONE_OVER_PI;
    S.isoAlpha = base.w * (std::isnan(io->opacity) ? 0.f : io->opacity);
    ray.N = toh(V3<float>(io->N[0], io->N[1], io->N[2]));
  }
  PathState st;
  st.throughput = {io->tp[0], io->tp[1], io->tp[2]};
  st.misWeight = io->mis;
  st.numDiffuseBounces = io->diffuse_bounces;
  st.numVolumeBounces = io->volume_bounces;
  Ray sray;
  PathState sst;
  bool sValid = false;
  const V3<float> f = bounce(S, ray, st, sray, sst, sValid, depth);
  fragment[0] = f.x; fragment[1] = f.y; fragment[2] = f.z;
  for (int a = 0; a < 3; a++) {
    io->org[a] = ray.org[a];
    io->dir[a] = ray.dir[a];
  }
  io->tmax = ray.tMax;
  io->seed = ray.rngSeed.state;
  io->hit = ray.hit ? (ray.surf ? 2 : 1) : 0;
  io->tp[0] = st.throughput.x; io->tp[1] = st.throughput.y; io->tp[2] = st.throughput.z;
  io->mis = st.misWeight;
  io->diffuse_bounces = st.numDiffuseBounces;
  io->volume_bounces = st.numVolumeBounces;
  std::memset(sh, 0, sizeof(*sh));
  sh->tmax = -1.f;
  if (sValid) {
    for (int a = 0; a < 3; a++) {
      sh->org[a] = sray.org[a];
      sh->dir[a] = sray.dir[a];
    }
    sh->tmax = sray.tMax;
    sh->seed = sray.rngSeed.state;
    sh->shadow = 1;
    sh->tp[0] = sst.throughput.x; sh->tp[1] = sst.throughput.y; sh->tp[2] = sst.throughput.z;
    sh->mis = sst.misWeight;
  }
}

// PerspectiveCamera::commit for these parameters: dir_00, dir_du, dir_dv,
// lens_00 (12 floats), as ref_camera_commit exposes the reference's
void orc_camera_commit(const float pos[3], const float dir[3], const float up[3], float fovy, float out[12]) {
  const Camera c = commit_camera(pos, dir, up, fovy);
  const V3<float> v[4] = {c.dir00, c.du, c.dv, c.lens00};
  for (int i = 0; i < 4; i++)
    for (int a = 0; a < 3; a++) out[3 * i + a] = v[i][a];
}

// _generateRays for pass accumID of a W x H frame, as ref_generate exposes
// the reference's: per pixel (row-major) org[3], dir[3], tMax, missColor[4]
// and the ray's seed state; returns the count of pixels whose path state is
// not throughput 1, misWeight 0 (none)
int orc_generate(const float pos[3], const float dir[3], const float up[3], float fovy, int W, int H, int accumID,
                 const float bg[4], float *out, uint64_t *seeds) {
  Scene S;
  S.cam = commit_camera(pos, dir, up, fovy);
  S.W = W;
  S.H = H;
  S.bg = {bg[0], bg[1], bg[2], bg[3]};
  int bad = 0;
  for (int iy = 0; iy < H; iy++)
    for (int ix = 0; ix < W; ix++) {
      Ray ray;
      PathState st;
      generate(S, ix, iy, accumID, ray, st);
      float *o = out + 11 * ((size_t)iy * W + ix);
      for (int a = 0; a < 3; a++) {
        o[a] = ray.org[a];
        o[3 + a] = ray.dir[a];
      }
      o[6] = ray.tMax;
      o[7] = ray.missColor.x; o[8] = ray.missColor.y; o[9] = ray.missColor.z; o[10] = ray.missColor.w;
      seeds[(size_t)iy * W + ix] = ray.rngSeed.state;
      if (st.throughput.x != 0x3c00 || st.throughput.y != 0x3c00 || st.throughput.z != 0x3c00 || st.misWeight != 0.f)
        bad++;
    }
  return bad;
}

void orc_render(const orc_scene *s, float *accum, int accum_id_start, int spp, int use_double, int nthreads,
                int row0, int row1, orc_stats *stats) {
  Scene S;
  build_scene(s, S);
  if (row1 <= 0 || row1 > S.H) row1 = S.H;
  if (row0 < 0) row0 = 0;
  const int W = S.W;
  int64_t n = (int64_t)(row1 - row0) * W;
  std::atomic<uint64_t> ns{0}, nm{0}, nr{0};
  parallel_for(n, nthreads, [&](int64_t i) {
    int ix = int(i % W), iy = row0 + int(i / W);
    float *acc = accum + 4 * ((size_t)iy * W + ix);
    Counters c;
    for (int p = 0; p < spp; p++) {
      if (use_double) render_pixel<double>(S, ix, iy, accum_id_start + p, acc, c);
      else render_pixel<float>(S, ix, iy, accum_id_start + p, acc, c);
    }
    ns += c.samples;
    nm += c.mcs;
    nr += c.rays;
  }, 16);
  if (stats) {
    stats->density_samples = ns;
    stats->mc_visits = nm;
    stats->rays = nr;
  }
}

// TiledFB.cu:13-50, LocalFB.cpp:60-70 (accumScale = 1/accumID), math.h:52-116
void orc_tonemap(const float *accum, int W, int H, int accum_id, int format, void *out) {
  float accumScale = 1.f / accum_id;
  auto make_8bit = [](float f) -> uint32_t { return (uint32_t)mn(255, mx(0, int(f * 256.f))); };
  auto srgb = [](float x) -> float {
    if (x <= 0.0031308f) return 12.92f * x;
    return 1.055f * powf(x, 1.f / 2.4f) - 0.055f;
  };
  for (int64_t i = 0; i < (int64_t)W * H; i++) {
    float c[4];
    for (int k = 0; k < 4; k++) c[k] = accum[4 * i + k] * accumScale;
    if (format == 0) {
      for (int k = 0; k < 4; k++) ((float *)out)[4 * i + k] = c[k];
    } else {
      if (format == 2) for (int k = 0; k < 3; k++) c[k] = srgb(c[k]);
      ((uint32_t *)out)[i] = (make_8bit(c[0]) << 0) + (make_8bit(c[1]) << 8) + (make_8bit(c[2]) << 16) +
                             (make_8bit(c[3]) << 24);
    }
  }
}

void orc_env_cdfs(const float *texels, const int dims[2], const int addr[2], float *cdf_y, float *cdf_x) {
  env_cdfs(texels, dims[0], dims[1], addr, cdf_y, cdf_x);
}

}  // extern "C"

// ===========================================================================
// Fixed-step emission-absorption march (project-defined form; the reference
// has only delta tracking).  Semantics shared with the CUDA product:
//   * camera: the perspective camera above at the pixel centre (the
//     accumID == 0 ray of _generateRays);
//   * [t0,t1] from boxTest against the field's world bounds, tmin 0, tmax 1e30;
//   * n = ceil((t1-t0)/dt) steps; step i samples at t = t0+(i+.5)*dt and is
//     skipped once t >= t1; every step covers a length dt;
//   * sampleAndMap gives (rgb, sigma) (sigma already times densityAt1);
//     x_i = sigma_i*dt, alpha_i = -expm1(-x_i), T_i = exp(-tau_i) with
//     tau_i = sum_{k<i} x_k (compensated sum);
//   * C = sum_i T_i*alpha_i*rgb_i, A = -expm1(-tau_n); pixel = (C, A).
// The adjoint uses dC/dx_j = rgb_j*T_{j+1} - (C - C_{<=j}), dA/dx_j = T_n,
// dC/drgb_j = T_j*alpha_j: a front-to-back replay that stores no per-step
// state.
// ===========================================================================
namespace orc {

struct EAView { Camera cam; int W, H; };

template <typename R> struct EAStep {
  R t0, t1, dt;
  int n;
};

template <typename R>
inline bool ea_setup(const Field &F, const EAView &v, int ix, int iy, R step, V3<R> &org, V3<R> &dir, EAStep<R> &st) {
  float image_u = ((ix + .5f) / float(v.W));
  float image_v = ((iy + .5f) / float(v.H));
  float aspect = v.W / float(v.H);
  V3<float> d = v.cam.dir00 + (1.f * aspect * (image_u - .5f)) * v.cam.du + (1.f * (image_v - .5f)) * v.cam.dv;
  d = normalize(d);
  org = cvt<R>(v.cam.lens00);
  dir = cvt<R>(d);
  R t0 = R(0), t1 = R(1e30f);
  if (!boxTest<R>(org, dir, t0, t1, cvt<R>(F.boundsLo), cvt<R>(F.boundsHi))) return false;
  if (!(t1 > t0)) return false;
  st.t0 = t0;
  st.t1 = t1;
  st.dt = step;
  st.n = (int)std::ceil((t1 - t0) / step);
  return true;
}

template <typename R>
inline void ea_forward_pixel(const Field &F, const XF &xf, const EAView &v, int ix, int iy, R step, R out[4]) {
  out[0] = out[1] = out[2] = out[3] = R(0);
  V3<R> org, dir;
  EAStep<R> st;
  if (!ea_setup<R>(F, v, ix, iy, step, org, dir, st)) return;
  R tau = 0, comp = 0;  // Neumaier-compensated optical depth
  R C[3] = {0, 0, 0};
  for (int i = 0; i < st.n; i++) {
    R t = st.t0 + (R(i) + R(.5)) * st.dt;
    if (t >= st.t1) break;
    V3<R> P = org + t * dir;
    V4<R> smp = sample_and_map<R>(F, xf, P);
    R x = smp.w * st.dt;
    R T = std::exp(-(tau + comp));
    R alpha = -std::expm1(-x);
    R w = T * alpha;
    C[0] += w * smp.x;
    C[1] += w * smp.y;
    C[2] += w * smp.z;
    R tnew = tau + x;
    if (std::fabs(tau) >= std::fabs(x)) comp += (tau - tnew) + x;
    else comp += (x - tnew) + tau;
    tau = tnew;
  }
  out[0] = C[0];
  out[1] = C[1];
  out[2] = C[2];
  out[3] = -std::expm1(-(tau + comp));
}

inline void ea_backward_pixel(const Field &F, const XF &xf, const EAView &v, int ix, int iy, double step,
                              const float g[4], double *d_vox, double *d_tf) {
  V3<double> org, dir;
  EAStep<double> st;
  if (!ea_setup<double>(F, v, ix, iy, step, org, dir, st)) return;
  double Cfin[4];
  ea_forward_pixel<double>(F, xf, v, ix, iy, step, Cfin);
  const double Tn = 1.0 - Cfin[3];
  double tau = 0, comp = 0;
  double Cacc[3] = {0, 0, 0};
  const double gs = double(xf.n - 1) / double(xf.span);
  const size_t Nx = F.N[0], Ny = F.N[1];
  for (int i = 0; i < st.n; i++) {
    double t = st.t0 + (double(i) + .5) * st.dt;
    if (t >= st.t1) break;
    V3<double> P = org + t * dir;
    Tri tri{};
    double s = sample_field<double>(F, P, &tri);
    if (std::isnan(s)) continue;  // sampleAndMap -> 0: no dependence
    int idx;
    double f;
    bool clamped;
    V4<double> m = xf_map<double>(xf, s, &idx, &f, &clamped);
    double x = m.w * st.dt;
    double T = std::exp(-(tau + comp));
    double alpha = -std::expm1(-x);
    double w = T * alpha;
    Cacc[0] += w * m.x;
    Cacc[1] += w * m.y;
    Cacc[2] += w * m.z;
    double tnew = tau + x;
    if (std::fabs(tau) >= std::fabs(x)) comp += (tau - tnew) + x;
    else comp += (x - tnew) + tau;
    tau = tnew;
    double Tnext = std::exp(-(tau + comp));
    // dL/dx
    double dLdx = g[3] * Tn;
    double rgb[3] = {m.x, m.y, m.z};
    for (int c = 0; c < 3; c++) dLdx += g[c] * (rgb[c] * Tnext - (Cfin[c] - Cacc[c]));
    double dLdsigma = dLdx * st.dt;        // sigma = w_tf * baseDensity
    double dLdrgb[3];
    for (int c = 0; c < 3; c++) dLdrgb[c] = g[c] * w;
    // transfer-function entries
    const float *v0 = xf.v + 4 * idx, *v1 = xf.v + 4 * (idx + 1);
    double bd = xf.baseDensity;
    for (int c = 0; c < 3; c++) {
      d_tf[4 * idx + c] += dLdrgb[c] * (1.0 - f);
      d_tf[4 * (idx + 1) + c] += dLdrgb[c] * f;
    }
    d_tf[4 * idx + 3] += dLdsigma * bd * (1.0 - f);
    d_tf[4 * (idx + 1) + 3] += dLdsigma * bd * f;
    // scalar
    if (clamped) continue;
    double dLds = dLdsigma * bd * (double(v1[3]) - double(v0[3])) * gs;
    for (int c = 0; c < 3; c++) dLds += dLdrgb[c] * (double(v1[c]) - double(v0[c])) * gs;
    double wx[2] = {1.0 - tri.fx, tri.fx}, wy[2] = {1.0 - tri.fy, tri.fy}, wz[2] = {1.0 - tri.fz, tri.fz};
    for (int kz = 0; kz < 2; kz++)
      for (int ky = 0; ky < 2; ky++)
        for (int kx = 0; kx < 2; kx++) {
          size_t vi = tri.ix[kx] + Nx * (tri.iy[ky] + Ny * (size_t)tri.iz[kz]);
          d_vox[vi] += dLds * wx[kx] * wy[ky] * wz[kz];
        }
  }
}

}  // namespace orc

extern "C" {

void orc_ea_render(const orc_scene *s, const orc_ea_view *views, int num_views, float step, int use_double,
                   int nthreads, float *images) {
  Field F = make_field(s);
  std::vector<float> lohi;
  if (s->u8_scaled) u8_build(F, lohi);
  XF xf = make_xf(s->tf, s->tf_n, s->domain[0], s->domain[1], s->base_density);
  size_t off = 0;
  for (int vi = 0; vi < num_views; vi++) {
    EAView v{commit_camera(views[vi].pos, views[vi].dir, views[vi].up, views[vi].fovy), views[vi].width,
             views[vi].height};
    float *img = images + off;
    parallel_for((int64_t)v.W * v.H, nthreads, [&](int64_t i) {
      int ix = int(i % v.W), iy = int(i / v.W);
      if (use_double) {
        double o[4];
        ea_forward_pixel<double>(F, xf, v, ix, iy, (double)step, o);
        for (int k = 0; k < 4; k++) img[4 * i + k] = (float)o[k];
      } else {
        float o[4];
        ea_forward_pixel<float>(F, xf, v, ix, iy, step, o);
        for (int k = 0; k < 4; k++) img[4 * i + k] = o[k];
      }
    }, 64);
    off += (size_t)4 * v.W * v.H;
  }
}

void orc_ea_backward(const orc_scene *s, const orc_ea_view *views, int num_views, float step, const float *d_images,
                     int nthreads, double *d_scalars, double *d_tf) {
  Field F = make_field(s);
  XF xf = make_xf(s->tf, s->tf_n, s->domain[0], s->domain[1], s->base_density);
  size_t nvox = (size_t)s->dims[0] * s->dims[1] * s->dims[2];
  int nt = nthreads > 0 ? nthreads : (int)std::max(1u, std::thread::hardware_concurrency());
  // per-thread privatised gradients, reduced at the end (deterministic order)
  std::vector<std::vector<double>> gv(nt, std::vector<double>(nvox, 0.0));
  std::vector<std::vector<double>> gt(nt, std::vector<double>((size_t)4 * s->tf_n, 0.0));
  size_t off = 0;
  for (int vi = 0; vi < num_views; vi++) {
    EAView v{commit_camera(views[vi].pos, views[vi].dir, views[vi].up, views[vi].fovy), views[vi].width,
             views[vi].height};
    const float *g = d_images + off;
    int64_t npx = (int64_t)v.W * v.H;
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; t++)
      pool.emplace_back([&, t]() {
        for (int64_t i = t; i < npx; i += nt)
          ea_backward_pixel(F, xf, v, int(i % v.W), int(i / v.W), (double)step, g + 4 * i, gv[t].data(),
                            gt[t].data());
      });
    for (auto &th : pool) th.join();
    off += (size_t)4 * npx;
  }
  for (size_t i = 0; i < nvox; i++) {
    double a = 0;
    for (int t = 0; t < nt; t++) a += gv[t][i];
    d_scalars[i] = a;
  }
  for (size_t i = 0; i < (size_t)4 * s->tf_n; i++) {
    double a = 0;
    for (int t = 0; t < nt; t++) a += gt[t][i];
    d_tf[i] = a;
  }
}

}  // extern "C"
