// gbv_math.cuh -- host/device vector math, RNG and half conversion for the
// structured-volume path.
//
// Arithmetic follows the reference renderer's FP32 expressions operation by
// operation; translation units that include this header are compiled with
// -fmad=false (device) and -ffp-contract=off (host) so no multiply-add is
// fused and every result rounds exactly as the reference's CPU backend does.
// owl::common semantics (a third-party dependency of the reference, absent
// from its checkout) are written out here: min/max are std::min/std::max,
// clamp(v,lo,hi)=min(hi,max(lo,v)), rcp(x)=1/x, normalize(v)=v*(1/sqrt(v.v)).
#pragma once
#include <cstdint>
#include <cmath>

#if defined(__CUDACC__)
#define GBV_HD __host__ __device__ __forceinline__
#define GBV_HD_COLD static __host__ __device__ __noinline__  // rarely taken: one out-of-line copy
#else
#define GBV_HD inline
#define GBV_HD_COLD static inline
#endif

namespace gbv {

template <typename T> GBV_HD T mn(T a, T b) { return (b < a) ? b : a; }
template <typename T> GBV_HD T mx(T a, T b) { return (a < b) ? b : a; }
template <typename T> GBV_HD T clampv(T v, T lo, T hi) { return mn(hi, mx(lo, v)); }

struct vec3 {
  float x, y, z;
  GBV_HD vec3() : x(0.f), y(0.f), z(0.f) {}
  GBV_HD vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  GBV_HD explicit vec3(float a) : x(a), y(a), z(a) {}
};
GBV_HD vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
GBV_HD vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
GBV_HD vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
GBV_HD vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
GBV_HD vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
GBV_HD vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
GBV_HD vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
GBV_HD bool is_zero(vec3 a) { return a.x == 0.f && a.y == 0.f && a.z == 0.f; }
GBV_HD vec3 vmin(vec3 a, vec3 b) { return vec3(mn(a.x, b.x), mn(a.y, b.y), mn(a.z, b.z)); }
GBV_HD vec3 vmax(vec3 a, vec3 b) { return vec3(mx(a.x, b.x), mx(a.y, b.y), mx(a.z, b.z)); }
GBV_HD vec3 vabs(vec3 a) { return vec3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
GBV_HD vec3 rcp(vec3 a) { return vec3(1.f / a.x, 1.f / a.y, 1.f / a.z); }
GBV_HD vec3 vfloor(vec3 a) { return vec3(floorf(a.x), floorf(a.y), floorf(a.z)); }
GBV_HD float reduce_min(vec3 a) { return mn(mn(a.x, a.y), a.z); }
GBV_HD float reduce_max(vec3 a) { return mx(mx(a.x, a.y), a.z); }
GBV_HD float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
GBV_HD vec3 cross(vec3 a, vec3 b) {
  return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
GBV_HD vec3 normalize(vec3 v) { return v * (1.f / sqrtf(dot(v, v))); }
GBV_HD float comp(vec3 v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

struct vec4 { float x, y, z, w; };

#define GBV_INF (__int_as_float_hd(0x7f800000))
GBV_HD float __int_as_float_hd(int i) {
  union { int i; float f; } u;
  u.i = i;
  return u.f;
}
GBV_HD uint32_t float_bits(float f) {
  union { float f; uint32_t u; } u;
  u.f = f;
  return u.u;
}

constexpr float kPi = 3.14159265358979323846f;
constexpr float kTwoPi = 2.f * 3.14159265358979323846f;
constexpr float kFourPi = 4.f * 3.14159265358979323846f;
constexpr float kOneOverPi = 1.f / 3.14159265358979323846f;
constexpr float kOneOverTwoPi = 1.f / (2.f * 3.14159265358979323846f);
constexpr float kOneOverFourPi = 1.f / (4.f * 3.14159265358979323846f);

// ---------------------------------------------------------------------------
// Half precision, rounded as the reference's CPU backend rounds
// (rtcore/embree/Float16.cpp float32ToFloat16: to nearest, ties away from
// zero).  Path throughput lives in half precision (render/Ray.h:19), so the
// rounding rule is part of the path's arithmetic.
// ---------------------------------------------------------------------------
// The general conversion (every input; on the device only the values the
// short path below leaves out reach it)
GBV_HD_COLD uint16_t f2h_general(float value) {
  int i = (int)float_bits(value);
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
  }
  if (m & 0x00001000) {
    m += 0x00002000;
    if (m & 0x00800000) { m = 0; e += 1; }
  }
  if (e > 30) return uint16_t(s | 0x7c00);
  return uint16_t(s | (e << 10) | (m >> 13));
}
// On the device, values whose rounded magnitude is a normal half
// (2^-14 <= |v| < 65520) take a short path with the same result: adding half
// a unit of the 13 dropped bits to the float's bit pattern and clearing them
// rounds to nearest with ties away from zero (a carry into the exponent is
// the correct round-up), and the result is a half exactly, so the
// hardware's round-toward-zero conversion only re-encodes it.  Subnormal
// halves, overflow to infinity and NaN take the general path.
GBV_HD uint16_t f2h(float value) {
#if defined(__CUDA_ARCH__)
  const uint32_t b = float_bits(value);
  const uint32_t a = b & 0x7fffffffu;
  if (a >= 0x38800000u && a < 0x477ff000u) {
    const float r = __uint_as_float((b + 0x1000u) & ~0x1fffu);
    unsigned short h;
    asm("cvt.rz.f16.f32 %0, %1;" : "=h"(h) : "f"(r));
    return (uint16_t)h;
  }
#endif
  return f2h_general(value);
}
// exact widening (on the device the hardware conversion, which widens every
// finite and infinite half exactly; a NaN stays a NaN, and a NaN throughput
// never reaches the frame, so its payload is not observable)
GBV_HD float h2f(uint16_t h) {
#if defined(__CUDA_ARCH__)
  {
    float f;
    asm("cvt.f32.f16 %0, %1;" : "=f"(f) : "h"((unsigned short)h));
    return f;
  }
#endif
  uint32_t s = (h >> 15) & 1u, e = (h >> 10) & 0x1fu, m = h & 0x3ffu, out;
  if (e == 0) {
    if (m == 0) out = s << 31;
    else {
      while (!(m & 0x400u)) { m <<= 1; e -= 1; }
      e += 1;
      m &= ~0x400u;
      out = (s << 31) | ((e + 112u) << 23) | (m << 13);
    }
  } else if (e == 31) {
    out = (s << 31) | 0x7f800000u | (m << 13);
  } else {
    out = (s << 31) | ((e + 112u) << 23) | (m << 13);
  }
  union { uint32_t u; float f; } u;
  u.u = out;
  return u.f;
}
struct vec3h { uint16_t x, y, z; };
GBV_HD vec3h to_half(vec3 v) { return vec3h{f2h(v.x), f2h(v.y), f2h(v.z)}; }
GBV_HD vec3 from_half(vec3h v) { return vec3(h2f(v.x), h2f(v.y), h2f(v.z)); }

// ---------------------------------------------------------------------------
// RNG streams (barney/common/barney-common.h:65-152): a 64-bit multiplicative
// LCG with an xorshift output, 24-bit floats, FNV-style stream hashes.
// ---------------------------------------------------------------------------
struct RNGSeed {
  uint64_t state;
  // The output is the low word of (x ^ (x >> 22)) >> (22 + (x >> 61)).  The
  // shift is always 22..29, so on the device both shifts are 32-bit funnel
  // shifts of the state's halves (identical result, fewer instructions than
  // a general 64-bit shift).
  GBV_HD uint32_t next() {
    uint64_t x = state;
    state = x * 6364136223846793005ull;
#if defined(__CUDA_ARCH__)
    const uint32_t lo = (uint32_t)x, hi = (uint32_t)(x >> 32);
    const uint32_t ylo = lo ^ __funnelshift_r(lo, hi, 22);
    const uint32_t yhi = hi ^ (hi >> 22);
    return __funnelshift_r(ylo, yhi, 22u + (hi >> 29));
#else
    unsigned count = (unsigned)(x >> 61);
    x ^= x >> 22;
    return (uint32_t)(x >> (22 + count));
#endif
  }
  GBV_HD uint32_t next_h(uint64_t hash) {
    state ^= (hash << 1);
    return next();
  }
};
GBV_HD RNGSeed seeded(uint32_t a, uint32_t b) {
  RNGSeed r;
  r.state = 0xcafef00dd15ea5e5ull;
  r.state ^= (uint64_t)(uint32_t)(2u * a + 1u);
  r.next();
  r.state ^= (uint64_t)(uint32_t)(2u * b);
  r.next();
  return r;
}
struct Random {
  RNGSeed s;
  // Random2(RNGSeed &seed, b): copy, advance the source, then mix in b.
  GBV_HD static Random derive(RNGSeed &seed, uint64_t b) {
    Random r;
    r.s.state = seed.state;
    seed.next();
    r.s.next_h(b ? b : 290374ull);
    return r;
  }
  GBV_HD static Random from_pair(uint32_t a, uint32_t b) {
    Random r;
    r.s = seeded(a, b);
    return r;
  }
  GBV_HD float operator()() { return (s.next() & 0x00FFFFFF) * (1.f / (float)0x01000000); }
};
// hash(0,0,0): the stream id of the only instance/geometry of the world
constexpr uint64_t kFnvOffset = 0xcbf29ce484222325ull;
constexpr uint64_t kFnvPrime = 0x100000001b3ull;
constexpr uint64_t kVolumeStreamHash = ((kFnvOffset ^ (kFnvPrime * 0ull)) * kFnvPrime ^ 0ull) * kFnvPrime ^ 0ull;
// The hash a hit's distance gives the shading step's random streams
// (shadeRays.cu:610, 722: Random(ray.rngSeed, (const uint32_t&)ray.tMax) and
// ray.rngSeed.next((const uint32_t&)ray.tMax)).  A C-style cast to a const
// reference of another type is a static_cast that converts the value into a
// temporary, so the hash is the distance truncated to an integer (0 for
// t < 1, where Random2 falls back to 290374), not its bit pattern.  Hit
// distances are finite, positive and far below 2^32, where host and device
// conversions agree.
GBV_HD uint32_t hit_hash(float t) { return (uint32_t)t; }
// hash(a, b, c) (barney-common.h:132-146): the stream id of instance a,
// geometry b, primitive c
GBV_HD uint64_t fnv_hash3(uint32_t a, uint32_t b, uint32_t c) {
  return (((kFnvOffset ^ (kFnvPrime * (uint64_t)a)) * kFnvPrime ^ (uint64_t)b) * kFnvPrime) ^ (uint64_t)c;
}

// Volume.h:174-184: three-term atanh series for log
GBV_HD float fastLog(float f) {
  f = (f - 1.f) / (f + 1.f);
  float f2 = f * f;
  float s = f;
  f *= f2;
  s += (1.f / 3.f) * f;
  f *= f2;
  s += (1.f / 5.f) * f;
  return s + s;
}

GBV_HD float lerp_l(float f, float a, float b) { return (1.f - f) * a + f * b; }

// barney/common/math.h:52-116: 8-bit channel min(255, max(0, int(f * 256)))
// (a NaN converts to 0 on the device and is mapped to 0 on the host, as the
// device's conversion does) and the sRGB transfer curve
GBV_HD uint32_t make_8bit(float f) {
#if !defined(__CUDA_ARCH__)
  if (f != f) return 0u;
#endif
  const int v = (int)(f * 256.f);
  return (uint32_t)(v < 0 ? 0 : (v > 255 ? 255 : v));
}
GBV_HD float linear_to_srgb(float x) {
  if (x <= 0.0031308f) return 12.92f * x;
  return 1.055f * powf(x, 1.f / 2.4f) - 0.055f;
}

// Sine and cosine of x in [-pi/4, 2pi + pi/4], the range of the angles the
// renderer forms from [0, 1) random numbers (env-map directions and pdfs,
// phase-function azimuths).  Cody-Waite reduction (Cody & Waite, Software
// Manual for the Elementary Functions, 1980): r = x - k pi/2 with pi/2 split
// into three floats, the first two short enough that k times them is exact,
// so r is accurate to its last bit even next to a multiple of pi/2; then the
// Taylor polynomials of sin and cos on |r| <= pi/4 (truncation error below
// 3e-9) in Horner form.  No large-argument path: a few dozen instructions
// where a general sincosf carries a long one.  Same arithmetic on host and
// device (no contraction), so both give identical results.
GBV_HD void sincos_angle(float x, float &sn, float &cs) {
  const float kTwoOverPi = 0.636619772f;
  const float kPio2A = 0x1.92p+0f;       // 201/128
  const float kPio2B = 0x1.fb544p-12f;   // next 21 bits of pi/2
  const float kPio2C = 0x1.0b4612p-34f;  // the rest, rounded to float
  const float k = rintf(x * kTwoOverPi);
  const float r = ((x - k * kPio2A) - k * kPio2B) - k * kPio2C;
  const float r2 = r * r;
  const float ps = r + (r * r2) * (-1.f / 6.f + r2 * (1.f / 120.f + r2 * (-1.f / 5040.f + r2 * (1.f / 362880.f))));
  const float pc =
      1.f - .5f * r2 + (r2 * r2) * (1.f / 24.f + r2 * (-1.f / 720.f + r2 * (1.f / 40320.f + r2 * (-1.f / 3628800.f))));
  switch ((int)k & 3) {
    case 0: sn = ps; cs = pc; break;
    case 1: sn = pc; cs = -ps; break;
    case 2: sn = -ps; cs = -pc; break;
    default: sn = -pc; cs = ps; break;
  }
}

// Arc cosine and two-argument arc tangent of the env-map angles (theta =
// acos z and phi = atan2(y, x) of a direction), written from the series of
// arcsin and arctan so that host and device compute the same bits:
// * asin(s) = s + s t P(t), t = s^2, for s in [0, 1/2]; acos z = pi/2 -
//   asin z for |z| <= 1/2, and acos z = 2 asin(sqrt((1 - z)/2)) (z > 1/2) or
//   pi - 2 asin(sqrt((1 + z)/2)) (z < -1/2);
// * atan(u) = u + u w Q(w), w = u^2, for |u| <= tan(pi/8); atan2 reduces the
//   ratio of the smaller to the larger magnitude to that range with
//   atan(t) = pi/4 + atan((t - 1)/(t + 1)), then pi/2 - a, pi - a and the
//   sign of y place it in its octant.
// P (degree 5) and Q (degree 6) are least-squares fits, reweighted toward the
// largest relative error, of (asin s - s)/(s t) and (atan u - u)/(u w) on
// those ranges (fitted for this library).  pi/2, pi and pi/4 enter as
// two-float sums.  Against float64: acos within 1.2 ulp, atan2 within 2.2
// ulp (tests); no contraction, the same on host and device.
constexpr float kPio2Hi = 0x1.921fb6p+0f, kPio2Lo = -0x1.777a5cp-25f;
constexpr float kPiHi = 0x1.921fb6p+1f, kPiLo = -0x1.777a5cp-24f;
constexpr float kPio4Hi = 0x1.921fb6p-1f, kPio4Lo = -0x1.777a5cp-26f;
constexpr float kTanPi8 = 0x1.a8279ap-2f;
GBV_HD float asin_series(float s, float t) {  // asin(s), s in [0, 1/2], t = s^2
  const float p =
      ((((0x1.06a85p-5f * t + 0x1.28e096p-6f) * t + 0x1.fa3d84p-6f) * t + 0x1.6d7fd6p-5f) * t + 0x1.3333a6p-4f) * t +
      0x1.555556p-3f;
  return s + (s * t) * p;
}
// Both functions pick their operands with selects, so that a warp whose
// lanes fall on both sides of a reduction evaluates one series and (atan2)
// one division, not both branches.
GBV_HD float acos_angle(float z) {  // z in [-1, 1]
  const float a = fabsf(z);
  const bool mid = a <= .5f;
  const float tb = (1.f - a) * .5f;
  const float t = mid ? a * a : tb;
  const float s = mid ? a : sqrtf(tb);
  const float w = asin_series(s, t);
  const float wm = copysignf(w, z), w2 = 2.f * w;
  if (mid) return (kPio2Lo - wm) + kPio2Hi;
  return z > 0.f ? w2 : (kPiLo - w2) + kPiHi;
}
GBV_HD float atan_series(float u) {  // atan(u), |u| <= tan(pi/8)
  const float w = u * u;
  const float q =
      (((((-0x1.4b32d6p-5f * w + 0x1.2441d2p-4f) * w - 0x1.71d376p-4f) * w + 0x1.c6f68p-4f) * w - 0x1.2491cp-3f) * w +
       0x1.999998p-3f) * w -
      0x1.555556p-2f;
  return u + (u * w) * q;
}
GBV_HD float atan2_angle(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float mx = ax < ay ? ay : ax, mn = ax < ay ? ax : ay;
  const bool red = mn > kTanPi8 * mx;
  const float c = atan_series((red ? mn - mx : mn) / (red ? mn + mx : mx));
  float a = red ? (kPio4Lo + c) + kPio4Hi : c;
  if (mx == 0.f) a = 0.f;
  if (ay > ax) a = (kPio2Lo - a) + kPio2Hi;
  if (signbit(x)) a = (kPiLo - a) + kPiHi;
  return copysignf(a, y);
}

// rtcore/embree/Texture.cpp:324-336
GBV_HD void lerp_coords(int N, float tc, int &i0, int &i1, float &f) {
  if (tc - .5f <= 0.f) { i0 = i1 = 0; f = 0.f; return; }
  if (tc - .5f >= (float)(N - 1)) { i0 = i1 = N - 1; f = 0.f; return; }
  f = (tc - .5f) - (float)(int)(tc - .5f);
  i0 = (int)(tc - .5f);
  i1 = i0 + 1;
}

}  // namespace gbv
