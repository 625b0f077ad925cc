// gbv_nanovdb.cuh -- NanoVDB grids on the structured-volume path: value
// lookup in a grid buffer, the reference's NanoVDB sampler and its macrocell
// footprint.
//
// The grid buffer is one NanoVDB grid in the NanoVDB memory layout of format
// version 32 (the layout nanovdb::GridHandle holds and nanovdb::io writes),
// of one of the value types the reference's NanoVDB field reads: Float, or
// the quantized Fp4, Fp8, Fp16 and FpN.  A 672-byte grid header, a 64-byte
// tree header, then the nodes -- a root of 32-byte tiles keyed by the
// coordinates of their 4096^3 region, upper internal nodes of 32^3 entries,
// lower internal nodes of 16^3 entries and 8^3-voxel leaves.  An internal
// entry whose child-mask bit is set holds the signed byte offset of its
// child node, otherwise a float tile value; child offsets are relative to the
// parent node (to the root node for the root's tiles).  Root and internal
// nodes are the same for every type; leaves differ: a Float leaf holds 512
// floats, a quantized leaf a minimum m and a quantum q and 512 codes c of 4,
// 8 or 16 bits (FpN: 1, 2, 4, 8 or 16 bits, the leaf's choice, in the top 3
// bits of its flags byte), the value being float(c) * q + m.  The byte
// offsets below are those of that layout; the pin tests check them against
// the NanoVDB headers the reference vendors (3rdParty/nanovdb, version
// 32.7).
#pragma once
#include <stdint.h>
#include "gbv_math.cuh"

namespace gbv {

constexpr uint64_t kNvdbMagic0 = 0x304244566f6e614eull;  // "NanoVDB0"
constexpr uint64_t kNvdbMagic1 = 0x314244566f6e614eull;  // "NanoVDB1"
// nanovdb::GridType of the types read
constexpr uint32_t kNvdbGridTypeFloat = 1, kNvdbGridTypeFp4 = 13, kNvdbGridTypeFp8 = 14, kNvdbGridTypeFp16 = 15,
                   kNvdbGridTypeFpN = 16;
// grid header
constexpr size_t kNvdbGridVersion = 16, kNvdbGridSize = 32, kNvdbGridInvMatF = 332, kNvdbGridVecF = 368;
constexpr size_t kNvdbGridWorldBBox = 560, kNvdbGridVoxelSize = 608, kNvdbGridType = 636;
constexpr size_t kNvdbGridHeader = 672;
// tree header (after the grid header): byte offset of the root node
constexpr size_t kNvdbTreeRootOffset = 24;
// root node: index bbox, table size, background; tiles after 64 bytes
constexpr size_t kNvdbRootTableSize = 24, kNvdbRootBackground = 28, kNvdbRootTiles = 64, kNvdbRootTile = 32;
constexpr size_t kNvdbTileChild = 8, kNvdbTileValue = 20;
// internal nodes: child mask and the table of values / child offsets
constexpr size_t kNvdbUpperChildMask = 32 + 4096, kNvdbUpperTable = 8256;
constexpr size_t kNvdbLowerChildMask = 32 + 512, kNvdbLowerTable = 1088;
// leaves: the 512 values (Float) or codes (quantized); a quantized leaf's
// flags byte, minimum and quantum
constexpr size_t kNvdbLeafValues = 96, kNvdbLeafFlags = 15, kNvdbLeafMinimum = 80, kNvdbLeafQuantum = 84;
// leaf bytes: Float, Fp4, Fp8, Fp16; FpN: 96 + 64 x its bit width
constexpr long long kNvdbLeafBytesFloat = 2144, kNvdbLeafBytesFp4 = 352, kNvdbLeafBytesFp8 = 608,
                    kNvdbLeafBytesFp16 = 1120;

// A parsed grid (host-side header fields, device pointer to the buffer).
struct NvdbGrid {
  const unsigned char *base;  // the grid buffer (device memory for kernels)
  uint32_t type;              // kNvdbGridType*
  long long root;             // byte offset of the root node from base
  uint32_t tiles;             // root table size
  float background;
  float invMatF[9], vecF[3];  // world -> index map, single precision
  int lo[3], hi[3];           // index bbox of the active values
  bool fixedMap;              // the bbox lies within +-2^21: nvdb_axis may work in fixed point
};

// One axis of the sampler's index position, as the reference computes it in
// double: x = clamp((double)r - 0.5, lo, hi), i = floor(x), u = (float)(x - i).
// For |r| in [2^-17, 2^22) (and a bbox within +-2^21) every one of those
// double operations is exact, so they are done exactly in 64-bit fixed point
// with 40 fraction bits instead (r * 2^40 is an integer there: r's last bit
// is worth at least 2^-40), rounding u to float once as the double path's
// conversion does.  Other r (tiny, huge, NaN) take the double path.
// GB300's FP64 rate is low; this keeps the sampler off it for nearly every
// sample.
GBV_HD void nvdb_axis(float r, int lo, int hi, bool fixedMap, int &i, float &u) {
  const float a = fabsf(r);
  if (fixedMap && a >= 0x1p-17f && a < 0x1p22f) {
    long long d = (long long)(r * 0x1p40f) - (1ll << 39);
    const long long l = (long long)lo * (1ll << 40), h = (long long)hi * (1ll << 40);
    d = d < l ? l : d > h ? h : d;
    i = (int)(d >> 40);  // floor (arithmetic shift)
    u = (float)(d & ((1ll << 40) - 1)) * 0x1p-40f;
    return;
  }
  double x = (double)r - 0.5;
  // nanovdb::math::Clamp(x, a, b) = fmax(fmin(x, b), a)
  x = fmax(fmin(x, (double)hi), (double)lo);
  i = (int)floor(x);
  u = (float)(x - (double)i);
}

template <typename T> GBV_HD T nvdb_ld(const unsigned char *p) {
#if defined(__CUDA_ARCH__)
  return *reinterpret_cast<const T *>(p);
#else
  T v;
  __builtin_memcpy(&v, p, sizeof(T));
  return v;
#endif
}

// LeafData<BuildType>::getValue(n) (NanoVDB.h, LeafData<float>, LeafData<Fp4>,
// <Fp8>, <Fp16>, <FpN>): the value of voxel n of the leaf at lf.
GBV_HD float nvdb_leaf_value(uint32_t type, const unsigned char *lf, uint32_t n) {
  if (type == kNvdbGridTypeFloat) return nvdb_ld<float>(lf + kNvdbLeafValues + 4 * (size_t)n);
  uint32_t code;
  if (type == kNvdbGridTypeFp8) {
    code = nvdb_ld<uint8_t>(lf + kNvdbLeafValues + n);
  } else if (type == kNvdbGridTypeFp16) {
    code = nvdb_ld<uint16_t>(lf + kNvdbLeafValues + 2 * (size_t)n);
  } else if (type == kNvdbGridTypeFp4) {
    code = ((uint32_t)nvdb_ld<uint8_t>(lf + kNvdbLeafValues + (n >> 1)) >> ((n & 1u) << 2)) & 15u;
  } else {  // FpN: b = log2 of the bit width (0..4, checked when the grid is parsed)
    const uint32_t b = (uint32_t)nvdb_ld<uint8_t>(lf + kNvdbLeafFlags) >> 5;
    code = nvdb_ld<uint32_t>(lf + kNvdbLeafValues + 4 * (size_t)(n >> (5u - b)));
    code >>= (n & ((32u >> b) - 1u)) << b;
    code &= (1u << (1u << b)) - 1u;
  }
  return (float)code * nvdb_ld<float>(lf + kNvdbLeafQuantum) + nvdb_ld<float>(lf + kNvdbLeafMinimum);
}

// ReadAccessor::getValue: the value at index coordinates (x, y, z) --
// an active or inactive voxel, a tile value, or the background.
GBV_HD float nvdb_value(const NvdbGrid &g, int x, int y, int z) {
  const unsigned char *root = g.base + g.root;
  const uint64_t key = (uint64_t)((uint32_t)z >> 12) | ((uint64_t)((uint32_t)y >> 12) << 21) |
                       ((uint64_t)((uint32_t)x >> 12) << 42);
  const unsigned char *tile = nullptr;
  for (uint32_t i = 0; i < g.tiles; i++) {
    const unsigned char *t = root + kNvdbRootTiles + (size_t)kNvdbRootTile * i;
    if (nvdb_ld<uint64_t>(t) == key) {
      tile = t;
      break;
    }
  }
  if (!tile) return g.background;
  const long long child = nvdb_ld<long long>(tile + kNvdbTileChild);
  if (child == 0) return nvdb_ld<float>(tile + kNvdbTileValue);
  const unsigned char *up = root + child;
  uint32_t n = (((uint32_t)x & 4095u) >> 7 << 10) | (((uint32_t)y & 4095u) >> 7 << 5) | (((uint32_t)z & 4095u) >> 7);
  if (!((nvdb_ld<uint64_t>(up + kNvdbUpperChildMask + 8 * (n >> 6)) >> (n & 63)) & 1ull))
    return nvdb_ld<float>(up + kNvdbUpperTable + 8 * (size_t)n);
  const unsigned char *lw = up + nvdb_ld<long long>(up + kNvdbUpperTable + 8 * (size_t)n);
  n = (((uint32_t)x & 127u) >> 3 << 8) | (((uint32_t)y & 127u) >> 3 << 4) | (((uint32_t)z & 127u) >> 3);
  if (!((nvdb_ld<uint64_t>(lw + kNvdbLowerChildMask + 8 * (n >> 6)) >> (n & 63)) & 1ull))
    return nvdb_ld<float>(lw + kNvdbLowerTable + 8 * (size_t)n);
  const unsigned char *lf = lw + nvdb_ld<long long>(lw + kNvdbLowerTable + 8 * (size_t)n);
  n = (((uint32_t)x & 7u) << 6) | (((uint32_t)y & 7u) << 3) | ((uint32_t)z & 7u);
  return nvdb_leaf_value(g.type, lf, n);
}

// NanoVDBDataSampler::DD::sample (barney/volume/NanoVDB.h:100-129): world ->
// index with the grid's single-precision inverse map (worldToIndexF: the
// translation subtracted in double, the 3x3 product in float with fused
// multiply-adds), shifted by -0.5 to voxel centres and clamped to the index
// bbox, then the trilinear sampler (SampleFromVoxels<acc, 1>): the 8 values
// at floor(x) + {0,1}^3 and lerp(a, b, w) = a + float(w) * (b - a) along z,
// then y, then x.  Never NaN: points outside take the border values.
GBV_HD float nvdb_sample(const NvdbGrid &g, float px, float py, float pz) {
  // (float)((double)p - (double)v) is the float difference p - v: when the
  // double difference is exact both round it once, else |v| < 2^-29 |p| (or
  // the reverse) and both give p (v)
  const float fx = px - g.vecF[0], fy = py - g.vecF[1], fz = pz - g.vecF[2];
  const float *m = g.invMatF;
  int i, j, k;
  float fu, fv, fw;
  nvdb_axis(fmaf(fx, m[0], fmaf(fy, m[1], fz * m[2])), g.lo[0], g.hi[0], g.fixedMap, i, fu);
  nvdb_axis(fmaf(fx, m[3], fmaf(fy, m[4], fz * m[5])), g.lo[1], g.hi[1], g.fixedMap, j, fv);
  nvdb_axis(fmaf(fx, m[6], fmaf(fy, m[7], fz * m[8])), g.lo[2], g.hi[2], g.fixedMap, k, fw);
  float s[2][2][2];
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++)
#pragma unroll
      for (int c = 0; c < 2; c++) s[a][b][c] = nvdb_value(g, i + a, j + b, k + c);
  auto lerp = [](float p, float q, float t) { return p + t * (q - p); };
  return lerp(lerp(lerp(s[0][0][0], s[0][0][1], fw), lerp(s[0][1][0], s[0][1][1], fw), fv),
              lerp(lerp(s[1][0][0], s[1][0][1], fw), lerp(s[1][1][0], s[1][1][1], fw), fv), fu);
}

// The index footprint of macrocell (mx, my, mz) of a grid of mc[3]
// macrocells over an index bbox of size[3] voxels starting at lo[3]
// (NanoVDBData_computeMCs, barney/volume/NanoVDB.cu:28-60): from
// lo + (m * size) / mc to lo + ((m + 1) * size) / mc + 1, both inclusive.
GBV_HD void nvdb_mc_footprint(const int lo[3], const int size[3], const int mc[3], int m[3], int a[3], int b[3]) {
  for (int t = 0; t < 3; t++) {
    a[t] = lo[t] + (m[t] * size[t]) / mc[t];
    b[t] = lo[t] + ((m[t] + 1) * size[t]) / mc[t] + 1;
  }
}

}  // namespace gbv
