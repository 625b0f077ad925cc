// nanovdb_writer.cpp -- input generator: a NanoVDB grid (memory layout of
// NanoVDB format 32.7, the version the reference vendors) of value type
// Float, Fp4, Fp8, Fp16 or FpN from a dense array, so that workloads of any
// size can be given to the NanoVDB field path where no NanoVDB tooling is
// installed.
//
// The tree: one root tile per 4096^3 region the array touches, each with an
// upper node (32^3 entries of 128^3), lower nodes (16^3 entries of 8^3) and
// 8^3-voxel leaves for every leaf region the array touches; voxels outside
// the array, and voxels equal to the background, are inactive and hold the
// background.  Nodes are stored breadth first (root, upper nodes, lower
// nodes, leaves) after the 672-byte grid header and 64-byte tree header,
// each child offset relative to its parent node, root tiles sorted by key.
// The node statistics (min, max, average, deviation) are left zero: the
// NanoVDB sampler and macrocell build read only values, masks and offsets.
// Unlike NanoVDB's builders it keeps leaves whose voxels are all inactive
// (they hold the background), so grids are larger but read the same.
// Quantized leaves are encoded as NanoVDB's builder encodes them with
// dithering off (tools/CreateNanoGrid.h, processLeafs): over the leaf's 512
// values (inactive ones hold the background) min and max, quantum =
// (max - min) / (2^bits - 1), code = trunc(encode * (v - min) + 0.5) with
// encode = (2^bits - 1) / (max - min) in float (in double for 16 bits); an
// FpN leaf takes the fewest bits of 1, 2, 4, 8 whose codes decode within the
// tolerance of every value, else 16 (its preProcess), the tolerance being
// the builder's default of 0.01 for a fog volume unless one is given.  A
// leaf whose values are all equal gets codes 0.
#include <algorithm>
#include <array>
#include <cstdint>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <vector>

#include "scene_gen.h"

namespace {

constexpr size_t kGrid = 672, kTree = 64, kRootHead = 64, kTile = 32;
constexpr size_t kUpper = 8256 + 8 * 32768, kLower = 1088 + 8 * 4096;
template <typename T> void put(std::vector<unsigned char> &b, size_t off, T v) {
  std::memcpy(b.data() + off, &v, sizeof(T));
}
void put_f(std::vector<unsigned char> &b, size_t off, float v) { put<float>(b, off, v); }
// nanovdb::GridType
constexpr int kFloat = 1, kFp4 = 13, kFp8 = 14, kFp16 = 15, kFpN = 16;

// bytes of a leaf of the type; log2w: an FpN leaf's log2 of its bit width
size_t leaf_bytes(int type, int log2w) {
  switch (type) {
  case kFloat: return 96 + 4 * 512;
  case kFp4: return 96 + 256;
  case kFp8: return 96 + 512;
  case kFp16: return 96 + 1024;
  default: return 96 + 64 * ((size_t)1 << log2w);
  }
}

// float -> unsigned code as the builder's static_cast, for the finite,
// non-negative values it meets; anything else (a leaf of equal values:
// inf * 0) gives 0
template <typename T, typename F> T to_code(F x, double limit) {
  if (!(x >= (F)0)) return 0;
  if (!((double)x < limit)) return (T)(limit - 1.0);
  return (T)x;
}

// FpN's choice (CreateNanoGrid::preProcess<FpN>): log2 of the bit width
int fpn_log2_width(const float v[512], float mn, float mx, float tolerance) {
  const float range = mx - mn;
  int lw = 0;
  while (range > 0.0f && lw < 4) {
    const uint32_t mask = (uint32_t(1) << (uint32_t(1) << lw)) - 1u;
    const float encode = (float)mask / range, decode = range / (float)mask;
    int j = 0;
    for (; j < 512; j++) {
      const uint32_t code = to_code<uint32_t, float>(encode * (v[j] - mn) + 0.5f, 4294967296.0);
      const float approx = (float)code * decode + mn;
      if (!(std::fabs(v[j] - approx) <= tolerance)) break;
    }
    if (j == 512) break;
    ++lw;
  }
  return lw;
}

// A quantized leaf's minimum, quantum, flags and codes (at L + 96)
void encode_leaf(std::vector<unsigned char> &b, size_t L, int type, int lw, const float v[512], float mn, float mx) {
  const int bits = type == kFp4 ? 4 : type == kFp8 ? 8 : type == kFp16 ? 16 : 1 << lw;
  const float range = mx - mn;
  put_f(b, L + 80, mn);
  put_f(b, L + 84, range / (float)((1u << bits) - 1u));
  if (type == kFpN) b[L + 15] = (unsigned char)(lw << 5);
  unsigned char *c = b.data() + L + 96;
  if (bits == 16) {
    const double encode = (double)((1u << 16) - 1u) / (double)range;
    for (int j = 0; j < 512; j++) {
      const uint16_t q = to_code<uint16_t, double>(encode * (double)(v[j] - mn) + 0.5, 65536.0);
      std::memcpy(c + 2 * j, &q, 2);
    }
    return;
  }
  const float encode = (float)((1u << bits) - 1u) / range;
  for (int j = 0; j < 512; j++) {
    const uint32_t q = to_code<uint8_t, float>(encode * (v[j] - mn) + 0.5f, 256.0);
    switch (bits) {
    case 1: c[j >> 3] |= (unsigned char)((q & 1u) << (j & 7)); break;
    case 2: c[j >> 2] |= (unsigned char)((q & 3u) << (2 * (j & 3))); break;
    case 4: c[j >> 1] |= (unsigned char)((q & 15u) << (4 * (j & 1))); break;
    default: c[j] = (unsigned char)q; break;
    }
  }
}

int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }
uint64_t root_key(int x, int y, int z) {
  return (uint64_t)((uint32_t)z >> 12) | ((uint64_t)((uint32_t)y >> 12) << 21) |
         ((uint64_t)((uint32_t)x >> 12) << 42);
}

}  // namespace

extern "C" int sg_nanovdb_from_dense_typed(const float *values, const int dims[3], const int origin[3],
                                           float background, double voxel_size, const double translation[3],
                                           int grid_type, float tolerance, void **out, size_t *bytes) {
  if (!values || !dims || !origin || !translation || !out || !bytes || dims[0] < 1 || dims[1] < 1 || dims[2] < 1 ||
      !(voxel_size > 0.0))
    return 1;
  if (grid_type != kFloat && grid_type != kFp4 && grid_type != kFp8 && grid_type != kFp16 && grid_type != kFpN)
    return 1;
  if (tolerance < 0.f) tolerance = 0.01f;  // AbsDiff's default for a fog volume
  const int nx = dims[0], ny = dims[1], nz = dims[2];
  const int lo[3] = {origin[0], origin[1], origin[2]};
  const int hi[3] = {origin[0] + nx - 1, origin[1] + ny - 1, origin[2] + nz - 1};
  auto value = [&](int x, int y, int z) -> float {
    const int i = x - lo[0], j = y - lo[1], k = z - lo[2];
    if (i < 0 || j < 0 || k < 0 || i >= nx || j >= ny || k >= nz) return background;
    return values[(size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * (size_t)k)];
  };
  // leaves (8^3 regions), lower nodes (128^3), upper nodes (4096^3) touched
  std::map<uint64_t, int> upperIdx;            // key -> index
  std::vector<std::array<int, 3>> upperOrg;    // origins
  std::map<std::array<int, 3>, int> lowerIdx;  // origin -> index
  std::vector<std::array<int, 3>> lowerOrg;
  std::vector<std::array<int, 3>> leafOrg;
  for (int lz = floor_div(lo[2], 8); lz <= floor_div(hi[2], 8); lz++)
    for (int ly = floor_div(lo[1], 8); ly <= floor_div(hi[1], 8); ly++)
      for (int lx = floor_div(lo[0], 8); lx <= floor_div(hi[0], 8); lx++) {
        const std::array<int, 3> leaf = {lx * 8, ly * 8, lz * 8};
        leafOrg.push_back(leaf);
        const std::array<int, 3> lower = {floor_div(leaf[0], 128) * 128, floor_div(leaf[1], 128) * 128,
                                          floor_div(leaf[2], 128) * 128};
        if (!lowerIdx.count(lower)) {
          lowerIdx[lower] = (int)lowerOrg.size();
          lowerOrg.push_back(lower);
        }
        const uint64_t key = root_key(leaf[0], leaf[1], leaf[2]);
        if (!upperIdx.count(key)) {
          upperIdx[key] = 0;
          upperOrg.push_back({floor_div(leaf[0], 4096) * 4096, floor_div(leaf[1], 4096) * 4096,
                              floor_div(leaf[2], 4096) * 4096});
        }
      }
  // upper nodes in ascending key order (the root table's order)
  std::sort(upperOrg.begin(), upperOrg.end(), [](const std::array<int, 3> &a, const std::array<int, 3> &b) {
    return root_key(a[0], a[1], a[2]) < root_key(b[0], b[1], b[2]);
  });
  for (size_t u = 0; u < upperOrg.size(); u++) upperIdx[root_key(upperOrg[u][0], upperOrg[u][1], upperOrg[u][2])] = (int)u;
  const size_t nU = upperOrg.size(), nL = lowerOrg.size(), nF = leafOrg.size();
  const size_t root = kGrid + kTree;
  const size_t upper0 = root + kRootHead + kTile * nU;
  const size_t lower0 = upper0 + kUpper * nU;
  const size_t leaf0 = lower0 + kLower * nL;
  // each leaf's 512 values (x-major: n = x << 6 | y << 3 | z), their range,
  // FpN's bit width and the leaf's byte offset
  std::vector<float> vals(nF * 512);
  std::vector<float> lmin(nF), lmax(nF);
  std::vector<int> lw(nF, 0);
  std::vector<size_t> leafAt(nF);
  size_t total = leaf0;
  for (size_t f = 0; f < nF; f++) {
    const auto &o = leafOrg[f];
    float mn = std::numeric_limits<float>::max(), mx = -mn;
    for (int n = 0; n < 512; n++) {
      const float v = value(o[0] + (n >> 6), o[1] + ((n >> 3) & 7), o[2] + (n & 7));
      vals[f * 512 + n] = v;
      if (v < mn) mn = v;
      if (v > mx) mx = v;
    }
    lmin[f] = mn;
    lmax[f] = mx;
    if (grid_type == kFpN) lw[f] = fpn_log2_width(&vals[f * 512], mn, mx, tolerance);
    leafAt[f] = total;
    total += leaf_bytes(grid_type, lw[f]);
  }
  std::vector<unsigned char> b(total, 0);

  // ---- leaves: origin, value mask, values; the active index bbox ----
  int amin[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, amax[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
  uint64_t active = 0;
  for (size_t f = 0; f < nF; f++) {
    const size_t L = leafAt[f];
    const auto &o = leafOrg[f];
    put<int32_t>(b, L + 0, o[0]);
    put<int32_t>(b, L + 4, o[1]);
    put<int32_t>(b, L + 8, o[2]);
    put<uint8_t>(b, L + 12, 7);
    put<uint8_t>(b, L + 13, 7);
    put<uint8_t>(b, L + 14, 7);
    for (int n = 0; n < 512; n++) {
      const int x = o[0] + (n >> 6), y = o[1] + ((n >> 3) & 7), z = o[2] + (n & 7);
      const float v = vals[f * 512 + n];
      if (grid_type == kFloat) put<float>(b, L + 96 + 4 * (size_t)n, v);
      const bool inside = x >= lo[0] && x <= hi[0] && y >= lo[1] && y <= hi[1] && z >= lo[2] && z <= hi[2];
      if (inside && v != background) {
        b[L + 16 + (n >> 3)] |= (unsigned char)(1u << (n & 7));
        active++;
        amin[0] = std::min(amin[0], x); amin[1] = std::min(amin[1], y); amin[2] = std::min(amin[2], z);
        amax[0] = std::max(amax[0], x); amax[1] = std::max(amax[1], y); amax[2] = std::max(amax[2], z);
      }
    }
    if (grid_type != kFloat) encode_leaf(b, L, grid_type, lw[f], &vals[f * 512], lmin[f], lmax[f]);
    // the leaf in its lower node's table
    const std::array<int, 3> lowerO = {floor_div(o[0], 128) * 128, floor_div(o[1], 128) * 128,
                                       floor_div(o[2], 128) * 128};
    const size_t Lw = lower0 + kLower * (size_t)lowerIdx[lowerO];
    const uint32_t n = (uint32_t)((((o[0] & 127) >> 3) << 8) | (((o[1] & 127) >> 3) << 4) | ((o[2] & 127) >> 3));
    b[Lw + 544 + (n >> 3)] |= (unsigned char)(1u << (n & 7));
    put<int64_t>(b, Lw + 1088 + 8 * (size_t)n, (int64_t)L - (int64_t)Lw);
  }
  if (active == 0) return 2;  // a grid needs active values
  // ---- lower nodes: bbox and their place in the upper nodes ----
  for (size_t l = 0; l < nL; l++) {
    const size_t Lw = lower0 + kLower * l;
    const auto &o = lowerOrg[l];
    put<int32_t>(b, Lw + 0, o[0]); put<int32_t>(b, Lw + 4, o[1]); put<int32_t>(b, Lw + 8, o[2]);
    put<int32_t>(b, Lw + 12, o[0] + 127); put<int32_t>(b, Lw + 16, o[1] + 127); put<int32_t>(b, Lw + 20, o[2] + 127);
    for (int n = 0; n < 4096; n++)  // entries without a child hold the background as a tile value
      if (!((b[Lw + 544 + (n >> 3)] >> (n & 7)) & 1)) put<float>(b, Lw + 1088 + 8 * (size_t)n, background);
    const size_t U = upper0 + kUpper * (size_t)upperIdx[root_key(o[0], o[1], o[2])];
    const uint32_t n = (uint32_t)((((o[0] & 4095) >> 7) << 10) | (((o[1] & 4095) >> 7) << 5) | ((o[2] & 4095) >> 7));
    b[U + 4128 + (n >> 3)] |= (unsigned char)(1u << (n & 7));
    put<int64_t>(b, U + 8256 + 8 * (size_t)n, (int64_t)Lw - (int64_t)U);
  }
  // ---- upper nodes and the root table ----
  for (size_t u = 0; u < nU; u++) {
    const size_t U = upper0 + kUpper * u;
    const auto &o = upperOrg[u];
    put<int32_t>(b, U + 0, o[0]); put<int32_t>(b, U + 4, o[1]); put<int32_t>(b, U + 8, o[2]);
    put<int32_t>(b, U + 12, o[0] + 4095); put<int32_t>(b, U + 16, o[1] + 4095); put<int32_t>(b, U + 20, o[2] + 4095);
    for (int n = 0; n < 32768; n++)
      if (!((b[U + 4128 + (n >> 3)] >> (n & 7)) & 1)) put<float>(b, U + 8256 + 8 * (size_t)n, background);
    const size_t T = root + kRootHead + kTile * u;
    put<uint64_t>(b, T + 0, root_key(o[0], o[1], o[2]));
    put<int64_t>(b, T + 8, (int64_t)U - (int64_t)root);
    put<uint32_t>(b, T + 16, 0);
    put<float>(b, T + 20, background);
  }
  for (int a = 0; a < 3; a++) {
    put<int32_t>(b, root + 4 * a, amin[a]);
    put<int32_t>(b, root + 12 + 4 * a, amax[a]);
  }
  put<uint32_t>(b, root + 24, (uint32_t)nU);
  put<float>(b, root + 28, background);
  // ---- tree header: offsets of the first leaf, lower, upper node and the root from the tree ----
  const size_t tree = kGrid;
  put<uint64_t>(b, tree + 0, leaf0 - tree);
  put<uint64_t>(b, tree + 8, lower0 - tree);
  put<uint64_t>(b, tree + 16, upper0 - tree);
  put<uint64_t>(b, tree + 24, root - tree);
  put<uint32_t>(b, tree + 32, (uint32_t)nF);
  put<uint32_t>(b, tree + 36, (uint32_t)nL);
  put<uint32_t>(b, tree + 40, (uint32_t)nU);
  put<uint64_t>(b, tree + 56, active);
  // ---- grid header ----
  put<uint64_t>(b, 0, 0x304244566f6e614eull);  // "NanoVDB0"
  put<uint32_t>(b, 16, (32u << 21) | (7u << 10));
  put<uint32_t>(b, 28, 1);  // grid count
  put<uint64_t>(b, 32, (uint64_t)total);
  std::memcpy(b.data() + 40, "density", 7);
  // map: index -> world = voxel_size * index + translation
  const double vs = voxel_size, inv = 1.0 / voxel_size;
  for (int a = 0; a < 3; a++) {
    put<float>(b, 296 + 4 * (4 * a), (float)vs);        // matF diagonal
    put<float>(b, 332 + 4 * (4 * a), (float)inv);       // invMatF diagonal
    put<float>(b, 368 + 4 * a, (float)translation[a]);   // vecF
    put<double>(b, 384 + 8 * (4 * a), vs);               // matD diagonal
    put<double>(b, 456 + 8 * (4 * a), inv);              // invMatD diagonal
    put<double>(b, 528 + 8 * a, translation[a]);         // vecD
  }
  put<float>(b, 380, 1.f);   // taperF
  put<double>(b, 552, 1.0);  // taperD
  // world bbox: the index bbox [min, max + 1] through the map (tools/GridStats.h:595)
  for (int a = 0; a < 3; a++) {
    put<double>(b, 560 + 8 * a, translation[a] + vs * (double)amin[a]);
    put<double>(b, 584 + 8 * a, translation[a] + vs * ((double)amax[a] + 1.0));
    // voxel size as NanoVDB derives it from the map: applyMap(1) - applyMap(0)
    put<double>(b, 608 + 8 * a, (vs + translation[a]) - translation[a]);
  }
  put<uint32_t>(b, 632, 2);  // grid class: fog volume
  put<uint32_t>(b, 636, (uint32_t)grid_type);
  void *mem = std::malloc(total);
  if (!mem) return 3;
  std::memcpy(mem, b.data(), total);
  *out = mem;
  *bytes = total;
  return 0;
}

extern "C" int sg_nanovdb_from_dense(const float *values, const int dims[3], const int origin[3], float background,
                                     double voxel_size, const double translation[3], void **out, size_t *bytes) {
  return sg_nanovdb_from_dense_typed(values, dims, origin, background, voxel_size, translation, kFloat, -1.f, out,
                                     bytes);
}

extern "C" void sg_free(void *p) { std::free(p); }
