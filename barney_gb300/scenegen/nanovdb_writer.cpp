// nanovdb_writer.cpp -- input generator: a NanoVDB float grid (memory layout
// of NanoVDB format 32.7, the version the reference vendors) from a dense
// array, so that workloads of any size can be given to the NanoVDB field
// path where no NanoVDB tooling is installed.
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
#include <algorithm>
#include <array>
#include <cstdint>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>

#include "scene_gen.h"

namespace {

constexpr size_t kGrid = 672, kTree = 64, kRootHead = 64, kTile = 32;
constexpr size_t kUpper = 8256 + 8 * 32768, kLower = 1088 + 8 * 4096, kLeaf = 96 + 4 * 512;

template <typename T> void put(std::vector<unsigned char> &b, size_t off, T v) {
  std::memcpy(b.data() + off, &v, sizeof(T));
}
int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }
uint64_t root_key(int x, int y, int z) {
  return (uint64_t)((uint32_t)z >> 12) | ((uint64_t)((uint32_t)y >> 12) << 21) |
         ((uint64_t)((uint32_t)x >> 12) << 42);
}

}  // namespace

extern "C" int sg_nanovdb_from_dense(const float *values, const int dims[3], const int origin[3], float background,
                                     double voxel_size, const double translation[3], void **out, size_t *bytes) {
  if (!values || !dims || !origin || !translation || !out || !bytes || dims[0] < 1 || dims[1] < 1 || dims[2] < 1 ||
      !(voxel_size > 0.0))
    return 1;
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
  const size_t total = leaf0 + kLeaf * nF;
  std::vector<unsigned char> b(total, 0);

  // ---- leaves: origin, value mask, values; the active index bbox ----
  int amin[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, amax[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
  uint64_t active = 0;
  for (size_t f = 0; f < nF; f++) {
    const size_t L = leaf0 + kLeaf * f;
    const auto &o = leafOrg[f];
    put<int32_t>(b, L + 0, o[0]);
    put<int32_t>(b, L + 4, o[1]);
    put<int32_t>(b, L + 8, o[2]);
    put<uint8_t>(b, L + 12, 7);
    put<uint8_t>(b, L + 13, 7);
    put<uint8_t>(b, L + 14, 7);
    for (int n = 0; n < 512; n++) {
      const int x = o[0] + (n >> 6), y = o[1] + ((n >> 3) & 7), z = o[2] + (n & 7);
      const float v = value(x, y, z);
      put<float>(b, L + 96 + 4 * (size_t)n, v);
      const bool inside = x >= lo[0] && x <= hi[0] && y >= lo[1] && y <= hi[1] && z >= lo[2] && z <= hi[2];
      if (inside && v != background) {
        b[L + 16 + (n >> 3)] |= (unsigned char)(1u << (n & 7));
        active++;
        amin[0] = std::min(amin[0], x); amin[1] = std::min(amin[1], y); amin[2] = std::min(amin[2], z);
        amax[0] = std::max(amax[0], x); amax[1] = std::max(amax[1], y); amax[2] = std::max(amax[2], z);
      }
    }
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
  put<uint32_t>(b, 636, 1);  // grid type: float
  void *mem = std::malloc(total);
  if (!mem) return 3;
  std::memcpy(mem, b.data(), total);
  *out = mem;
  *bytes = total;
  return 0;
}

extern "C" void sg_free(void *p) { std::free(p); }
