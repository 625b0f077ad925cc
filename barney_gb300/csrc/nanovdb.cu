// nanovdb.cu -- NanoVDB grids (Float, Fp4, Fp8, Fp16, FpN): header parsing
// (host), the macrocell range build and a sampling entry point (device).
#include <cmath>
#include <cstring>
#include <cuda_runtime.h>
#include "gbv_nanovdb.cuh"
#include "gbv_internal.h"

namespace gbv {

NvdbGrid make_nvdb_grid(const void *d_grid, const gbv_nanovdb_info &info) {
  NvdbGrid g;
  g.base = reinterpret_cast<const unsigned char *>(d_grid);
  g.type = (uint32_t)info.grid_type;
  g.root = info.root_offset;
  g.tiles = info.root_tiles;
  g.background = info.background;
  for (int i = 0; i < 9; i++) g.invMatF[i] = info.inv_map[i];
  g.fixedMap = true;
  for (int i = 0; i < 3; i++) {
    g.vecF[i] = info.map_offset[i];
    g.lo[i] = info.index_lo[i];
    g.hi[i] = info.index_hi[i];
    if (g.lo[i] < -(1 << 21) || g.hi[i] > (1 << 21)) g.fixedMap = false;
  }
  return g;
}

// One thread per macrocell (NanoVDBData_computeMCs, NanoVDB.cu:28-60).
__global__ void __launch_bounds__(128) nvdb_mc_ranges_kernel(NvdbGrid g, int ncx, int ncy, int ncz,
                                                             float2 *__restrict__ ranges) {
  const long long n = (long long)ncx * ncy * ncz;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (tid >= n) return;
  int m[3] = {(int)(tid % ncx), (int)((tid / ncx) % ncy), (int)(tid / ((long long)ncx * ncy))};
  const int mc[3] = {ncx, ncy, ncz};
  const int size[3] = {g.hi[0] - g.lo[0] + 1, g.hi[1] - g.lo[1] + 1, g.hi[2] - g.lo[2] + 1};
  int a[3], b[3];
  nvdb_mc_footprint(g.lo, size, mc, m, a, b);
  // range1f starts empty (+inf, -inf) and extends by min/max
  float lo = __int_as_float(0x7f800000), hi = __int_as_float(0xff800000);
  for (int x = a[0]; x <= b[0]; x++)
    for (int y = a[1]; y <= b[1]; y++)
      for (int z = a[2]; z <= b[2]; z++) {
        const float v = nvdb_value(g, x, y, z);
        lo = mn(lo, v);
        hi = mx(hi, v);
      }
  ranges[tid] = make_float2(lo, hi);
}

__global__ void __launch_bounds__(128) nvdb_sample_kernel(NvdbGrid g, const float *__restrict__ P, long long n,
                                                          float *__restrict__ out) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = nvdb_sample(g, P[3 * i], P[3 * i + 1], P[3 * i + 2]);
}

static bool nvdb_type_read(uint32_t t) {
  return t == kNvdbGridTypeFloat || t == kNvdbGridTypeFp4 || t == kNvdbGridTypeFp8 || t == kNvdbGridTypeFp16 ||
         t == kNvdbGridTypeFpN;
}

static bool nvdb_info_ok(const gbv_nanovdb_info *info) {
  if (!info || !nvdb_type_read((uint32_t)info->grid_type)) return false;
  for (int i = 0; i < 3; i++)
    if (info->index_hi[i] < info->index_lo[i] || info->mc_dims[i] <= 0) return false;
  return info->root_offset > 0 && (unsigned long long)info->root_offset < info->bytes;
}

}  // namespace gbv

using namespace gbv;

extern "C" gbv_status gbv_nanovdb_parse(const void *h_grid, size_t bytes, gbv_nanovdb_info *info) {
  if (!h_grid || !info) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_nanovdb_parse: null pointer");
  const unsigned char *b = reinterpret_cast<const unsigned char *>(h_grid);
  if (bytes < kNvdbGridHeader + 64 + kNvdbRootTiles)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_nanovdb_parse: buffer smaller than a grid header");
  const uint64_t magic = nvdb_ld<uint64_t>(b);
  if (magic != kNvdbMagic0 && magic != kNvdbMagic1)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_nanovdb_parse: not a NanoVDB grid (magic number)");
  const uint32_t version = nvdb_ld<uint32_t>(b + kNvdbGridVersion);
  if ((version >> 21) != 32)
    return set_error(GBV_ERROR_UNSUPPORTED, "gbv_nanovdb_parse: NanoVDB format version other than 32");
  // the types of BARNEY_NANOVDB_FLOAT_TYPES (barney/volume/NanoVDB.h:23-28)
  const uint32_t type = nvdb_ld<uint32_t>(b + kNvdbGridType);
  if (!nvdb_type_read(type))
    return set_error(GBV_ERROR_UNSUPPORTED,
                     "gbv_nanovdb_parse: grid value type other than Float, Fp4, Fp8, Fp16 or FpN");
  const uint64_t gridSize = nvdb_ld<uint64_t>(b + kNvdbGridSize);
  if (gridSize > bytes) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_nanovdb_parse: buffer shorter than the grid");
  const long long rootRel = nvdb_ld<long long>(b + kNvdbGridHeader + kNvdbTreeRootOffset);
  const long long root = (long long)kNvdbGridHeader + rootRel;
  if (rootRel <= 0 || (root & 31) != 0 || (unsigned long long)root + kNvdbRootTiles > gridSize)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_nanovdb_parse: root node outside the grid");
  gbv_nanovdb_info r;
  std::memset(&r, 0, sizeof r);
  r.bytes = gridSize;
  r.grid_type = (int)type;
  r.root_offset = root;
  r.root_tiles = nvdb_ld<uint32_t>(b + root + kNvdbRootTableSize);
  if ((unsigned long long)root + kNvdbRootTiles + (unsigned long long)kNvdbRootTile * r.root_tiles > gridSize)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_nanovdb_parse: root table outside the grid");
  r.background = nvdb_ld<float>(b + root + kNvdbRootBackground);
  for (int i = 0; i < 9; i++) r.inv_map[i] = nvdb_ld<float>(b + kNvdbGridInvMatF + 4 * i);
  for (int i = 0; i < 3; i++) {
    r.map_offset[i] = nvdb_ld<float>(b + kNvdbGridVecF + 4 * i);
    r.index_lo[i] = nvdb_ld<int>(b + root + 4 * i);
    r.index_hi[i] = nvdb_ld<int>(b + root + 12 + 4 * i);
    // NanoVDBData::commit: world bounds as floats
    r.world_lo[i] = (float)nvdb_ld<double>(b + kNvdbGridWorldBBox + 8 * i);
    r.world_hi[i] = (float)nvdb_ld<double>(b + kNvdbGridWorldBBox + 24 + 8 * i);
    r.voxel_size[i] = nvdb_ld<double>(b + kNvdbGridVoxelSize + 8 * i);
    if (r.index_hi[i] < r.index_lo[i])
      return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_nanovdb_parse: grid without active values");
    // NanoVDBData::buildMCs: divRoundUp(gridSize, 16)
    const long long size = (long long)r.index_hi[i] - r.index_lo[i] + 1;
    if (size > (1ll << 24)) return set_error(GBV_ERROR_UNSUPPORTED, "gbv_nanovdb_parse: index bbox too large");
    r.mc_dims[i] = (int)((size + 15) / 16);
  }
  // Every child offset must land a whole node inside the grid, on NanoVDB's
  // 32-byte node alignment: the device follows them without checks and reads
  // up to 8-byte words from the nodes.
  constexpr long long kUpperBytes = (long long)kNvdbUpperTable + 8ll * 32768;
  constexpr long long kLowerBytes = (long long)kNvdbLowerTable + 8ll * 4096;
  const long long leafBytes = type == kNvdbGridTypeFloat  ? kNvdbLeafBytesFloat
                            : type == kNvdbGridTypeFp4  ? kNvdbLeafBytesFp4
                            : type == kNvdbGridTypeFp8  ? kNvdbLeafBytesFp8
                            : type == kNvdbGridTypeFp16 ? kNvdbLeafBytesFp16
                                                        : (long long)kNvdbLeafValues;  // FpN: its header first
  const long long end = (long long)gridSize;
  auto inside = [&](long long off, long long size) { return off > 0 && (off & 31) == 0 && off + size <= end; };
  for (uint32_t t = 0; t < r.root_tiles; t++) {
    const long long tile = root + (long long)kNvdbRootTiles + (long long)kNvdbRootTile * t;
    const long long c = nvdb_ld<long long>(b + tile + kNvdbTileChild);
    if (c == 0) continue;
    const long long up = root + c;
    if (!inside(up, kUpperBytes)) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_nanovdb_parse: bad upper node");
    for (uint32_t n = 0; n < 32768; n++) {
      if (!((nvdb_ld<uint64_t>(b + up + kNvdbUpperChildMask + 8 * (n >> 6)) >> (n & 63)) & 1ull)) continue;
      const long long lw = up + nvdb_ld<long long>(b + up + kNvdbUpperTable + 8ll * n);
      if (!inside(lw, kLowerBytes))
        return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_nanovdb_parse: bad lower node");
      for (uint32_t k = 0; k < 4096; k++) {
        if (!((nvdb_ld<uint64_t>(b + lw + kNvdbLowerChildMask + 8 * (k >> 6)) >> (k & 63)) & 1ull)) continue;
        const long long lf = lw + nvdb_ld<long long>(b + lw + kNvdbLowerTable + 8ll * k);
        if (!inside(lf, leafBytes)) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_nanovdb_parse: bad leaf");
        if (type == kNvdbGridTypeFpN) {  // codes of 1 << (flags >> 5) bits, 1 to 16
          const uint32_t lb = (uint32_t)nvdb_ld<uint8_t>(b + lf + kNvdbLeafFlags) >> 5;
          if (lb > 4)
            return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_nanovdb_parse: FpN leaf with a bit width above 16");
          if (!inside(lf, (long long)kNvdbLeafValues + 64ll * (1ll << lb)))
            return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_nanovdb_parse: bad leaf");
        }
      }
    }
  }
  *info = r;
  return GBV_OK;
}

extern "C" gbv_status gbv_nanovdb_mc_ranges(const void *d_grid, const gbv_nanovdb_info *info, float *d_ranges,
                                            void *stream) {
  if (!d_grid || !d_ranges || !nvdb_info_ok(info))
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_nanovdb_mc_ranges: null pointer or bad grid info");
  const NvdbGrid g = make_nvdb_grid(d_grid, *info);
  const long long n = (long long)info->mc_dims[0] * info->mc_dims[1] * info->mc_dims[2];
  if (n > (1ll << 31) - 1) return set_error(GBV_ERROR_UNSUPPORTED, "gbv_nanovdb_mc_ranges: too many macrocells");
  nvdb_mc_ranges_kernel<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
      g, info->mc_dims[0], info->mc_dims[1], info->mc_dims[2], reinterpret_cast<float2 *>(d_ranges));
  return check_launch("nvdb_mc_ranges_kernel");
}

extern "C" gbv_status gbv_nanovdb_sample(const void *d_grid, const gbv_nanovdb_info *info, const float *d_points,
                                         long long n, float *d_values, void *stream) {
  if (!d_grid || !d_points || !d_values || n < 0 || !nvdb_info_ok(info))
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_nanovdb_sample: null pointer or bad grid info");
  if (n == 0) return GBV_OK;
  const NvdbGrid g = make_nvdb_grid(d_grid, *info);
  nvdb_sample_kernel<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(g, d_points, n, d_values);
  return check_launch("nvdb_sample_kernel");
}
