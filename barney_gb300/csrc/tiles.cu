// tiles.cu -- the compressed tile format of the frame gather across ranks.
//
// DistFB (barney/fb/DistFB.h:43-48, DistFB.cu:25-101) ships each rank's
// finished 32x32 tiles to the owner as CompressedColorTile: per pixel the
// colour divided by its largest channel, as RGBA8 (alpha without scale), and
// that largest channel as a 16-bit float -- 6 bytes instead of 16.  The
// half conversion is the CPU backend's float16_t (ties away from zero,
// rtcore/embree/Float16.cpp), as for the path throughput.
#include "render_kernel.cuh"

namespace gbv {

constexpr int kTilePixels = kRefTile * kRefTile;

// Layout of one compressed tile in memory: kTilePixels uint32 RGBA8, then
// kTilePixels uint16 halves (6144 bytes; the reference's struct layout).
struct CompressedTileView {
  uint32_t *rgba;
  uint16_t *scale;
};
__device__ __forceinline__ CompressedTileView tile_view(void *base, long long k) {
  unsigned char *t = static_cast<unsigned char *>(base) + (size_t)k * (kTilePixels * 6);
  return CompressedTileView{reinterpret_cast<uint32_t *>(t), reinterpret_cast<uint16_t *>(t + kTilePixels * 4)};
}

// CompressTiles::run (DistFB.cu:92-108): one block per tile, one thread per
// pixel; pixels past the frame's edge get zeros.
__global__ void __launch_bounds__(kTilePixels) compress_tiles_kernel(const float4 *__restrict__ accum, int W, int H,
                                                                       float accumScale, int rank, int numRanks,
                                                                       void *out) {
  const long long k = blockIdx.x;
  const int pixelID = threadIdx.x;
  const long long id = (long long)rank + k * numRanks;
  const int tilesX = (W + kRefTile - 1) / kRefTile;
  const int ix = (int)(id % tilesX) * kRefTile + pixelID % kRefTile;
  const int iy = (int)(id / tilesX) * kRefTile + pixelID / kRefTile;
  CompressedTileView v = tile_view(out, k);
  if (ix >= W || iy >= H) {
    v.rgba[pixelID] = 0u;
    v.scale[pixelID] = 0u;
    return;
  }
  const float4 a = accum[(size_t)iy * W + ix];
  float4 c = make_float4(a.x * accumScale, a.y * accumScale, a.z * accumScale, a.w * accumScale);
  const float scale = mx(mx(c.x, c.y), c.z);
  const float rs = 1.f / scale;
  c.x *= rs;
  c.y *= rs;
  c.z *= rs;
  v.scale[pixelID] = f2h(scale);
  v.rgba[pixelID] = (make_8bit(c.x) << 0) + (make_8bit(c.y) << 8) + (make_8bit(c.z) << 16) + (make_8bit(c.w) << 24);
}

// UnpackTiles::run (DistFB.cu:39-79): channels back as float(v) * (1/255),
// rgb times the scale, written as float4, RGBA8 or sRGB RGBA8.
__global__ void __launch_bounds__(kTilePixels) unpack_tiles_kernel(const void *in, int W, int H, int rank,
                                                                     int numRanks, int format, void *out) {
  const long long k = blockIdx.x;
  const int pixelID = threadIdx.x;
  const long long id = (long long)rank + k * numRanks;
  const int tilesX = (W + kRefTile - 1) / kRefTile;
  const int ix = (int)(id % tilesX) * kRefTile + pixelID % kRefTile;
  const int iy = (int)(id / tilesX) * kRefTile + pixelID / kRefTile;
  if (ix >= W || iy >= H) return;
  const CompressedTileView v = tile_view(const_cast<void *>(in), k);
  const uint32_t p = v.rgba[pixelID];
  float4 c = make_float4((float)((p >> 0) & 0xffu) * (1.f / 255.f), (float)((p >> 8) & 0xffu) * (1.f / 255.f),
                         (float)((p >> 16) & 0xffu) * (1.f / 255.f), (float)((p >> 24) & 0xffu) * (1.f / 255.f));
  const float scale = h2f(v.scale[pixelID]);
  c.x *= scale;
  c.y *= scale;
  c.z *= scale;
  const size_t i = (size_t)iy * W + ix;
  if (format == GBV_FB_FLOAT4) {
    reinterpret_cast<float4 *>(out)[i] = c;
    return;
  }
  if (format == GBV_FB_RGBA8_SRGB) {
    c.x = linear_to_srgb(c.x);
    c.y = linear_to_srgb(c.y);
    c.z = linear_to_srgb(c.z);
  }
  reinterpret_cast<uint32_t *>(out)[i] =
      (make_8bit(c.x) << 0) + (make_8bit(c.y) << 8) + (make_8bit(c.z) << 16) + (make_8bit(c.w) << 24);
}

}  // namespace gbv

using namespace gbv;

extern "C" {

size_t gbv_compressed_tile_bytes(void) { return (size_t)kTilePixels * 6; }

gbv_status gbv_compress_tiles(const float *d_accum, int width, int height, int accum_id, int rank, int num_ranks,
                              void *d_tiles, void *stream) {
  if (!d_accum || !d_tiles || width <= 0 || height <= 0 || accum_id <= 0)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_compress_tiles: bad argument (accum_id must be >= 1)");
  if (num_ranks < 1 || rank < 0 || rank >= num_ranks)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_compress_tiles: rank must be in [0, num_ranks)");
  const long long n = owned_ref_tiles(width, height, rank, num_ranks);
  if (n == 0) return GBV_OK;
  if (n > (1ll << 31) - 1) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_compress_tiles: too many tiles");
  compress_tiles_kernel<<<(unsigned)n, kTilePixels, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float4 *>(d_accum), width, height, 1.f / (float)accum_id, rank, num_ranks, d_tiles);
  return check_launch("compress_tiles_kernel");
}

gbv_status gbv_unpack_tiles(const void *d_tiles, int width, int height, int rank, int num_ranks, int format,
                            void *d_out, void *stream) {
  if (!d_tiles || !d_out || width <= 0 || height <= 0)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_unpack_tiles: bad argument");
  if (num_ranks < 1 || rank < 0 || rank >= num_ranks)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_unpack_tiles: rank must be in [0, num_ranks)");
  if (format < GBV_FB_FLOAT4 || format > GBV_FB_RGBA8_SRGB)
    return set_error(GBV_ERROR_UNSUPPORTED, "gbv_unpack_tiles: unsupported format");
  const long long n = owned_ref_tiles(width, height, rank, num_ranks);
  if (n == 0) return GBV_OK;
  if (n > (1ll << 31) - 1) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_unpack_tiles: too many tiles");
  unpack_tiles_kernel<<<(unsigned)n, kTilePixels, 0, (cudaStream_t)stream>>>(d_tiles, width, height, rank, num_ranks,
                                                                             format, d_out);
  return check_launch("unpack_tiles_kernel");
}

}  // extern "C"
