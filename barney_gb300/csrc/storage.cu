// storage.cu -- brick-corner voxel stores and env-map importance tables.
#include <cuda_runtime.h>
#include "gbv_volume.cuh"
#include "gbv_internal.h"

namespace gbv {

__global__ void mc_ranges_kernel(const float *__restrict__ scalars, int nx, int ny, int nz, int cpm, int mx_,
                                 int my_, int mz_, float2 *__restrict__ ranges);

// One thread per cell of the padded brick grid, in store order, so each
// thread writes one contiguous 8-voxel record.  Bricks have 2^lx x 2^ly x
// 2^lz cells; U8 quantizes with the (min, max) of the cell's 8^3 scale brick
// (lohi: nsx x nsy x ... scale bricks).
template <int FMT>
__global__ void brick_store_kernel(const float *__restrict__ s, int nx, int ny, int nz, int nbx, int nby, int lx,
                                   int ly, int lz, int nsx, int nsy, long long numCells,
                                   const float2 *__restrict__ lohi, void *__restrict__ out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= numCells) return;
  const long long brick = t >> (lx + ly + lz);
  const int local = (int)(t & ((1ll << (lx + ly + lz)) - 1));
  const int bx = (int)(brick % nbx), by = (int)((brick / nbx) % nby), bz = (int)(brick / ((long long)nbx * nby));
  const int cx = (bx << lx) | (local & ((1 << lx) - 1)), cy = (by << ly) | ((local >> lx) & ((1 << ly) - 1)),
            cz = (bz << lz) | (local >> (lx + ly));
  const bool inside = cx < nx - 1 && cy < ny - 1 && cz < nz - 1;
  float c[8];
  if (inside) {
    const size_t sy = (size_t)nx, sz = (size_t)nx * ny;
    const size_t b = (size_t)cx + sy * cy + sz * cz;
    c[0] = s[b];
    c[1] = s[b + 1];
    c[2] = s[b + sy];
    c[3] = s[b + sy + 1];
    c[4] = s[b + sz];
    c[5] = s[b + sz + 1];
    c[6] = s[b + sz + sy];
    c[7] = s[b + sz + sy + 1];
  } else {
#pragma unroll
    for (int k = 0; k < 8; k++) c[k] = 0.f;
  }
  if (FMT == GBV_VOXEL_F32) {
    float4 *o = reinterpret_cast<float4 *>(out) + 2 * t;
    o[0] = make_float4(c[0], c[1], c[2], c[3]);
    o[1] = make_float4(c[4], c[5], c[6], c[7]);
  } else if (FMT == GBV_VOXEL_F16) {
    uint32_t w[4];
#pragma unroll
    for (int k = 0; k < 4; k++)
      w[k] = (uint32_t)__half_as_ushort(__float2half_rn(c[2 * k])) |
             ((uint32_t)__half_as_ushort(__float2half_rn(c[2 * k + 1])) << 16);
    reinterpret_cast<uint4 *>(out)[t] = make_uint4(w[0], w[1], w[2], w[3]);
  } else if (FMT == GBV_VOXEL_BF16) {
    uint32_t w[4];
#pragma unroll
    for (int k = 0; k < 4; k++)
      w[k] = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(c[2 * k])) |
             ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(c[2 * k + 1])) << 16);
    reinterpret_cast<uint4 *>(out)[t] = make_uint4(w[0], w[1], w[2], w[3]);
  } else {
    // u8 = round(255 (v - min_b) / (max_b - min_b)) over the scale brick's
    // 9^3 voxels; padding cells (never sampled) store 0
    uint32_t w[2] = {0u, 0u};
    if (inside) {
      const float2 r = lohi[(size_t)(cx >> kScaleBrickLog2) +
                            (size_t)nsx * ((size_t)(cy >> kScaleBrickLog2) + (size_t)nsy * (cz >> kScaleBrickLog2))];
      const float span = r.y - r.x;
#pragma unroll
      for (int k = 0; k < 8; k++) {
        int q = 0;
        if (span > 0.f) q = (int)floorf((c[k] - r.x) * (255.f / span) + .5f);
        q = min(255, max(0, q));
        w[k >> 2] |= (uint32_t)q << (8 * (k & 3));
      }
    }
    reinterpret_cast<uint2 *>(out)[t] = make_uint2(w[0], w[1]);
  }
}

__global__ void lohi_to_scale_offset(float2 *so, long long n) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float2 r = so[i];
  float span = r.y - r.x;
  so[i] = make_float2(span > 0.f ? span / 255.f : 0.f, r.x);
}

// ---- env map tables (EnvMap.cu:61-137) ----
struct EnvTex {
  const float4 *tex;
  int W, H, ax, ay;
};
__device__ __forceinline__ void env_addr(int mode, float tc, int N, int &i0, int &i1, float &f) {
  i0 = 0; i1 = 0; f = 0.f;
  if (mode == GBV_ADDR_WRAP) {
    tc = tc * (float)N - .5f;
    tc = fmodf(tc, (float)N);
    if (tc < 0.f) tc += (float)N;
    float fc = floorf(tc);
    int ic = (int)fc;
    f = tc - (float)ic;
    i0 = ic;
    i1 = (int)fmodf(tc + 1.f, (float)N);
  } else if (mode == GBV_ADDR_MIRROR) {
    tc = tc * (float)N + .5f;
    float fc = floorf(tc);
    int ic = (int)fc;
    f = tc - (float)ic;
    int a = ic - 1, b = ic;
    if (a < 0) a = -a;
    if (b < 0) b = -b;
    a = a % (2 * N);
    b = b % (2 * N);
    if (a >= N) a = 2 * N - 1 - a;
    if (b >= N) b = 2 * N - 1 - b;
    i0 = a;
    i1 = b;
  } else if (mode == GBV_ADDR_CLAMP) {
    tc = tc * (float)N;
    if (tc - .5f <= 0.f) { i0 = i1 = 0; f = 0.f; }
    else if (tc - .5f >= (float)(N - 1)) { i0 = i1 = N - 1; f = 0.f; }
    else {
      f = (tc - .5f) - (float)(int)(tc - .5f);
      i0 = (int)(tc - .5f);
      i1 = i0 + 1;
    }
  }
}
__device__ __forceinline__ float4 env_lerp(float f, float4 a, float4 b) {
  return make_float4((1.f - f) * a.x + f * b.x, (1.f - f) * a.y + f * b.y, (1.f - f) * a.z + f * b.z,
                     (1.f - f) * a.w + f * b.w);
}
__device__ __forceinline__ float4 env_tex2D(const EnvTex &e, float u, float v) {
  int x0, x1, y0, y1;
  float fx, fy;
  env_addr(e.ax, u, e.W, x0, x1, fx);
  env_addr(e.ay, v, e.H, y0, y1, fy);
  float4 v00 = e.tex[x0 + (size_t)y0 * e.W], v01 = e.tex[x1 + (size_t)y0 * e.W];
  float4 v10 = e.tex[x0 + (size_t)y1 * e.W], v11 = e.tex[x1 + (size_t)y1 * e.W];
  return env_lerp(fy, env_lerp(fx, v00, v01), env_lerp(fx, v10, v11));
}
__global__ void env_weights_kernel(EnvTex e, float *cdf_x) {
  int ix = blockIdx.x * blockDim.x + threadIdx.x, iy = blockIdx.y * blockDim.y + threadIdx.y;
  if (ix >= e.W || iy >= e.H) return;
  float weight = 0.f;
  for (int iiy = 0; iiy <= 2; iiy++)
    for (int iix = 0; iix <= 2; iix++) {
      float4 t = env_tex2D(e, ((float)ix + (float)iix * .5f) / (float)e.W, ((float)iy + (float)iiy * .5f) / (float)e.H);
      weight = mx(weight, mx(mx(t.x, t.y), t.z));
    }
  cdf_x[ix + (size_t)e.W * iy] = weight;
}
__global__ void env_lines_kernel(int W, int H, float *cdf_y, float *cdf_x) {
  int y = blockIdx.x * blockDim.x + threadIdx.x;
  if (y >= H) return;
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
  float rel_y = ((float)y + .5f) / (float)H;
  const float theta = kPi * rel_y;
  float sinTheta, cosTheta;
  sincos_angle(theta, sinTheta, cosTheta);  // theta in (0, pi): the renderer's bounded sine
  cdf_y[y] = sum * sinTheta;
}
__global__ void env_normalize_kernel(int H, float *cdf_y) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
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

}  // namespace gbv

using namespace gbv;

extern "C" {

gbv_status gbv_brick_store_bytes_shaped(const int dims[3], int format, const int brick_log2[3], size_t *voxel_bytes,
                                        size_t *scale_offset_bytes) {
  if (!dims || !voxel_bytes) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_brick_store_bytes: null pointer");
  int l[3];
  if (!resolve_brick_shape(brick_log2, l))
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "brick_log2: each 1..6 (0 = 3), sum at most 15");
  int nb[3], ns[3];
  brick_counts(dims, nb, l);
  brick_counts(dims, ns);
  const size_t cells = ((size_t)nb[0] * nb[1] * nb[2]) << (l[0] + l[1] + l[2]);
  size_t elem = 0;
  switch (format) {
    case GBV_VOXEL_F32: elem = 4; break;
    case GBV_VOXEL_F16:
    case GBV_VOXEL_BF16: elem = 2; break;
    case GBV_VOXEL_U8_SCALED: elem = 1; break;
    default: return set_error(GBV_ERROR_UNSUPPORTED, "gbv_brick_store_bytes: unknown format");
  }
  *voxel_bytes = cells * 8 * elem;
  if (scale_offset_bytes)
    *scale_offset_bytes = format == GBV_VOXEL_U8_SCALED ? (size_t)ns[0] * ns[1] * ns[2] * 2 * sizeof(float) : 0;
  return GBV_OK;
}

gbv_status gbv_brick_store_bytes(const int dims[3], int format, size_t *voxel_bytes, size_t *scale_offset_bytes) {
  return gbv_brick_store_bytes_shaped(dims, format, nullptr, voxel_bytes, scale_offset_bytes);
}

gbv_status gbv_build_brick_store_shaped(const float *d_scalars, const int dims[3], int format, const int brick_log2[3],
                                        void *d_voxels, float *d_scale_offset, void *stream) {
  if (!d_scalars || !dims || !d_voxels) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_build_brick_store: null");
  if (dims[0] < 2 || dims[1] < 2 || dims[2] < 2)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_build_brick_store: a volume needs at least 2 voxels per axis");
  if (format == GBV_VOXEL_U8_SCALED && !d_scale_offset)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_build_brick_store: U8 needs the scale/offset table");
  int l[3];
  if (!resolve_brick_shape(brick_log2, l))
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "brick_log2: each 1..6 (0 = 3), sum at most 15");
  int nb[3], ns[3];
  brick_counts(dims, nb, l);
  brick_counts(dims, ns);
  const long long cells = ((long long)nb[0] * nb[1] * nb[2]) << (l[0] + l[1] + l[2]);
  const long long scaleBricks = (long long)ns[0] * ns[1] * ns[2];
  cudaStream_t cs = (cudaStream_t)stream;
  unsigned blocks = (unsigned)((cells + 255) / 256);
  float2 *lohi = reinterpret_cast<float2 *>(d_scale_offset);
#define GBV_STORE_ARGS dims[0], dims[1], dims[2], nb[0], nb[1], l[0], l[1], l[2], ns[0], ns[1], cells
  switch (format) {
    case GBV_VOXEL_F32:
      brick_store_kernel<GBV_VOXEL_F32><<<blocks, 256, 0, cs>>>(d_scalars, GBV_STORE_ARGS, nullptr, d_voxels);
      break;
    case GBV_VOXEL_F16:
      brick_store_kernel<GBV_VOXEL_F16><<<blocks, 256, 0, cs>>>(d_scalars, GBV_STORE_ARGS, nullptr, d_voxels);
      break;
    case GBV_VOXEL_BF16:
      brick_store_kernel<GBV_VOXEL_BF16><<<blocks, 256, 0, cs>>>(d_scalars, GBV_STORE_ARGS, nullptr, d_voxels);
      break;
    case GBV_VOXEL_U8_SCALED: {
      // scale brick (min,max) over 9^3 voxels = the 8-cell macrocell range
      mc_ranges_kernel<<<(unsigned)((scaleBricks + 7) / 8), 256, 0, cs>>>(d_scalars, dims[0], dims[1], dims[2], 8,
                                                                          ns[0], ns[1], ns[2], lohi);
      gbv_status st = check_launch("brick ranges");
      if (st != GBV_OK) return st;
      brick_store_kernel<GBV_VOXEL_U8_SCALED><<<blocks, 256, 0, cs>>>(d_scalars, GBV_STORE_ARGS, lohi, d_voxels);
      st = check_launch("brick_store_kernel");
      if (st != GBV_OK) return st;
      lohi_to_scale_offset<<<(unsigned)((scaleBricks + 255) / 256), 256, 0, cs>>>(lohi, scaleBricks);
      break;
    }
    default:
      return set_error(GBV_ERROR_UNSUPPORTED, "gbv_build_brick_store: unknown format");
  }
#undef GBV_STORE_ARGS
  return check_launch("brick_store_kernel");
}

gbv_status gbv_build_brick_store(const float *d_scalars, const int dims[3], int format, void *d_voxels,
                                 float *d_scale_offset, void *stream) {
  return gbv_build_brick_store_shaped(d_scalars, dims, format, nullptr, d_voxels, d_scale_offset, stream);
}

gbv_status gbv_env_build_cdfs(const float *d_texels, int width, int height, const int addr[2], float *d_cdf_y,
                              float *d_cdf_x, void *stream) {
  if (!d_texels || !d_cdf_y || !d_cdf_x || width <= 0 || height <= 0 || !addr)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_env_build_cdfs: bad argument");
  cudaStream_t cs = (cudaStream_t)stream;
  EnvTex e{reinterpret_cast<const float4 *>(d_texels), width, height, addr[0], addr[1]};
  dim3 bs(16, 16), nb((width + 15) / 16, (height + 15) / 16);
  env_weights_kernel<<<nb, bs, 0, cs>>>(e, d_cdf_x);
  gbv_status st = check_launch("env_weights_kernel");
  if (st != GBV_OK) return st;
  env_lines_kernel<<<(height + 127) / 128, 128, 0, cs>>>(width, height, d_cdf_y, d_cdf_x);
  st = check_launch("env_lines_kernel");
  if (st != GBV_OK) return st;
  env_normalize_kernel<<<1, 1, 0, cs>>>(height, d_cdf_y);
  return check_launch("env_normalize_kernel");
}

}  // extern "C"

namespace gbv {

// Macrocell ranges from a brick-corner store: one warp per macrocell, lanes
// over its cells; each cell contributes the 8 dequantized corners it stores.
template <int FMT>
__global__ void __launch_bounds__(256) mc_ranges_store_kernel(StoreBrickCorners<FMT> store, int cx_, int cy_,
                                                              int cz_, int cpm, int mx_, int my_, int mz_,
                                                              float2 *__restrict__ ranges) {
  const int lane = threadIdx.x & 31;
  const long long mc = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const long long numMC = (long long)mx_ * my_ * mz_;
  if (mc >= numMC) return;
  const int mx0 = (int)(mc % mx_) * cpm, my0 = (int)((mc / mx_) % my_) * cpm,
            mz0 = (int)(mc / ((long long)mx_ * my_)) * cpm;
  const int ex = min(cpm, cx_ - mx0), ey = min(cpm, cy_ - my0), ez = min(cpm, cz_ - mz0);
  const float INF = __int_as_float(0x7f800000);
  float lo = INF, hi = -INF;
  const int total = ex * ey * ez;
  for (int f = lane; f < total; f += 32) {
    const int ix = f % ex, r = f / ex, iy = r % ey, iz = r / ey;
    float c[8];
    store.cell(mx0 + ix, my0 + iy, mz0 + iz, c);
#pragma unroll
    for (int k = 0; k < 8; k++) {
      lo = mn(lo, c[k]);
      hi = mx(hi, c[k]);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = mn(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = mx(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (lane == 0) ranges[mc] = make_float2(lo, hi);
}

}  // namespace gbv

extern "C" gbv_status gbv_build_mc_ranges_from_store_shaped(const void *d_voxels, const float *d_scale_offset,
                                                            int format, const int dims[3], const int brick_log2[3],
                                                            int cells_per_mc, float *d_ranges, void *stream) {
  int M[3];
  gbv_status st = gbv_mc_dims(dims, cells_per_mc, M);
  if (st != GBV_OK) return st;
  if (!d_voxels || !d_ranges) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_build_mc_ranges_from_store: null");
  if (format == GBV_VOXEL_U8_SCALED && !d_scale_offset)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_build_mc_ranges_from_store: U8 needs the scale table");
  int l[3];
  if (!resolve_brick_shape(brick_log2, l))
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "brick_log2: each 1..6 (0 = 3), sum at most 15");
  long long n = (long long)M[0] * M[1] * M[2];
  if (n == 0) return GBV_OK;
  unsigned blocks = (unsigned)((n + 7) / 8);
  cudaStream_t cs = (cudaStream_t)stream;
  float2 *r = reinterpret_cast<float2 *>(d_ranges);
  const int C0 = dims[0] - 1, C1 = dims[1] - 1, C2 = dims[2] - 1;
  const float2 *so = reinterpret_cast<const float2 *>(d_scale_offset);
#define GBV_RANGES(FMT)                                                                                        \
  mc_ranges_store_kernel<FMT><<<blocks, 256, 0, cs>>>(                                                         \
      StoreBrickCorners<FMT>{d_voxels, so, make_brick_geom(dims, l)}, C0, C1, C2, cells_per_mc,             \
      M[0], M[1], M[2], r)
  switch (format) {
    case GBV_VOXEL_F32: GBV_RANGES(GBV_VOXEL_F32); break;
    case GBV_VOXEL_F16: GBV_RANGES(GBV_VOXEL_F16); break;
    case GBV_VOXEL_BF16: GBV_RANGES(GBV_VOXEL_BF16); break;
    case GBV_VOXEL_U8_SCALED: GBV_RANGES(GBV_VOXEL_U8_SCALED); break;
    default:
      return set_error(GBV_ERROR_UNSUPPORTED, "gbv_build_mc_ranges_from_store: unknown format");
  }
#undef GBV_RANGES
  return check_launch("mc_ranges_store_kernel");
}

extern "C" gbv_status gbv_build_mc_ranges_from_store(const void *d_voxels, const float *d_scale_offset, int format,
                                                     const int dims[3], int cells_per_mc, float *d_ranges,
                                                     void *stream) {
  return gbv_build_mc_ranges_from_store_shaped(d_voxels, d_scale_offset, format, dims, nullptr, cells_per_mc,
                                               d_ranges, stream);
}
