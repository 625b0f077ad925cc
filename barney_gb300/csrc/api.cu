// api.cu -- status handling, macrocell build and frame-buffer read.
#include <cstdio>
#include <cstring>
#include <string>
#include <cuda_runtime.h>
#include "gbv_volume.cuh"
#include "gbv_internal.h"
#include "../../include/gbvol_diag.h"

namespace gbv {

static thread_local std::string g_last_error;

gbv_status set_error(gbv_status st, const char *msg) {
  g_last_error = msg ? msg : "";
  return st;
}

gbv_status check_cuda(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return GBV_OK;
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  g_last_error = m;
  return e == cudaErrorMemoryAllocation ? GBV_ERROR_OUT_OF_MEMORY : GBV_ERROR_CUDA;
}

gbv_status check_launch(const char *what) { return check_cuda(cudaGetLastError(), what); }

// -------------------------------------------------------------------------
// Macrocell ranges: one warp per macrocell.  The (cpm+1)^3 footprint
// (StructuredData.cu:45-57, inclusive upper corner, clipped to the volume)
// is flattened so consecutive lanes read consecutive x.  min/max are exact,
// so the result is independent of the reduction order.
// -------------------------------------------------------------------------
__global__ void __launch_bounds__(256) mc_ranges_kernel(const float *__restrict__ scalars, int nx, int ny, int nz,
                                                        int cpm, int mx_, int my_, int mz_,
                                                        float2 *__restrict__ ranges) {
  const int lane = threadIdx.x & 31;
  const long long mc = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const long long numMC = (long long)mx_ * my_ * mz_;
  if (mc >= numMC) return;
  const int cx = (int)(mc % mx_), cy = (int)((mc / mx_) % my_), cz = (int)(mc / ((long long)mx_ * my_));
  const int e = cpm + 1;
  // footprint clipped to the volume
  const int x0 = cx * cpm, y0 = cy * cpm, z0 = cz * cpm;
  const int ex = min(e, nx - x0), ey = min(e, ny - y0), ez = min(e, nz - z0);
  const float INF = __int_as_float(0x7f800000);
  float lo = INF, hi = -INF;
  const int total = ex * ey * ez;
  for (int f = lane; f < total; f += 32) {
    const int ix = f % ex;
    const int r = f / ex;
    const int iy = r % ey;
    const int iz = r / ey;
    const float v = __ldg(scalars + (size_t)(x0 + ix) + (size_t)nx * ((size_t)(y0 + iy) + (size_t)ny * (z0 + iz)));
    lo = mn(lo, v);  // interval::extend: NaN never replaces the bound
    hi = mx(hi, v);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = mn(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = mx(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (lane == 0) ranges[mc] = make_float2(lo, hi);
}

// mapMCs (MCGrid.cu:94-116): one thread per macrocell
__global__ void majorants_kernel(const float2 *__restrict__ ranges, long long numMC, const float4 *__restrict__ tf,
                                 int n, float lo, float span, float bd, float *__restrict__ out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= numMC) return;
  float2 r = ranges[i];
  out[i] = xf_majorant(tf, n, lo, span, bd, r.x, r.y);
}

// linearizeColorAndNormalKernel (TiledFB.cu:13-50); make_8bit and
// linear_to_srgb (math.h:52-116) are in gbv_math.cuh
__global__ void tonemap_kernel(const float4 *__restrict__ accum, long long n, float accumScale, int format,
                               void *out) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 a = accum[i];
  float4 c = make_float4(a.x * accumScale, a.y * accumScale, a.z * accumScale, a.w * accumScale);
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

// Normalised integer texels (cudaReadModeNormalizedFloat of the reference's
// CUDA texture objects, rtcore/cudaCommon/TextureData.cu:34-39; the CPU
// backend's getTexel<unsigned char>, rtcore/embree/Texture.cpp:216-225):
// v / 255 or v / 65535, one IEEE division per texel.
template <typename T>
__global__ void normalize_texels_kernel(const T *__restrict__ in, long long n, float scale_max,
                                        float *__restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i] / scale_max;
}

__global__ void sincos_angle_kernel(const float *__restrict__ x, long long n, float *__restrict__ sn,
                                    float *__restrict__ cs) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s, c;
  sincos_angle(x[i], s, c);
  sn[i] = s;
  cs[i] = c;
}

}  // namespace gbv

using namespace gbv;

extern "C" {

const char *gbv_last_error(void) { return g_last_error.c_str(); }
int gbv_version(void) { return 1; }

gbv_status gbv_mc_dims(const int dims[3], int cells_per_mc, int mc_dims[3]) {
  if (!dims || !mc_dims || cells_per_mc <= 0) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_mc_dims: bad argument");
  for (int i = 0; i < 3; i++) {
    if (dims[i] < 0) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_mc_dims: negative dims");
    int cells = dims[i] - 1;
    mc_dims[i] = cells <= 0 ? 0 : (cells + cells_per_mc - 1) / cells_per_mc;
  }
  long long n = (long long)mc_dims[0] * mc_dims[1] * mc_dims[2];
  if (n != (long long)(int)n)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "number of macrocells cannot be expressed in a 32-bit value");
  return GBV_OK;
}

gbv_status gbv_build_mc_ranges(const float *d_scalars, const int dims[3], int cells_per_mc, float *d_ranges,
                               void *stream) {
  int M[3];
  gbv_status st = gbv_mc_dims(dims, cells_per_mc, M);
  if (st != GBV_OK) return st;
  if (!d_scalars || !d_ranges) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_build_mc_ranges: null pointer");
  long long n = (long long)M[0] * M[1] * M[2];
  if (n == 0) return GBV_OK;
  const int warpsPerBlock = 8;
  long long blocks = (n + warpsPerBlock - 1) / warpsPerBlock;
  mc_ranges_kernel<<<(unsigned)blocks, 32 * warpsPerBlock, 0, (cudaStream_t)stream>>>(
      d_scalars, dims[0], dims[1], dims[2], cells_per_mc, M[0], M[1], M[2], reinterpret_cast<float2 *>(d_ranges));
  return check_launch("mc_ranges_kernel");
}

gbv_status gbv_map_majorants(const float *d_ranges, int num_mc, const float *d_tf, int tf_n, float domain_lo,
                             float domain_hi, float base_density, float *d_majorants, void *stream) {
  if (!d_ranges || !d_tf || !d_majorants || num_mc < 0 || tf_n < 2)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_map_majorants: bad argument");
  if (num_mc == 0) return GBV_OK;
  int bs = 256;
  majorants_kernel<<<(num_mc + bs - 1) / bs, bs, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float2 *>(d_ranges), num_mc, reinterpret_cast<const float4 *>(d_tf), tf_n, domain_lo,
      domain_hi - domain_lo, base_density, d_majorants);
  return check_launch("majorants_kernel");
}

gbv_status gbv_tonemap(const float *d_accum, int width, int height, int accum_id, int format, void *d_out,
                       void *stream) {
  if (!d_accum || !d_out || width <= 0 || height <= 0 || accum_id <= 0)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_tonemap: bad argument (accum_id must be >= 1)");
  if (format < GBV_FB_FLOAT4 || format > GBV_FB_RGBA8_SRGB)
    return set_error(GBV_ERROR_UNSUPPORTED, "gbv_tonemap: unsupported format");
  long long n = (long long)width * height;
  float accumScale = 1.f / (float)accum_id;
  tonemap_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float4 *>(d_accum), n, accumScale, format, d_out);
  return check_launch("tonemap_kernel");
}

gbv_status gbv_selftest_sincos(const float *x, long long n, float *sn, float *cs, int on_device, void *stream) {
  if (!x || !sn || !cs || n < 0) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_selftest_sincos: bad argument");
  if (n == 0) return GBV_OK;
  if (!on_device) {
    for (long long i = 0; i < n; i++) sincos_angle(x[i], sn[i], cs[i]);
    return GBV_OK;
  }
  sincos_angle_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(x, n, sn, cs);
  return check_launch("sincos_angle_kernel");
}

__global__ void angles_kernel(const float *__restrict__ y, const float *__restrict__ x, long long n,
                              float *__restrict__ acos_x, float *__restrict__ atan2_yx) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  acos_x[i] = acos_angle(x[i]);
  atan2_yx[i] = atan2_angle(y[i], x[i]);
}

gbv_status gbv_selftest_angles(const float *y, const float *x, long long n, float *acos_x, float *atan2_yx,
                               int on_device, void *stream) {
  if (!y || !x || !acos_x || !atan2_yx || n < 0)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_selftest_angles: bad argument");
  if (n == 0) return GBV_OK;
  if (!on_device) {
    for (long long i = 0; i < n; i++) {
      acos_x[i] = acos_angle(x[i]);
      atan2_yx[i] = atan2_angle(y[i], x[i]);
    }
    return GBV_OK;
  }
  angles_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(y, x, n, acos_x, atan2_yx);
  return check_launch("angles_kernel");
}

gbv_status gbv_normalize_texels(const void *d_texels, int bits, long long n, float *d_scalars, void *stream) {
  if (!d_texels || !d_scalars || n < 0 || (bits != 8 && bits != 16))
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_normalize_texels: bad argument (bits must be 8 or 16)");
  if (n == 0) return GBV_OK;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  if (bits == 8)
    normalize_texels_kernel<uint8_t><<<blocks, 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const uint8_t *>(d_texels), n, 255.f, d_scalars);
  else
    normalize_texels_kernel<uint16_t><<<blocks, 256, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const uint16_t *>(d_texels), n, 65535.f, d_scalars);
  return check_launch("normalize_texels_kernel");
}

}  // extern "C"
