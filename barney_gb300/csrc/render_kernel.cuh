// render_kernel.cuh -- the structured-volume frame render on sm_103a: device
// code, the persistent kernel and its launch templates (instantiated once per
// voxel store in render_store_*.cu).
//
// One thread owns one pixel for all of a launch's accumulation passes, so
// the frame buffer needs no atomics and every pixel accumulates its
// fragments in the reference's order (pass-major, then generation; within a
// generation the shadow ray before the bounce ray).  A pass follows
// Context::renderTiles (barney/Context.cpp:142-185): _generateRays, then per
// generation the trace (MCVolumeAccel::isProg) and _shadeRays/bounce
// (barney/kernels/shadeRays.cu:477-1041) of the pixel's queued rays.
#pragma once
#include <cstring>
#include <mutex>
#include <vector>
#include <cuda_runtime.h>
#include "gbv_volume.cuh"
#include "gbv_internal.h"

namespace gbv {

struct DirLightDev { vec3 direction; float radiance; vec3 color; };
struct M3 { vec3 vx, vy, vz; };
__device__ __forceinline__ vec3 xfm_vector(const M3 &m, vec3 v) { return m.vx * v.x + m.vy * v.y + m.vz * v.z; }

struct EnvDev {
  const float4 *tex;
  const float *cdf_y, *cdf_x;
  int W, H;
  int addr[2];
  M3 toWorld, toLocal;
  float scale;
};

struct RenderParams {
  FieldGeom F;
  XF xf;
  MCGridDev G;
  // camera (PerspectiveCamera::commit)
  vec3 lens00, dir00, du, dv;
  int W, H;
  int numDir;
  DirLightDev dir[4];
  int hasEnv;
  EnvDev env;
  float4 bg;
  float ambient;
  int multi, volMS, maxVB;
  float aniso, scatAlb;
  float4 *accum;
  int accumIdStart, spp;
  unsigned long long *counters;
  int *capFlag;   // if set, a loop-cap event stores 1 here (no counting needed)
  int skip;       // empty macrocells crossed per traversal step
  int threshold;  // keep traversing while at least this % of busy lanes trace
  // shared-memory staging (offsets in 32-bit words of the dynamic smem)
  int maskWords;  // >0: bitmask of non-zero majorants staged at offset 0 (a multiple of 4 words)
  const uint32_t *maskSrc;  // the bitmask in HBM (16-byte aligned), staged by one bulk copy; null: by ballots
  int cdfYOff;    // >=0: env cdf_y staged here
  int pivOff;     // >=0: per-row pivots of cdf_x staged here
  int pivPerRow;
  int rowOff;     // >=0: per env-map row (pdf_y, pdf denominator) staged here
  int profile;    // accumulate per-phase cycle counts
  int maskMode;   // 0: the staged bitmask arrives by one bulk copy of a precomputed mask; 1: by ballots
  // voxel store of this scene (see make_store)
  const void *vox;
  const float2 *so;
  BrickGeom brick;
  NvdbGrid nvdb;  // GBV_LAYOUT_NANOVDB: the grid (vox is its buffer)
  vec3 rcpMc;     // 1 / macrocell spacing
  // frame partition across ranks (TiledFB.cu:226-255): with numRanks > 1
  // this launch renders only the 32x32-pixel tiles rank, rank + numRanks, ...
  int rank, numRanks;
  // the world's instances: the volume's stream hash, and an iso-surface
  // (gbv_iso_surface) with its matte material, intersected before the
  // volume when its instance index is the lower one
  uint64_t volHash;
  int hasVolume;
  int isoOn, isoFirst;
  float isoValue, isoDelta, isoAlpha;
  const float2 *isoRanges;
  vec3 isoAlbedo;
  uint64_t isoHash;
  // auxiliary channels (gbv_scene.d_depth, ...; null: not written) and the
  // hit IDs they take
  float *depth;
  int *primId, *instId, *objId;
  int volInst, isoInst, volUser, isoUser;
};

// The reference frame buffer's tiles (TiledFB tileSize) and their
// round-robin assignment to ranks: rank r owns tiles r, r + R, r + 2R, ...
// of the row-major tile grid (TiledFB::resize numActiveTilesThisGPU and
// setTileCoordsKernel, barney/fb/TiledFB.cu:226-255).
constexpr int kRefTile = 32;
__host__ __device__ inline long long owned_ref_tiles(int W, int H, int rank, int numRanks) {
  const long long total = (((long long)W + kRefTile - 1) / kRefTile) * (((long long)H + kRefTile - 1) / kRefTile);
  return total > rank ? (total - rank + numRanks - 1) / numRanks : 0;
}
// 8x4-pixel warp tiles one (non-batched) launch hands out
__host__ __device__ inline long long warp_tile_count(const RenderParams &p) {
  if (p.numRanks > 1) return owned_ref_tiles(p.W, p.H, p.rank, p.numRanks) * 32;
  return (((long long)p.W + 7) >> 3) * (((long long)p.H + 3) >> 2);
}

template <class Store> __device__ __forceinline__ Store make_store(const RenderParams &p);
template <> __device__ __forceinline__ StoreLinearF32 make_store<StoreLinearF32>(const RenderParams &p) {
  return StoreLinearF32{reinterpret_cast<const float *>(p.vox), p.F.N[0], p.F.N[1]};
}
template <> __device__ __forceinline__ StoreNanoVDB make_store<StoreNanoVDB>(const RenderParams &p) {
  return StoreNanoVDB{p.nvdb};
}
#define GBV_BRICK_STORE(FMT)                                                                         \
  template <> __device__ __forceinline__ StoreBrickCorners<FMT> make_store<StoreBrickCorners<FMT>>(  \
      const RenderParams &p) {                                                                       \
    return StoreBrickCorners<FMT>{p.vox, p.so, p.brick};                                             \
  }
GBV_BRICK_STORE(GBV_VOXEL_F32)
GBV_BRICK_STORE(GBV_VOXEL_F16)
GBV_BRICK_STORE(GBV_VOXEL_BF16)
GBV_BRICK_STORE(GBV_VOXEL_U8_SCALED)
#undef GBV_BRICK_STORE

// Dynamic shared memory of the render kernel (layout in RenderParams).
extern __shared__ uint32_t g_smem[];

// One warp per 32 macrocells: bit k of word w is set when macrocell
// 32 w + k has a non-zero majorant (words up to `words`, zero-padded).
static __global__ void __launch_bounds__(256) majorant_mask_kernel(const float *__restrict__ maj, int nmc, int words,
                                                            uint32_t *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  for (int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); w < words;
       w += (int)((gridDim.x * blockDim.x) >> 5)) {
    const int i = w * 32 + lane;
    const float m = i < nmc ? __ldg(maj + i) : 0.f;
    const unsigned b = __ballot_sync(0xffffffffu, m != 0.f);
    if (lane == 0) out[w] = b;
  }
}

// Stages the bitmask of non-zero majorants in shared-memory words
// [0, p.maskWords).  With the precomputed mask in HBM (p.maskSrc) one thread
// issues one bulk copy (cp.async.bulk global -> shared, completion counted
// in bytes on an mbarrier) and every thread waits on the barrier; the wait
// is bounded, and a copy that has not completed in time (which no working
// GPU produces) sets *capFlag and the block builds the mask from the
// majorants with warp ballots instead (the same bits).  Without a
// precomputed mask the warps build it that way directly.  Every thread of
// the block calls this.
__device__ __forceinline__ void stage_majorant_mask(const RenderParams &p) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  bool staged = false;
  if (p.maskSrc) {
    __shared__ __align__(8) unsigned long long mbar;
    const unsigned mb = (unsigned)__cvta_generic_to_shared(&mbar);
    const unsigned bytes = (unsigned)p.maskWords * 4u;
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
              (unsigned)__cvta_generic_to_shared(g_smem)),
          "l"(p.maskSrc), "r"(bytes), "r"(mb)
          : "memory");
    }
    __syncthreads();  // the barrier is initialised before anyone waits on it
    unsigned done = 0;
    for (int it = 0; it < (1 << 20) && !done; it++)
      asm volatile(
          "{\n .reg .pred P;\n mbarrier.try_wait.parity.shared::cta.b64 P, [%1], 0;\n selp.u32 %0, 1, 0, P;\n}"
          : "=r"(done)
          : "r"(mb)
          : "memory");
    staged = __syncthreads_and(done != 0) != 0;
    if (!staged && threadIdx.x == 0 && p.capFlag) *p.capFlag = 1;
  }
  if (!staged) {
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int nmc = p.G.M[0] * p.G.M[1] * p.G.M[2];
    for (int w = warp; w < p.maskWords; w += nwarps) {
      const int i = w * 32 + lane;
      const float m = i < nmc ? __ldg(p.G.maj + i) : 0.f;
      const unsigned b = __ballot_sync(FULL, m != 0.f);
      if (lane == 0) g_smem[w] = b;
    }
  }
}

struct LightSample {
  vec3 radiance, direction;
  float distance, pdf;
};

// fmod(x, y), whose result is exact by definition (x - n y for the integer n
// that truncates x / y, carrying the sign of x).  The wrap addressing of an
// env-map lookup only meets |x| < 2|y|: there the result is x itself, or
// |x| - |y| with the sign of x, a subtraction that is exact because
// |y| <= |x| < 2|y| (Sterbenz's lemma).  Other arguments (and NaN, inf, zero
// y) go to fmodf.  Identical results, a few instructions instead of a
// general remainder.
static __device__ __noinline__ float fmod_general(float x, float y) { return fmodf(x, y); }
__device__ __forceinline__ float fmod_wrap(float x, float y) {
  const float ax = fabsf(x), ay = fabsf(y);
  if (ax < ay) return x;
  if (ax < 2.f * ay) return copysignf(ax - ay, x);
  return fmod_general(x, y);
}

// rtcore/embree/Texture.cpp:25-93, mirror mode (out of line: env maps here
// wrap or clamp)
static __device__ __noinline__ void compute_address_mirror(float tc, int N, int &i0, int &i1, float &f) {
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
}
// rtcore/embree/Texture.cpp:25-93 (normalized coordinates)
__device__ __forceinline__ void compute_address(int mode, float tc, int N, int &i0, int &i1, float &f) {
  i0 = 0; i1 = 0; f = 0.f;
  if (mode == GBV_ADDR_WRAP) {
    tc = tc * (float)N - .5f;
    tc = fmod_wrap(tc, (float)N);
    if (tc < 0.f) tc += (float)N;
    float fc = floorf(tc);
    int ic = (int)fc;
    f = tc - (float)ic;
    i0 = ic;
    i1 = (int)fmod_wrap(tc + 1.f, (float)N);
  } else if (mode == GBV_ADDR_MIRROR) {
    compute_address_mirror(tc, N, i0, i1, f);
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
__device__ __forceinline__ float4 lerp4(float f, float4 a, float4 b) {
  return make_float4((1.f - f) * a.x + f * b.x, (1.f - f) * a.y + f * b.y, (1.f - f) * a.z + f * b.z,
                     (1.f - f) * a.w + f * b.w);
}
// rtcore/embree/Texture.cpp:295-321 (one call site: the shading phase
// fetches the texels of the env-map samples and the miss lookups together)
__device__ __forceinline__ float4 tex2D(const EnvDev &e, float u, float v) {
  int x0, x1, y0, y1;
  float fx, fy;
  compute_address(e.addr[0], u, e.W, x0, x1, fx);
  compute_address(e.addr[1], v, e.H, y0, y1, fy);
  float4 v00 = __ldg(e.tex + (size_t)x0 + (size_t)y0 * e.W), v01 = __ldg(e.tex + (size_t)x1 + (size_t)y0 * e.W);
  float4 v10 = __ldg(e.tex + (size_t)x0 + (size_t)y1 * e.W), v11 = __ldg(e.tex + (size_t)x1 + (size_t)y1 * e.W);
  return lerp4(fy, lerp4(fx, v00, v01), lerp4(fx, v10, v11));
}

// DG.h:97-106 (acos and atan2 by this library's series, gbv_math.cuh)
__device__ __forceinline__ float spherical_theta(vec3 v) { return acos_angle(clampv(v.z, -1.f, 1.f)); }
__device__ __forceinline__ float spherical_phi(vec3 v) {
  float p = atan2_angle(v.y, v.x);
  return (p < 0.f) ? (p + float(2.f * 3.14159265358979323846)) : p;
}
// (theta, phi) of a direction in the env map's frame, for the env-map pdf
// and the env lookup
__device__ __forceinline__ float2 spherical_theta_phi(vec3 v) {
  return make_float2(spherical_theta(v), spherical_phi(v));
}
// EnvMap.h:98-134
__device__ __forceinline__ float cdf_get_pdf(int position, const float *cdf, int N) {
  float at = __ldg(cdf + position);
  float before = position ? __ldg(cdf + position - 1) : 0.f;
  return (float)N * (at - before);
}
__device__ __forceinline__ int sample_cdf(const float *cdf, int N, float v, float &pdf) {
  int begin = 0, end = N;
  while ((end - begin) > 1) {
    int mid = (begin + end) / 2;
    float f_mid = __ldg(cdf + mid - 1);
    if (v < f_mid) end = mid;
    else begin = mid;
  }
  float at = __ldg(cdf + begin);
  float before = begin ? __ldg(cdf + begin - 1) : 0.f;
  pdf = (float)N * (at - before);
  return begin;
}
// cdfGetPDF / sampleCDF on the staged cdf_y (binary search in shared memory)
__device__ __forceinline__ float cdf_y_at(const RenderParams &p, int i) {
  return p.cdfYOff >= 0 ? __int_as_float(g_smem[p.cdfYOff + i]) : __ldg(p.env.cdf_y + i);
}
__device__ __forceinline__ int sample_cdf_y(const RenderParams &p, float v, float &pdf) {
  const int N = p.env.H;
  int begin = 0, end = N;
  while ((end - begin) > 1) {
    int mid = (begin + end) / 2;
    if (v < cdf_y_at(p, mid - 1)) end = mid;
    else begin = mid;
  }
  const float at = cdf_y_at(p, begin);
  const float before = begin ? cdf_y_at(p, begin - 1) : 0.f;
  pdf = (float)N * (at - before);
  return begin;
}
// sampleCDF over one row of cdf_x.  The binary search returns the number of
// entries cdf[0..N-2] that are <= v (the CDF is non-decreasing); with staged
// pivots (the last counted entry of every 32-entry segment) the same count is
// the number of segments whose pivot is <= v, times 32, plus a count inside
// the next segment, whose 32 entries are fetched with independent loads.
static __device__ __noinline__ int sample_cdf_x_pivots(const RenderParams &p, int row, float v, float &pdf) {
  const int N = p.env.W;
  const float *cdf = p.env.cdf_x + (size_t)row * N;
  const float *piv = reinterpret_cast<const float *>(g_smem + p.pivOff) + (size_t)row * p.pivPerRow;
  const int nseg = p.pivPerRow;
  int lo = 0, hi = nseg;  // first segment whose pivot is > v
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (piv[mid] <= v) lo = mid + 1;
    else hi = mid;
  }
  int begin;
  if (lo == nseg) {
    begin = N - 1;
  } else {
    const int s0 = lo * 32;
    const int last = min(s0 + 31, N - 2);
    float seg[32];
#pragma unroll
    for (int k = 0; k < 32; k++) seg[k] = (s0 + k <= last) ? __ldg(cdf + s0 + k) : 0.f;
    int c = 0;
#pragma unroll
    for (int k = 0; k < 32; k++) c += (s0 + k <= last && seg[k] <= v) ? 1 : 0;
    begin = s0 + c;
  }
  const float at = __ldg(cdf + begin);
  const float before = begin ? __ldg(cdf + begin - 1) : 0.f;
  pdf = (float)N * (at - before);
  return begin;
}
__device__ __forceinline__ int sample_cdf_x(const RenderParams &p, int row, float v, float &pdf) {
  if (p.pivOff >= 0) return sample_cdf_x_pivots(p, row, v, pdf);
  return sample_cdf(p.env.cdf_x + (size_t)row * p.env.W, p.env.W, v, pdf);
}

// Code layout.  The render kernel is limited as much by instruction fetch
// as by memory: warps of one SM sit in different phases (start, traverse,
// shade) at once, so the whole loop body is the instruction working set
// (ncu: about 40% of the stall samples of a 1080p launch are "no
// instruction").  The shading helpers are inlined: the trace set-up, the
// texel fetch, the env coordinates and the bounce have one call site each,
// only the env pdf (one call per MIS weight) is duplicated, and no registers
// are saved around calls (measured on the 512^3 frame: +9% against
// out-of-line helpers).  Rarely taken branches (general fmod, mirror addressing, the
// pivot search, subnormal half rounding) stay out of line.
// The two factors of the env-map pdf that depend on the pixel row only
// (EnvMap.h:160-179): the row's marginal pdf and the solid-angle
// denominator 2 pi^2 sin(theta) at the row centre.
__device__ __forceinline__ float2 env_row_terms(const EnvDev &e, int py) {
  const float pdf_y = (float)e.H * (__ldg(e.cdf_y + py) - (py ? __ldg(e.cdf_y + py - 1) : 0.f));
  const float rel_y = ((float)py + .5f) / (float)e.H;
  const float theta2 = kPi * rel_y;
  float sinTheta2, cosTheta2;
  sincos_angle(theta2, sinTheta2, cosTheta2);
  return make_float2(pdf_y, kTwoPi * kPi * sinTheta2);
}
// EnvMap.h:136-180.  With the row terms staged in shared memory (rowOff >= 0,
// computed by the same expressions at kernel start) the pdf is one shared
// and two global loads.
__device__ __forceinline__ float env_pdf(const RenderParams &p, vec3 dir) {
  if (!p.hasEnv) return kOneOverFourPi;
  const EnvDev &e = p.env;
  const float2 tp = spherical_theta_phi(xfm_vector(e.toLocal, dir));
  float theta = tp.x;
  float phi = tp.y;
  float u = phi * kOneOverTwoPi, v = theta * kOneOverPi;
  int px = (int)clampv(u * (float)e.W, 0.f, (float)e.W - 1.f);
  int py = (int)clampv(v * (float)e.H, 0.f, (float)e.H - 1.f);
  const float2 row = p.rowOff >= 0 ? reinterpret_cast<const float2 *>(g_smem + p.rowOff)[py] : env_row_terms(e, py);
  float pdf_x = cdf_get_pdf(px, e.cdf_x + (size_t)py * e.W, e.W);
  return pdf_x * row.x * 1.f / row.y;
}
// EnvMap.h:198-250, in two parts.  The light selection of sampleLights
// needs only the sample's radiance, so the direction and pdf (two
// sine/cosine pairs, a transform and a division) are formed only when the
// env light is the one selected; they use no random numbers, so the random
// stream is consumed exactly as in one piece.
struct EnvPick {
  vec3 radiance; // scale * texel(sx, sy)
  float sx, sy;  // sampled texture coordinates
  float pdfxy;   // pdf_x * pdf_y
};
// The random draws and CDF searches of the sample; the texel at (sx, sy)
// is fetched by the caller (see the shading phase of render_kernel).
__device__ __forceinline__ EnvPick env_pick_coords(const RenderParams &p, Random &r) {
  const EnvDev &e = p.env;
  EnvPick k;
  float r_y = r();
  float r_x = r();
  float pdf_y, pdf_x;
  int iy = sample_cdf_y(p, r_y, pdf_y);
  int ix = sample_cdf_x(p, iy, r_x, pdf_x);
  k.sx = ((float)ix + r()) / (float)e.W;
  k.sy = ((float)iy + r()) / (float)e.H;
  k.pdfxy = pdf_x * pdf_y;
  return k;
}
__device__ __forceinline__ void env_pick_direction(const RenderParams &p, const EnvPick &k, LightSample &s) {
  const EnvDev &e = p.env;
  const float phi = kTwoPi * k.sx;
  const float theta = kPi * k.sy;
  float sinTheta, cosTheta, sinPhi, cosPhi;
  sincos_angle(theta, sinTheta, cosTheta);  // theta in [0, pi]
  sincos_angle(phi, sinPhi, cosPhi);        // phi in [0, 2 pi]
  vec3 d;
  d.z = cosTheta;
  d.x = cosPhi * sinTheta;
  d.y = sinPhi * sinTheta;
  s.direction = xfm_vector(e.toWorld, d);
  s.pdf = k.pdfxy * 1.f / (kTwoPi * kPi * sinTheta);
}

// DG.h:183-193
__device__ __forceinline__ vec3 random_direction(Random &rng) {
#pragma unroll 1
  for (int k = 0; k < 64; k++) {
    vec3 v;
    v.x = 1.f - 2.f * rng();
    v.y = 1.f - 2.f * rng();
    v.z = 1.f - 2.f * rng();
    if (dot(v, v) <= 1.f) return normalize(v);
  }
  return vec3(0.f, 0.f, 1.f);
}

// shadeRays.cu:141-191.  Surf = false: a volume hit, whose normal is zero
// (weight 1); Surf = true: the light's weight is dot(lightDir, N) for the
// front-facing surface normal N.
template <bool Surf = false>
__device__ __forceinline__ bool sample_dir_lights(const RenderParams &p, Random &random, LightSample &ls,
                                                  vec3 N = vec3()) {
  if (p.numDir == 0) return false;
  int lID[2];
  float weights[2];
  float sumWeights = 0.f;
#pragma unroll
  for (int i = 0; i < 2; i++) {
    lID[i] = mn((int)(random() * (float)p.numDir), p.numDir - 1);
    weights[i] = 0.f;
    const DirLightDev &light = p.dir[lID[i]];
    vec3 lr = light.color * light.radiance;
    float weight = 1.f;  // N == 0
    if (Surf) {
      weight = is_zero(N) ? 1.f : dot(-light.direction, N);
      if (weight <= 1e-3f) continue;
    }
    weight *= reduce_max(lr);
    if (weight <= 1e-3f) continue;
    weights[i] = weight;
    sumWeights += weight;
  }
  if (sumWeights == 0.f) return false;
  float r = random() * sumWeights;
  int i = 0;
  while (i < 2 && r >= weights[i]) { r -= weights[i]; ++i; }
  if (i == 2) return false;
  const DirLightDev &light = p.dir[lID[i]];
  ls.direction = -light.direction;
  ls.distance = __int_as_float(0x7f800000);
  ls.radiance = light.color * light.radiance * 1.f / (weights[i] / sumWeights * (2.f / (float)p.numDir));
  ls.pdf = __int_as_float(0x7f800000);
  return weights[i] != 0.f;
}

// shadeRays.cu:268-404 (no area or point lights in this world).  Surf:
// sampling at a surface of front-facing normal N, where the ambient light's
// direction turns into N's hemisphere (radiance 2 pi ambient, pdf 1/(2 pi)).
template <bool Surf = false>
__device__ __forceinline__ bool sample_lights(const RenderParams &p, Random &random, const EnvPick &pick,
                                              LightSample &ls, bool &needsMIS, bool &isDir, vec3 N = vec3()) {
  needsMIS = false;
  LightSample els;
  if (p.hasEnv) {
    els.radiance = pick.radiance;
    els.distance = __int_as_float(0x7f800000);
  } else {
    els.direction = random_direction(random);
    els.distance = __int_as_float(0x7f800000);
    if (Surf && !is_zero(N)) {
      els.radiance = vec3(kTwoPi * p.ambient);
      if (dot(els.direction, N) < 0.f) els.direction = -els.direction;
      els.pdf = kOneOverTwoPi;
    } else {
      els.radiance = vec3(kFourPi * p.ambient);
      els.pdf = kOneOverFourPi;
    }
  }
  float elsWeight = reduce_max(els.radiance);
  LightSample dls;
  dls.pdf = 0.f;
  float dlsWeight = sample_dir_lights<Surf>(p, random, dls, N) ? reduce_max(dls.radiance) : 0.f;
  float alsWeight = 0.f, plsWeight = 0.f;
  float sumWeights = alsWeight + dlsWeight + elsWeight + plsWeight;
  if (sumWeights == 0.f) return false;
  elsWeight *= 1.f / sumWeights;
  alsWeight *= 1.f / sumWeights;
  dlsWeight *= 1.f / sumWeights;
  float r = random();
  if (r <= alsWeight) {
    return false;  // empty area-light sample (pdf 0)
  } else if (r <= alsWeight + elsWeight) {
    if (p.hasEnv) env_pick_direction(p, pick, els);
    ls = els;
    ls.radiance = ls.radiance * (1.f / elsWeight);
    needsMIS = true;
  } else if (r <= alsWeight + elsWeight + plsWeight) {
    return false;
  } else {
    ls = dls;
    ls.radiance = ls.radiance * (1.f / dlsWeight);
    isDir = true;
  }
  if (isnan(ls.pdf) || (ls.pdf <= 0.f)) return false;
  return true;
}

// radianceFromEnv (shadeRays.cu:437-456) up to the texture read: the
// env-map coordinates of a ray direction
__device__ __forceinline__ float2 env_miss_coords(const RenderParams &p, vec3 rayDir) {
  vec3 d = xfm_vector(p.env.toLocal, normalize(rayDir));
  const float2 tp = spherical_theta_phi(d);
  float theta = tp.x;
  float phi = tp.y;
  const float invPi = 1.f / (float)3.14159265358979323846;
  const float inv2Pi = 1.f / (2.f * (float)3.14159265358979323846);
  return make_float2(phi * inv2Pi, theta * invPi);
}

// Phase.h:49-57
__device__ __forceinline__ float hg_phase(float g, float cosTheta) {
  if (fabsf(g) < 1e-3f) return kOneOverFourPi;
  float g2 = g * g;
  float denom = 1.f + g2 - 2.f * g * cosTheta;
  return kOneOverFourPi * (1.f - g2) / (denom * sqrtf(denom));
}
__device__ __forceinline__ float phase_pdf(const RenderParams &p, float g, vec3 wo, vec3 wi) {
  if (!p.multi) return kOneOverFourPi;
  if (fabsf(g) < 1e-3f) return kOneOverFourPi;  // isotropic: no directions needed
  vec3 wi_in = normalize(-wo);
  return hg_phase(g, dot(wi_in, normalize(wi)));
}
// Phase.h:74-99
__device__ __forceinline__ vec3 sample_hg_direction(vec3 wi_in, float g, Random &random) {
  float u0 = random();
  float u1 = random();
  float cosTheta;
  if (fabsf(g) < 1e-3f) cosTheta = 1.f - 2.f * u0;
  else {
    float sqrTerm = (1.f - g * g) / (1.f + g - 2.f * g * u0);
    cosTheta = (1.f + g * g - sqrTerm * sqrTerm) / (2.f * g);
  }
  float sinTheta = sqrtf(mx(0.f, 1.f - cosTheta * cosTheta));
  float phi = kTwoPi * u1;
  float sinPhi, cosPhi;
  sincos_angle(phi, sinPhi, cosPhi);  // phi in [0, 2 pi)
  vec3 local(cosPhi * sinTheta, sinPhi * sinTheta, cosTheta);
  vec3 w = normalize(wi_in);
  vec3 u, v;
  if (fabsf(w.x) > 0.1f) u = normalize(cross(vec3(0.f, 1.f, 0.f), w));
  else u = normalize(cross(vec3(1.f, 0.f, 0.f), w));
  v = cross(w, u);
  return normalize(local.x * u + local.y * v + local.z * w);
}

// Per-ray state of the pixel's path (Ray + PathState, render/Ray.h:18-99)
struct PathRay {
  vec3 org, dir;
  float tMax;
  RNGSeed seed;
  vec3h tp;
  float misWeight;
  int numVolumeBounces;
  int numDiffuseBounces;  // surface bounces (iso-surface worlds only)
};

struct ShadeOut {
  vec3 fragment;
  bool shadowValid;
  PathRay shadow;
};

// bounce() for a volume hit (shadeRays.cu:605-878).  Updates `ray`; a dead
// ray has tMax = -1.
// `random` is the hit's stream, Random2(ray.rngSeed, tHit), already derived
// (it advanced ray.seed); with an env map `pick` holds the light sample's
// texel coordinates and radiance.
__device__ __forceinline__ void bounce_volume_hit(const RenderParams &p, PathRay &ray, const Hit &h, vec3 P,
                                                  int pathDepth, Random &random, const EnvPick &pick,
                                                  ShadeOut &out) {
  out.shadowValid = false;
  const float tHit = h.t;
  const vec3 albedo = p.multi ? p.scatAlb * h.rgb : .7f * h.rgb;
  const float g = p.multi ? p.aniso : 0.f;
  const vec3 incomingThroughput = from_half(ray.tp);
  const vec3 wo = -normalize(ray.dir);
  const float offsetEpsilon = mx(1e-4f, 1e-6f * reduce_max(vabs(P)));
  LightSample ls;
  bool needsMIS = false, isDir = false;
  if (sample_lights(p, random, pick, ls, needsMIS, isDir)) {
    float density = p.multi ? phase_pdf(p, g, wo, ls.direction) : kOneOverFourPi;
    vec3 fr = density * albedo;
    if (!(density > 0.f) || reduce_max(fr) < 1e-4f) {
      out.shadowValid = false;
    } else {
      fr = vmin(fr, vec3(13.f));
      vec3 tp_sr = incomingThroughput * (isinf(ls.pdf) ? 1.f : 1.f / ls.pdf) * fr * ls.radiance * 1.f;
      out.shadow.dir = ls.direction;
      out.shadow.org = P + offsetEpsilon * wo;
      out.shadow.tMax = ls.distance * (1.f - 2.f * offsetEpsilon);
      out.shadow.tp = to_half(tp_sr);
      out.shadow.seed = ray.seed;
      ray.seed.next_h((uint64_t)hit_hash(tHit));
      out.shadow.misWeight = 1.f;
      out.shadowValid = true;
      if (!isDir && needsMIS) {
        float pdf_l = env_pdf(p, ls.direction);
        float pdf_s = p.multi ? phase_pdf(p, g, wo, ls.direction) : kOneOverFourPi;
        out.shadow.misWeight = pdf_l / (pdf_l + pdf_s + 1e-10f);
        if (out.shadow.misWeight < 1e-5f) out.shadowValid = false;
      }
    }
  }
  if (pathDepth >= 10) {  // MAX_PATH_DEPTH
    ray.tMax = -1.f;
    return;
  }
  ray.tMax = __int_as_float(0x7f800000);
  if (!p.multi) {
    // SCI_VIS_MODE: a volume scatter ends the path after its shadow ray
    // (the scatter direction is drawn but never used).
    ray.tMax = -1.f;
    return;
  }
  vec3 wi_in = normalize(-wo);
  vec3 sdir = sample_hg_direction(wi_in, g, random);
  float spdf = hg_phase(g, dot(wi_in, sdir));
  vec3 sf_r = albedo * spdf;
  if (!(spdf > 0.f) || spdf <= 1e-6f) return;
  if (!p.volMS || ray.numVolumeBounces >= p.maxVB) {
    ray.tMax = -1.f;
    return;
  }
  ray.numVolumeBounces = ray.numVolumeBounces + 1;
  ray.org = P + (1.f * offsetEpsilon) * wo;
  ray.dir = normalize(sdir);
  vec3 scatterFactor = sf_r * 1.f / (isinf(spdf) ? 1.f : (spdf + 1e-10f));
  scatterFactor = vmin(scatterFactor, vec3(2.5f));
  ray.tp = to_half(from_half(ray.tp) * scatterFactor);
  if (needsMIS && !isinf(spdf)) {
    float pdf_s = phase_pdf(p, g, wo, ray.dir);
    float pdf_l = env_pdf(p, ray.dir);
    ray.misWeight = pdf_s / (pdf_s + pdf_l);
  } else {
    ray.misWeight = 1.f;
  }
}

// Out-of-line copies of the shading helpers for the batched kernel: its
// lanes read their scenes' parameters from global memory (one record per
// item), and inlined helpers keep more of them live than the registers hold
// (measured on the 64-item workload: 13% slower inlined).  The one-scene
// kernel inlines the helpers themselves.
static __device__ __noinline__ void bounce_volume_hit_ool(const RenderParams &p, PathRay &ray, const Hit &h, vec3 P,
                                                      int pathDepth, Random &random, const EnvPick &pick,
                                                      ShadeOut &out) {
  bounce_volume_hit(p, ray, h, P, pathDepth, random, pick, out);
}
// owl::common::frame: the orthonormal frame about a unit normal N that
// xfmVector(frame(N), v) uses -- dx the longer of (1,0,0) x N and
// (0,1,0) x N, normalized, dy = normalize(N x dx)
__device__ __forceinline__ void frame_of(vec3 N, vec3 &dx, vec3 &dy) {
  const vec3 dx0 = cross(vec3(1.f, 0.f, 0.f), N), dx1 = cross(vec3(0.f, 1.f, 0.f), N);
  dx = normalize(dot(dx0, dx0) > dot(dx1, dx1) ? dx0 : dx1);
  dy = normalize(cross(N, dx));
}
// Lambertian::pdf (packedBSDF/Lambertian.h:46-55): the cosine-hemisphere
// pdf about the normal turned toward wi
__device__ __forceinline__ float lambert_pdf(vec3 Ng, vec3 wi) {
  const vec3 N = dot(wi, Ng) < 0.f ? -Ng : Ng;
  return mx(dot(wi, N), 0.f) * kOneOverPi;
}

// bounce() for an iso-surface hit (shadeRays.cu:541-878 with isVolumeHit
// false), the matte material's Lambertian (AnariMatte.h:50-62,
// packedBSDF/Lambertian.h:57-90): Ng = normalize(ray.N), offsets and light
// sampling along the front-facing normal, the cosine factors of the surface
// branches and a diffuse scatter, at most MAX_DIFFUSE_BOUNCES = 1 per path
// (shadeRays.cu:18, 795-808).  Updates `ray` like bounce_volume_hit.
static __device__ __noinline__ void bounce_surface_hit(const RenderParams &p, PathRay &ray, vec3h Nh, float tHit,
                                                      vec3 P, int pathDepth, Random &random, const EnvPick &pick,
                                                      ShadeOut &out) {
  out.shadowValid = false;
  const vec3 Ng = normalize(from_half(Nh));
  const vec3 Ngff = dot(ray.dir, Ng) < 0.f ? Ng : -Ng;
  const vec3 incomingThroughput = from_half(ray.tp);
  const vec3 wo = -normalize(ray.dir);
  const float offsetEpsilon = mx(1e-4f, 1e-6f * reduce_max(vabs(P)));
  LightSample ls;
  bool needsMIS = false, isDir = false;
  if (sample_lights<true>(p, random, pick, ls, needsMIS, isDir, Ngff)) {
    // Lambertian::eval: the cosine against the unflipped normal
    const float cosThetaI = mx(dot(ls.direction, Ng), 0.f);
    vec3 fr = p.isoAlbedo * kOneOverPi * cosThetaI;
    if (!(cosThetaI * kOneOverPi > 0.f) || reduce_max(fr) < 1e-4f) {
      out.shadowValid = false;
    } else {
      fr = vmin(fr, vec3(13.f));
      vec3 tp_sr = incomingThroughput * (isinf(ls.pdf) ? 1.f : 1.f / ls.pdf) * fr * ls.radiance *
                   (kOneOverPi * fabsf(dot(Ng, ls.direction)));
      out.shadow.dir = ls.direction;
      out.shadow.org = P + offsetEpsilon * Ngff;
      out.shadow.tMax = ls.distance * (1.f - 2.f * offsetEpsilon);
      out.shadow.tp = to_half(tp_sr);
      out.shadow.seed = ray.seed;
      ray.seed.next_h((uint64_t)hit_hash(tHit));
      out.shadow.misWeight = 1.f;
      out.shadowValid = true;
      if (!isDir && needsMIS) {
        const float pdf_l = env_pdf(p, ls.direction);
        const float pdf_s = lambert_pdf(Ng, ls.direction);
        out.shadow.misWeight = pdf_l / (pdf_l + pdf_s + 1e-10f);
        if (out.shadow.misWeight < 1e-5f) out.shadowValid = false;
      }
    }
  }
  if (pathDepth >= 10) {  // MAX_PATH_DEPTH
    ray.tMax = -1.f;
    return;
  }
  ray.tMax = __int_as_float(0x7f800000);
  // Lambertian::scatter: cosineSampleHemisphere (DG.h:135-168) about the
  // normal turned toward wo.  Its vec2f s(random(), random()) takes the
  // second argument's draw first, as the reference's CPU backend (built
  // with gcc, which evaluates arguments right to left) does.
  const vec3 N = dot(wo, Ng) < 0.f ? -Ng : Ng;
  const float r0 = random();
  const float r1 = random();
  const float phi = kTwoPi * r1;
  const float cosTheta = sqrtf(r0);
  const float sinTheta = sqrtf(1.0f - r0);
  float sinPhi, cosPhi;
  sincos_angle(phi, sinPhi, cosPhi);  // phi in [0, 2 pi)
  vec3 dx, dy;
  frame_of(N, dx, dy);
  const vec3 sdir = dx * (cosPhi * sinTheta) + dy * (sinPhi * sinTheta) + N * cosTheta;
  const float spdf = cosTheta * kOneOverPi;
  if (!(spdf > 0.f) || spdf <= 1e-6f) return;  // the ray stays alive unchanged
  if (ray.numDiffuseBounces >= 1) {
    ray.tMax = -1.f;
    return;
  }
  ray.numDiffuseBounces = ray.numDiffuseBounces + 1;
  ray.org = P + (1.f * offsetEpsilon) * Ngff;
  ray.dir = normalize(sdir);
  vec3 scatterFactor = p.isoAlbedo * fabsf(dot(Ng, normalize(ray.dir))) / (isinf(spdf) ? 1.f : (spdf + 1e-10f));
  scatterFactor = vmin(scatterFactor, vec3(2.5f));
  ray.tp = to_half(from_half(ray.tp) * scatterFactor);
  if (needsMIS && !isinf(spdf)) {
    const float pdf_s = lambert_pdf(Ng, ray.dir);
    const float pdf_l = env_pdf(p, ray.dir);
    ray.misWeight = pdf_s / (pdf_s + pdf_l);
  } else {
    ray.misWeight = 1.f;
  }
}

static __device__ __noinline__ float4 tex2D_ool(const EnvDev &e, float u, float v) { return tex2D(e, u, v); }
static __device__ __noinline__ float2 env_miss_coords_ool(const RenderParams &p, vec3 rayDir) {
  return env_miss_coords(p, rayDir);
}
static __device__ __noinline__ EnvPick env_pick_coords_ool(const RenderParams &p, Random &r) {
  return env_pick_coords(p, r);
}

__device__ __forceinline__ void accum_add(float4 &acc, vec3 frag) {
  if (frag.x > 0.f) acc.x += frag.x;
  if (frag.y > 0.f) acc.y += frag.y;
  if (frag.z > 0.f) acc.z += frag.z;
}

// -------------------------------------------------------------------------
// Traversal of one ray through the macrocell grid: dda::dda3 (DDA.h:65-206)
// with Woodcock::sampleRange (Volume.h:188-223) inside each cell of non-zero
// majorant, as set up by MCVolumeAccel::isProg (MCAccelerator.h:569-708).
// The state advances by bounded units so that a warp's lanes stay in one
// loop: per warp iteration a lane makes at most `skip` (default
// kSkipDefault) cell tests and distance draws to reach its next sample
// position, then the warp's ready lanes take their density samples together.
// -------------------------------------------------------------------------
// Defaults of the launch shape (the best of a same-box sweep of 3..64 units
// per seek and thresholds 3..30% on the 512^3 1080p frame; units 5..8 with
// thresholds 16..25 are within 1% of each other; results never depend on
// them)
constexpr int kSkipDefault = 6;
constexpr int kThresholdDefault = 20;

// Per-lane event counts; with On == false the counting and its registers
// compile away (timed launches pass no counter buffer).
template <bool On> struct Ctr {
  static constexpr bool kOn = On;
  unsigned samples = 0, mcs = 0, rays = 0, caps = 0, cells = 0;
};
#define GBV_COUNT(cnt, field) \
  do {                       \
    if (cnt.kOn) cnt.field++; \
  } while (0)
constexpr int kWoodcockCap = 1 << 20;
enum { TR_CONTINUE = 0, TR_HIT = 1, TR_MISS = 2 };

struct Traversal {
  vec3 org, dir;   // trace direction: zero components replaced by 1e-6
  float rayTMax;   // ray.tMax of the ray record
  vec3 t_next, t_step;
  int cx, cy, cz;
  int stopx, stopy, stopz;
  float ray_t0, tMax, ncb;
  float tc;            // t_closest of the current cell
  float t, segHi, maj; // delta tracking in the current cell
  Random rng;
  int inCell;
  int steps;           // Woodcock steps in the current cell
  int cells;           // cells visited
};

__device__ __forceinline__ float majorant_at(const MCGridDev &G, int cx, int cy, int cz) {
  return __ldg(G.maj + (cx + G.M[0] * (cy + G.M[1] * cz)));
}

// Box test, RNG stream and DDA set-up.  Returns false when the ray reaches
// no cell.  `seed` advances exactly when the reference advances ray.rngSeed
// (once the box test passes); the stream is Random2(seed, streamHash), the
// hash of the geometry's instance (hash(0, 0, 0) for a lone volume).
template <class Cnt>
__device__ __forceinline__ bool trace_begin(const FieldGeom &F, const MCGridDev &G, const vec3 &rcpMc, vec3 org,
                                            vec3 rayDir, float rayTMax, RNGSeed &seed, Traversal &T, Cnt &cnt,
                                            uint64_t streamHash = kVolumeStreamHash) {
  GBV_COUNT(cnt, rays);
  vec3 dir = rayDir;
  if (dir.x == 0.f) dir.x = 1e-6f;
  if (dir.y == 0.f) dir.y = 1e-6f;
  if (dir.z == 0.f) dir.z = 1e-6f;
  if (G.M[0] <= 0 || G.M[1] <= 0 || G.M[2] <= 0) return false;
  float tLo = 0.f, tHi = rayTMax;
  if (!box_test(org, dir, tLo, tHi, F.boundsLo, F.boundsHi)) return false;
  const vec3 dda_org = (org - G.origin) * rcpMc;
  const vec3 dda_dir = dir * rcpMc;
  T.rng = Random::derive(seed, streamHash);
  const float tMax = tHi;
  const vec3 f_size((float)G.M[0], (float)G.M[1], (float)G.M[2]);
  const vec3 rcp_dir = rcp(dda_dir);
  vec3 t_lo = (vec3(0.f) - dda_org) * rcp_dir;
  vec3 t_hi = (f_size - dda_org) * rcp_dir;
  vec3 t_nr = vmin(t_lo, t_hi), t_fr = vmax(t_lo, t_hi);
  const float INF = __int_as_float(0x7f800000);
  if (dda_dir.x == 0.f) {
    if (dda_org.x < 0.f || dda_org.x > f_size.x) return false;
    t_nr.x = -INF; t_fr.x = INF;
  }
  if (dda_dir.y == 0.f) {
    if (dda_org.y < 0.f || dda_org.y > f_size.y) return false;
    t_nr.y = -INF; t_fr.y = INF;
  }
  if (dda_dir.z == 0.f) {
    if (dda_org.z < 0.f || dda_org.z > f_size.z) return false;
    t_nr.z = -INF; t_fr.z = INF;
  }
  const float ray_t0 = mx(0.f, reduce_max(t_nr));
  const float ray_t1 = mn(tMax, reduce_min(t_fr));
  if (ray_t0 > ray_t1) return false;
  const vec3 oiv = dda_org + ray_t0 * dda_dir;
  const vec3 f_cell = vmax(vec3(0.f), vmin(f_size - vec3(1.f), vfloor(oiv)));
  const vec3 f_end(dda_dir.x > 0.f ? f_cell.x + 1.f : f_cell.x, dda_dir.y > 0.f ? f_cell.y + 1.f : f_cell.y,
                   dda_dir.z > 0.f ? f_cell.z + 1.f : f_cell.z);
  T.t_step = vabs(rcp_dir);
  T.t_next = vec3((dda_dir.x == 0.f) ? INF : (fabsf(f_end.x - oiv.x) * T.t_step.x),
                  (dda_dir.y == 0.f) ? INF : (fabsf(f_end.y - oiv.y) * T.t_step.y),
                  (dda_dir.z == 0.f) ? INF : (fabsf(f_end.z - oiv.z) * T.t_step.z));
  T.stopx = dda_dir.x > 0.f ? G.M[0] : -1;
  T.stopy = dda_dir.y > 0.f ? G.M[1] : -1;
  T.stopz = dda_dir.z > 0.f ? G.M[2] : -1;
  T.cx = (int)f_cell.x;
  T.cy = (int)f_cell.y;
  T.cz = (int)f_cell.z;
  T.ray_t0 = ray_t0;
  T.tMax = tMax;
  T.ncb = 0.f;
  T.org = org;
  T.dir = dir;
  T.rayTMax = rayTMax;
  T.inCell = 0;
  T.cells = 0;
  return true;
}

// next_cell_begin = t_closest, then step every axis whose t_next equals it
__device__ __forceinline__ bool trace_advance(Traversal &T, float tc, bool sx, bool sy, bool sz) {
  T.ncb = tc;
  if (T.t_next.x == tc) {
    T.t_next.x += T.t_step.x;
    T.cx += sx ? 1 : -1;
    if (T.cx == T.stopx) return false;
  }
  if (T.t_next.y == tc) {
    T.t_next.y += T.t_step.y;
    T.cy += sy ? 1 : -1;
    if (T.cy == T.stopy) return false;
  }
  if (T.t_next.z == tc) {
    T.t_next.z += T.t_step.z;
    T.cz += sz ? 1 : -1;
    if (T.cz == T.stopz) return false;
  }
  return true;
}

// The traversal is split so that the expensive part, the density sample,
// runs for all of a warp's tracing lanes at once.  trace_seek advances a lane
// to its next sample position: it crosses empty macrocells, enters the next
// cell of non-zero majorant and draws Woodcock distances until one falls
// inside the current cell (T.inCell = 2: a position is ready), at most
// `units` cell tests and distance draws per call.  trace_sample then
// samples there and makes the accept test.  Every lane performs exactly the
// operations, in exactly the order, of the one-step-at-a-time loop
// (dda::dda3 with Woodcock::sampleRange inside each cell); only the grouping
// of a lane's steps into warp iterations differs.
template <class Cnt>
__device__ __forceinline__ int trace_seek(const MCGridDev &G, Traversal &T, Cnt &cnt, int units, bool staged,
                                          int *capFlag) {
  const bool sx = T.stopx >= 0, sy = T.stopy >= 0, sz = T.stopz >= 0;
  const int maxCells = G.M[0] + G.M[1] + G.M[2] + 8;
  for (int k = 0; k < units; k++) {
    if (!T.inCell) {
      GBV_COUNT(cnt, cells);
      if (++T.cells > maxCells) {
        GBV_COUNT(cnt, caps);
        if (capFlag) *capFlag = 1;
        return TR_MISS;
      }
      const float tc = reduce_min(T.t_next);
      const int ci = T.cx + G.M[0] * (T.cy + G.M[1] * T.cz);
      const bool nonzero = staged ? ((g_smem[ci >> 5] >> (ci & 31)) & 1u) != 0u : __ldg(G.maj + ci) != 0.f;
      if (!nonzero) {
        if (!trace_advance(T, tc, sx, sy, sz)) return TR_MISS;
        continue;
      }
      const float maj = __ldg(G.maj + ci);
      const float cell_t0 = T.ray_t0 + T.ncb;
      const float cell_t1 = T.ray_t0 + mn(tc, T.tMax);
      T.inCell = 1;
      T.tc = tc;
      T.maj = maj;
      T.t = cell_t0;
      T.segHi = mn(cell_t1, T.rayTMax);
      T.steps = 0;
      GBV_COUNT(cnt, mcs);
    }
    // one Woodcock distance
    const float r = T.rng();
    const float dt = -fastLog(1.f - r) / T.maj;
    T.t += dt;
    if (T.t >= T.segHi || ++T.steps > kWoodcockCap) {
      if (T.steps > kWoodcockCap) {
        GBV_COUNT(cnt, caps);
        if (capFlag) *capFlag = 1;
      }
      T.inCell = 0;
      if (!trace_advance(T, T.tc, sx, sy, sz)) return TR_MISS;
      continue;
    }
    T.inCell = 2;
    return TR_CONTINUE;
  }
  return TR_CONTINUE;
}

template <class Store, class Cnt>
__device__ __forceinline__ int trace_sample(const FieldGeom &F, const Store &store, const XF &xf, Traversal &T,
                                            Hit &h, Cnt &cnt) {
  T.inCell = 1;
  const vec3 P = T.org + T.t * T.dir;
  const vec4 smp = sample_and_map(F, store, xf, P);
  GBV_COUNT(cnt, samples);
  if (smp.w >= T.rng() * T.maj) {
    h.hit = true;
    h.t = T.t;
    h.rgb = vec3(smp.x, smp.y, smp.z);
    return TR_HIT;
  }
  return TR_CONTINUE;
}

// The hit search and normal of MCIsoSurfaceAccel::isProg
// (MCAccelerator.h:393-503) along a DDA that trace_begin set up: per
// macrocell whose scalar range holds the iso value, the cell's t range is
// cut into 10 sub-steps; the first sub-step whose end values bracket the
// value gives the hit t by linear interpolation.  The normal is the central
// difference of the field at +-delta per axis, one-sided where a sample
// falls outside the field, normalized.  Returns whether t < tmax.
// `stop`: the search may end before a macrocell that begins beyond it (a
// crossing found there would lie beyond `stop`: an interpolated t is never
// more than a few ulps below its cell's start, far inside the 1e-5 margin);
// +inf searches the whole ray.
template <class Store>
__device__ __forceinline__ bool iso_search(const FieldGeom &F, const Store &renderStore, const MCGridDev &G,
                                           const float2 *__restrict__ ranges, float iso, float delta, Traversal &T,
                                           float tmax, float &tOut, vec3 &N,
                                           float stop = __int_as_float_hd(0x7f800000)) {
  // the sub-steps' samples lie close together along the ray: read through L1
  const auto &store = via_l1(renderStore);
  const bool sx = T.stopx >= 0, sy = T.stopy >= 0, sz = T.stopz >= 0;
  const int maxCells = G.M[0] + G.M[1] + G.M[2] + 8;
  float tHit = tmax;
  bool stopped = false;
#pragma unroll 1
  for (int it = 0; it < maxCells; it++) {
    const float tc = reduce_min(T.t_next);
    const float t0 = T.ray_t0 + T.ncb;
    const float t1 = T.ray_t0 + mn(tc, T.tMax);
    if (t0 > stop + fabsf(stop) * 1e-5f) break;
    // the iso lambda (MCAccelerator.h:405-471)
    if (!(t0 >= mn(t1, tmax))) {
      const float2 vr = __ldg(ranges + (T.cx + G.M[0] * (T.cy + G.M[1] * T.cz)));
      if (iso >= vr.x && iso <= vr.y) {
        float tt1 = t0;
        float ff1 = sample_field(F, store, T.org + tt1 * T.dir);
#pragma unroll 1
        for (int i = 1; i <= 10; i++) {
          const float tt0 = tt1;
          const float ff0 = ff1;
          tt1 = lerp_l((float)i / 10.f, t0, t1);
          ff1 = sample_field(F, store, T.org + tt1 * T.dir);
          if (isnan(ff0) || isnan(ff1)) continue;
          if (iso >= mn(ff0, ff1) && iso <= mx(ff0, ff1)) {
            float t = (iso - ff0) / (ff1 - ff0);
            t = lerp_l(t, tt0, tt1);
            tHit = mn(tHit, t);
            if (tHit < tmax) {
              stopped = true;
              break;
            }
          }
        }
      }
    }
    if (stopped || !trace_advance(T, tc, sx, sy, sz)) break;
  }
  if (!(tHit < tmax)) return false;
  const vec3 P = T.org + tHit * T.dir;
  const float d = delta;
  const float fP = sample_field(F, store, P);
  float fx0 = sample_field(F, store, P + vec3(-d, 0.f, 0.f));
  float fx1 = sample_field(F, store, P + vec3(+d, 0.f, 0.f));
  float fy0 = sample_field(F, store, P + vec3(0.f, -d, 0.f));
  float fy1 = sample_field(F, store, P + vec3(0.f, +d, 0.f));
  float fz0 = sample_field(F, store, P + vec3(0.f, 0.f, -d));
  float fz1 = sample_field(F, store, P + vec3(0.f, 0.f, +d));
  float dx = 2.f, dy = 2.f, dz = 2.f;
  if (isnan(fx0)) { dx -= 1.f; fx0 = fP; }
  if (isnan(fx1)) { dx -= 1.f; fx1 = fP; }
  if (isnan(fy0)) { dy -= 1.f; fy0 = fP; }
  if (isnan(fy1)) { dy -= 1.f; fy1 = fP; }
  if (isnan(fz0)) { dz -= 1.f; fz0 = fP; }
  if (isnan(fz1)) { dz -= 1.f; fz1 = fP; }
  N = vec3(dx == 0.f ? 0.f : (fx1 - fx0) / dx, dy == 0.f ? 0.f : (fy1 - fy0) / dy,
           dz == 0.f ? 0.f : (fz1 - fz0) / dz);
  if (is_zero(N)) N = -normalize(T.dir);
  N = normalize(N);
  tOut = tHit;
  return true;
}

// The iso-surface's intersection program for a render ray (org, rayDir,
// [0, tmax]): the box test and the geometry's random stream
// Random2(seed, hash(instance, 0, 0)), which advances `seed`; the hit
// search; the material's opacity test (opacity < 1: the ray passes when
// rng() > opacity, MCAccelerator.h:533-539); and Ray::setHit's record (the
// hit point and the normal in half precision).  Returns whether the surface
// records a hit.
// The iso-surface's box test and random stream alone -- what its
// intersection program does to the ray's seed -- when it runs before the
// volume's: the search itself waits until the volume's first collision is
// known (iso_trace_after).  Returns whether the box test passed; the stream's
// state goes to *rng.
__device__ __forceinline__ bool iso_begin(const RenderParams &p, vec3 org, vec3 rayDir, float tmax, RNGSeed &seed,
                                          uint64_t &rng) {
  vec3 dir = rayDir;
  if (dir.x == 0.f) dir.x = 1e-6f;
  if (dir.y == 0.f) dir.y = 1e-6f;
  if (dir.z == 0.f) dir.z = 1e-6f;
  if (p.G.M[0] <= 0 || p.G.M[1] <= 0 || p.G.M[2] <= 0) return false;
  float tLo = 0.f, tHi = tmax;
  if (!box_test(org, dir, tLo, tHi, p.F.boundsLo, p.F.boundsHi)) return false;
  rng = Random::derive(seed, p.isoHash).s.state;
  return true;
}

// The rest of that program, after the volume traced without the surface's
// bound and found its first collision at `stop` (+inf: none): the search on
// the ray's own [0, tmax], as the program makes it, ends at `stop`; the
// surface's hit counts when its t is at most `stop` (the volume's tracking,
// bounded by the surface's hit, would have stopped there: the surface wins a
// tie), after the material's opacity test on the stream iso_begin made.
// The final hit, point, normal and every random stream equal those of
// running the surface's program first.
template <class Store>
static __device__ __noinline__ bool iso_trace_after(const RenderParams &p, vec3 org, vec3 rayDir, float tmax,
                                                    float stop, uint64_t rng, float &tOut, vec3 &P, vec3h &Nh) {
  Traversal T;
  Ctr<false> none;
  RNGSeed scratch;  // the stream was derived by iso_begin
  scratch.state = 0;
  if (!trace_begin(p.F, p.G, p.rcpMc, org, rayDir, tmax, scratch, T, none, p.isoHash)) return false;
  float t;
  vec3 N;
  if (!iso_search(p.F, make_store<Store>(p), p.G, p.isoRanges, p.isoValue, p.isoDelta, T, tmax, t, N, stop))
    return false;
  if (!(t <= stop)) return false;
  Random r;
  r.s.state = rng;
  if (p.isoAlpha < 1.f && r() > p.isoAlpha) return false;
  tOut = t;
  P = T.org + t * T.dir;
  Nh = to_half(N);
  return true;
}

template <class Store>
static __device__ __noinline__ bool iso_trace(const RenderParams &p, vec3 org, vec3 rayDir, float tmax, RNGSeed &seed,
                                              float &tOut, vec3 &P, vec3h &Nh) {
  Traversal T;
  Ctr<false> none;
  if (!trace_begin(p.F, p.G, p.rcpMc, org, rayDir, tmax, seed, T, none, p.isoHash)) return false;
  float t;
  vec3 N;
  if (!iso_search(p.F, make_store<Store>(p), p.G, p.isoRanges, p.isoValue, p.isoDelta, T, tmax, t, N))
    return false;
  if (p.isoAlpha < 1.f && T.rng() > p.isoAlpha) return false;
  tOut = t;
  P = T.org + t * T.dir;
  Nh = to_half(N);
  return true;
}

// The auxiliary channels of pixel px from its primary ray (shadeRays.cu:
// 1003-1023): pass 0 writes the depth (the ray's tMax: the closest hit's t,
// or the generated 1e30 on a miss) and the closest hit's IDs (primitive 0 of
// the user geometry, its instance index and userID; -1 on a miss); later
// passes keep the smaller depth.  The lane owns the pixel: no atomics.
static __device__ __noinline__ void write_aux(const RenderParams &p, size_t px, int accumID, float z, int hitKind) {
  if (accumID == 0) {
    if (p.depth) p.depth[px] = z;
    if (p.primId) p.primId[px] = hitKind ? 0 : -1;
    if (p.instId) p.instId[px] = hitKind == 1 ? p.volInst : hitKind == 2 ? p.isoInst : -1;
    if (p.objId) p.objId[px] = hitKind == 1 ? p.volUser : hitKind == 2 ? p.isoUser : -1;
  } else if (p.depth && z < p.depth[px]) {
    p.depth[px] = z;
  }
}

// -------------------------------------------------------------------------
// The persistent frame kernel.  Each lane owns one pixel for all of the
// launch's passes, so fragments accumulate in the reference's order
// (pass-major, generation, shadow ray before bounce ray) without atomics.
// Warps take 8x4-pixel tiles from a global pool; a lane whose pixel is done
// takes the next pixel of its warp's tile.  Every loop iteration advances a
// lane by one bounded unit: a trace step, or a shade and the set-up of the
// next trace.
// -------------------------------------------------------------------------
// 9 warps per block: at 4 resident blocks per SM (36 warps) the register
// budget is 56 per thread (measured fastest: 256 x 5 with 48 registers
// -4.2%, 192 x 6 -2%)
constexpr int kThreads = 288;
enum { K_NONE = 0, K_MAIN = 1, K_SHADOW = 2 };

__device__ __forceinline__ float4 miss_color(const RenderParams &p, int iy) {
  const float t = ((float)iy + .5f) / (float)p.H;
  float4 m = p.bg;
  if (!(p.bg.w >= 0.f)) {
    m.x = (1.0f - t) * 0.9f + t * 0.15f;
    m.y = (1.0f - t) * 0.9f + t * 0.25f;
    m.z = (1.0f - t) * 0.9f + t * .8f;
    m.w = (1.0f - t) * 1.f + t * 1.f;
  }
  return m;
}

// _generateRays (generateRays.cu:72-243), perspective camera, no aperture
__device__ __forceinline__ void generate_primary(const RenderParams &p, int ix, int iy, int accumID, PathRay &ray) {
  const float aspect = (float)p.W / (float)p.H;
  Random rand = Random::from_pair((unsigned)(ix + p.W * accumID), (unsigned)(iy + p.H * accumID));
  ray.seed = seeded((uint32_t)(ix + accumID * p.W), (uint32_t)iy);
  const float pixel_u = (accumID == 0) ? .5f : rand();
  const float pixel_v = (accumID == 0) ? .5f : rand();
  const float image_u = ((float)ix + pixel_u) / (float)p.W;
  const float image_v = ((float)iy + pixel_v) / (float)p.H;
  const vec3 d = p.dir00 + (1.f * aspect * (image_u - .5f)) * p.du + (1.f * (image_v - .5f)) * p.dv;
  ray.org = p.lens00;
  ray.dir = normalize(d);
  ray.tMax = 1e30f;
  ray.tp = vec3h{0x3c00, 0x3c00, 0x3c00};  // 1.0 in half
  ray.misWeight = 0.f;
  ray.numVolumeBounces = 0;
  ray.numDiffuseBounces = 0;
}

// Batch: the launch renders `numItems` scenes (items[]), whose 8x4-pixel
// tiles are numbered consecutively (tileStart[] holds the prefix sums); a
// lane reads the scene of the pixel it owns.  Otherwise the launch renders
// the one scene `p0`.  Launch-wide settings (passes, thresholds, counters)
// always come from p0.  Count: whether to count events (see Ctr) and, with
// a profile requested in the launch config (gbv_render_config.profile),
// cycles and lanes per phase (the timed kernel, Count =
// false, carries no profiling code).
// p0 is __grid_constant__ so that helpers (inlined, or the batched kernel's
// out-of-line copies) can take it by reference without a copy to local
// memory.
// Iso: the world holds an iso-surface (p0.isoOn; never batched): each trace
// also runs its intersection program, before the volume's when its instance
// index is the lower one (p0.isoFirst) and otherwise after it, each bounded
// by the other's hit, and shading takes the surface branch on its hits.
template <class Store, int MinBlocks, bool Batch, bool Count, bool Iso = false>
__global__ void __launch_bounds__(kThreads, MinBlocks)
    render_kernel(const __grid_constant__ RenderParams p0, const RenderParams *__restrict__ items,
                  const long long *__restrict__ tileStart, int numItems, int *__restrict__ pool) {
  static_assert(!(Iso && Batch), "batched launches render volume-only worlds");
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const RenderParams &L = p0;  // launch-wide settings
  // ---- stage the majorant bitmask and env-map tables in shared memory ----
  if (!Batch) {
    const RenderParams &p = p0;
    if (p.maskWords > 0) stage_majorant_mask(p);
    if (p.cdfYOff >= 0)
      for (int i = threadIdx.x; i < p.env.H; i += blockDim.x) g_smem[p.cdfYOff + i] = __float_as_uint(__ldg(p.env.cdf_y + i));
    if (p.pivOff >= 0) {
      const int total = p.env.H * p.pivPerRow;
      for (int i = threadIdx.x; i < total; i += blockDim.x) {
        const int row = i / p.pivPerRow, k = i - row * p.pivPerRow;
        const int last = min(k * 32 + 31, p.env.W - 2);
        g_smem[p.pivOff + i] = __float_as_uint(__ldg(p.env.cdf_x + (size_t)row * p.env.W + last));
      }
    }
    if (p.rowOff >= 0)
      for (int i = threadIdx.x; i < p.env.H; i += blockDim.x)
        reinterpret_cast<float2 *>(g_smem + p.rowOff)[i] = env_row_terms(p.env, i);
    __syncthreads();
  }
  const long long numTiles = Batch ? tileStart[numItems] : warp_tile_count(p0);
  Ctr<Count> cnt;
  // warp-uniform tile pool
  int tile = 0, tileTaken = 32, tileItem = 0;
  bool poolDone = false;
  int item = 0;  // scene of the lane's pixel
  // lane state
  enum { NEED = 0, TRACING = 1, DONE = 2 };
  bool hasPixel = false;
  int ix = 0, iy = 0, s = 0, gen = 0, kind = K_NONE, tstate = NEED;
  bool newSample = false, mainAlive = false, shadowPending = false;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  PathRay ray, sray;
  Traversal T;
  Hit h;
  h.hit = false;
  // the iso-surface's hit of the current trace (Iso only); with the
  // surface's instance first, whether its box test passed and its stream
  bool sHit = false;
  float sT = 0.f;
  vec3 sP;
  vec3h sN{0, 0, 0};
  bool isoBox = false;
  uint64_t isoRng = 0;
  unsigned long long cyc[3] = {0ull, 0ull, 0ull};
  // profile: traversal iterations and tracing lanes summed over them, shading
  // passes and shaded lanes summed over them (lane 0 of each warp counts)
  unsigned long long simt[4] = {0ull, 0ull, 0ull, 0ull};
  while (true) {
    // ---- phase 1: pixels for idle lanes (from the warp's tile), then every
    // lane that needs one starts its next trace ----
    const unsigned need = __ballot_sync(FULL, !hasPixel);
    if (need != 0u && !poolDone) {
      if (tileTaken == 32) {
        int t = 0;
        if (lane == 0) t = atomicAdd(pool, 1);
        t = __shfl_sync(FULL, t, 0);
        if (t >= numTiles) {
          poolDone = true;
        } else {
          tileTaken = 0;
          if (Batch) {  // item owning global tile t: last i with tileStart[i] <= t
            int lo = 0, hi = numItems - 1;
            while (lo < hi) {
              const int mid = (lo + hi + 1) >> 1;
              if (tileStart[mid] <= t) lo = mid;
              else hi = mid - 1;
            }
            tileItem = lo;
            tile = (int)(t - tileStart[lo]);
          } else {
            tile = t;
          }
        }
      }
      if (!poolDone) {
        const RenderParams &tp = Batch ? items[tileItem] : p0;
        // the warp tile's upper-left pixel
        int tx, ty;
        if (!Batch && L.numRanks > 1) {  // the k-th 32x32 tile this rank owns, 4x8 warp tiles in it
          const long long big = (long long)L.rank + (long long)(tile >> 5) * L.numRanks;
          const int bigX = (int)(((long long)tp.W + kRefTile - 1) / kRefTile);
          tx = (int)(big % bigX) * kRefTile + (tile & 3) * 8;
          ty = (int)(big / bigX) * kRefTile + ((tile >> 2) & 7) * 4;
        } else {
          const int tilesX = (int)(((long long)tp.W + 7) >> 3);
          tx = (tile % tilesX) * 8;
          ty = (tile / tilesX) * 4;
        }
        const int rank = __popc(need & ((1u << lane) - 1u));
        const int take = min(__popc(need), 32 - tileTaken);
        if (!hasPixel && rank < take) {
          const int slot = tileTaken + rank;
          const int px = tx + (slot & 7), py = ty + (slot >> 3);
          if (px < tp.W && py < tp.H) {
            hasPixel = true;
            item = tileItem;
            ix = px;
            iy = py;
            s = 0;
            newSample = true;
            tstate = NEED;
            acc = L.accumIdStart == 0 ? make_float4(0.f, 0.f, 0.f, 0.f) : tp.accum[(size_t)iy * tp.W + ix];
          }
        }
        tileTaken += take;
      }
    }
    if (poolDone && __all_sync(FULL, !hasPixel)) break;
    const RenderParams &p = Batch ? items[item] : p0;
    long long c0 = (Count && L.profile) ? clock64() : 0;
    if (hasPixel && tstate == NEED) {
      if (newSample) {
        generate_primary(p, ix, iy, L.accumIdStart + s, ray);
        gen = 0;
        mainAlive = true;
        shadowPending = false;
        newSample = false;
      }
      h.hit = false;
      kind = shadowPending ? K_SHADOW : K_MAIN;
      RNGSeed seed = shadowPending ? sray.seed : ray.seed;
      bool active;
      if (Iso) {
        const vec3 org = shadowPending ? sray.org : ray.org, dir = shadowPending ? sray.dir : ray.dir;
        float tmax = shadowPending ? sray.tMax : ray.tMax;
        sHit = false;
        isoBox = false;
        if (!p.hasVolume) GBV_COUNT(cnt, rays);
        // the surface's instance first: its box test and stream now, its
        // search once the volume's collision is known (iso_trace_after)
        if (p.isoFirst) isoBox = iso_begin(p, org, dir, tmax, seed, isoRng);
        active = p.hasVolume && trace_begin(p.F, p.G, p.rcpMc, org, dir, tmax, seed, T, cnt, p.volHash);
      } else {
        active = trace_begin(p.F, p.G, p.rcpMc, shadowPending ? sray.org : ray.org, shadowPending ? sray.dir : ray.dir,
                             shadowPending ? sray.tMax : ray.tMax, seed, T, cnt);
      }
      if (shadowPending) sray.seed = seed;
      else ray.seed = seed;
      tstate = active ? TRACING : DONE;
    }
    // ---- phase 2: traverse while enough of the warp's busy lanes trace ----
    long long c1 = 0;
    if (Count && L.profile) {
      __syncwarp();
      c1 = clock64();
      if (lane == 0) cyc[0] += (unsigned long long)(c1 - c0);
    }
    {
      const int busy = __popc(__ballot_sync(FULL, hasPixel));
      while (true) {
        const int tracing = __popc(__ballot_sync(FULL, tstate == TRACING));
        if (tracing == 0 || tracing * 100 < busy * L.threshold) break;
        if (Count && L.profile && lane == 0) {
          simt[0]++;
          simt[1] += (unsigned)tracing;
        }
        if (tstate == TRACING && T.inCell != 2 &&
            trace_seek(p.G, T, cnt, L.skip, !Batch && L.maskWords > 0, L.capFlag) == TR_MISS)
          tstate = DONE;
        if (tstate == TRACING && T.inCell == 2 && trace_sample(p.F, make_store<Store>(p), p.xf, T, h, cnt) == TR_HIT)
          tstate = DONE;
      }
    }
    // ---- phase 3: shade the finished traces (bounce(), shadeRays.cu:477-878) ----
    long long c2 = 0;
    if (Count && L.profile) {
      __syncwarp();
      c2 = clock64();
      if (lane == 0) cyc[1] += (unsigned long long)(c2 - c1);
    }
    if (Count && L.profile) {
      const unsigned shading = __popc(__ballot_sync(FULL, tstate == DONE));
      if (lane == 0 && shading) {
        simt[2]++;
        simt[3] += shading;
      }
    }
    if (Iso && tstate == DONE && p.isoFirst && isoBox) {
      // the surface's search, up to the volume's first collision
      PathRay &r = kind == K_SHADOW ? sray : ray;
      sHit = iso_trace_after<Store>(p, r.org, r.dir, r.tMax, h.hit ? h.t : __int_as_float(0x7f800000), isoRng, sT,
                                    sP, sN);
      if (sHit) h.hit = false;
    }
    if (Iso && tstate == DONE && p.hasVolume && !p.isoFirst) {
      // the iso-surface after the volume, up to the volume's hit
      PathRay &r = kind == K_SHADOW ? sray : ray;
      sHit = iso_trace<Store>(p, r.org, r.dir, h.hit ? h.t : r.tMax, r.seed, sT, sP, sN);
      if (sHit) h.hit = false;
    }
    if (tstate == DONE) {
      // Env-map texels: a main ray's miss lookup (radianceFromEnv) and a
      // hit's env light sample (EnvMap::sample) each form their texture
      // coordinates first; then one call fetches the texels of all lanes
      // that need one, instead of one call per kind of lane.
      Random rnd;
      EnvPick pick;
      float2 uv = make_float2(0.f, 0.f);
      bool needTex = false;
      const bool anyHit = h.hit || (Iso && sHit);
      if (kind == K_MAIN) {
        if (anyHit) {
          rnd = Random::derive(ray.seed, (uint64_t)hit_hash(h.hit ? h.t : sT));
          if (p.hasEnv) {
            pick = Batch ? env_pick_coords_ool(p, rnd) : env_pick_coords(p, rnd);
            uv = make_float2(pick.sx, pick.sy);
            needTex = true;
          }
        } else if (p.hasEnv) {
          uv = Batch ? env_miss_coords_ool(p, ray.dir) : env_miss_coords(p, ray.dir);
          needTex = true;
        }
      }
      vec3 texel(0.f);
      if (needTex) {
        const float4 t = Batch ? tex2D_ool(p.env, uv.x, uv.y) : tex2D(p.env, uv.x, uv.y);
        texel = p.env.scale * vec3(t.x, t.y, t.z);
      }
      tstate = NEED;
      const int accumID = L.accumIdStart + s;
      const float clampMax = 10.f * (float)(1 + accumID);
      if (kind == K_SHADOW) {
        if (!anyHit) accum_add(acc, vmin(sray.misWeight * from_half(sray.tp), vec3(clampMax)));
        shadowPending = false;
      } else {
        if (!Batch && gen == 0 && (p.depth || p.primId || p.instId || p.objId))
          write_aux(p, (size_t)iy * p.W + ix, accumID, !anyHit ? ray.tMax : h.hit ? h.t : sT,
                    !anyHit ? 0 : h.hit ? 1 : 2);
        vec3 frag(0.f);
        float alpha = 0.f;
        if (!anyHit) {
          const float4 miss = miss_color(p, iy);
          const vec3 env = p.hasEnv ? texel : (gen != 0 ? vec3(p.ambient) : vec3(0.f));
          if (gen == 0) {
            alpha = miss.w;
            frag = p.hasEnv ? env : vec3(miss.x, miss.y, miss.z);
          } else {
            frag = from_half(ray.tp) * env * ray.misWeight;
          }
          ray.tMax = -1.f;
        } else {
          if (gen == 0) alpha = 1.f;
          ShadeOut so;
          // setVolumeHit's P = obj_org + t * obj_dir (MCAccelerator.h:79)
          pick.radiance = texel;
          if (Iso && !h.hit)
            bounce_surface_hit(p, ray, sN, sT, sP, gen, rnd, pick, so);
          else if (Batch)
            bounce_volume_hit_ool(p, ray, h, T.org + h.t * T.dir, gen, rnd, pick, so);
          else
            bounce_volume_hit(p, ray, h, T.org + h.t * T.dir, gen, rnd, pick, so);
          if (so.shadowValid && so.shadow.tMax > 0.f) {
            sray = so.shadow;
            shadowPending = true;
          }
        }
        frag = vmin(frag, vec3(clampMax));
        if (accumID == 0 && gen == 0) {
          acc = make_float4(frag.x, frag.y, frag.z, alpha);
        } else {
          if (gen == 0 && alpha > 0.f) acc.w += alpha;
          accum_add(acc, frag);
        }
        mainAlive = ray.tMax > 0.f;
        gen++;
      }
      if (!shadowPending && !mainAlive) {
        // this pixel's pass is complete
        if (++s == L.spp) {
          p.accum[(size_t)iy * p.W + ix] = acc;
          hasPixel = false;
        } else {
          newSample = true;
        }
      }
    }
    if (Count && L.profile) {
      __syncwarp();
      if (lane == 0) cyc[2] += (unsigned long long)(clock64() - c2);
    }
  }
  if (Count && L.counters) {
    unsigned long long v[12] = {cnt.samples, cnt.mcs, cnt.rays, cnt.caps, cnt.cells, cyc[0], cyc[1], cyc[2],
                                simt[0], simt[1], simt[2], simt[3]};
    // (per-lane counts are 32-bit; a lane processes far fewer than 2^32 events)
#pragma unroll
    for (int k = 0; k < 12; k++) {
      unsigned long long x = v[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(FULL, x, o);
      if (lane == 0 && x) atomicAdd(L.counters + k, x);
    }
  }
}


// 32-bit words of dynamic shared memory the staged tables take
inline size_t staged_words(const RenderParams &p) {
  long long end = p.maskWords;
  if (p.cdfYOff >= 0) end = end > p.cdfYOff + p.env.H ? end : p.cdfYOff + p.env.H;
  if (p.pivOff >= 0) end = end > p.pivOff + (long long)p.env.H * p.pivPerRow ? end : p.pivOff + (long long)p.env.H * p.pivPerRow;
  if (p.rowOff >= 0) end = end > p.rowOff + 2LL * p.env.H ? end : p.rowOff + 2LL * p.env.H;
  return (size_t)end;
}

// The one-scene render kernels of a launch: with and without event
// counting, for a volume-only world or (at 4 resident blocks per SM) one
// with an iso-surface.
using RenderKernelFn = void (*)(const RenderParams, const RenderParams *, const long long *, int, int *);
template <class Store, int MinBlocks>
inline void render_kernels(const RenderParams &p, RenderKernelFn &counting, RenderKernelFn &plain) {
  counting = render_kernel<Store, MinBlocks, false, true>;
  plain = render_kernel<Store, MinBlocks, false, false>;
  if constexpr (MinBlocks == 4) {
    if (p.isoOn) {
      counting = render_kernel<Store, 4, false, true, true>;
      plain = render_kernel<Store, 4, false, false, true>;
    }
  }
}

template <class Store, int MinBlocks>
inline gbv_status launch_render_t(const RenderParams &p, const Store &store, cudaStream_t stream) {
  // persistent grid: as many resident blocks as the device holds
  int dev = 0, sms = 0, perSM = 0;
  gbv_status st = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (st == GBV_OK) st = check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  if (st != GBV_OK) return st;
  RenderKernelFn kCount, kPlain;
  render_kernels<Store, MinBlocks>(p, kCount, kPlain);
  const size_t smem = staged_words(p) * sizeof(uint32_t);
  if (smem > 48 * 1024) {
    st = check_cuda(cudaFuncSetAttribute(kCount, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "render_kernel: shared-memory size");
    if (st == GBV_OK)
      st = check_cuda(cudaFuncSetAttribute(kPlain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "render_kernel: shared-memory size");
    if (st != GBV_OK) return st;
  }
  st = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kCount, kThreads, smem),
                  "render_kernel: occupancy");
  if (st != GBV_OK) return st;
  const long long tiles = warp_tile_count(p);
  const long long warpsPerBlock = kThreads / 32;
  long long blocks = (long long)sms * (perSM > 0 ? perSM : 1);
  const long long needed = (tiles + warpsPerBlock - 1) / warpsPerBlock;
  if (blocks > needed) blocks = needed;
  if (blocks < 1) blocks = 1;
  // the tile pool counter and the majorant bitmask live in stream-ordered
  // scratch memory (the mask at a 256-byte offset: 16-byte aligned for the
  // bulk copy)
  int *pool = nullptr;
  const size_t maskBytes = (size_t)p.maskWords * 4;
  st = check_cuda(cudaMallocAsync((void **)&pool, 256 + maskBytes, stream), "cudaMallocAsync(tile pool)");
  if (st != GBV_OK) return st;
  st = check_cuda(cudaMemsetAsync(pool, 0, sizeof(int), stream), "render_kernel: clearing the tile pool");
  RenderParams q = p;
  if (st == GBV_OK && p.maskWords > 0 && p.maskSrc == nullptr && p.maskMode == 0) {
    uint32_t *mask = reinterpret_cast<uint32_t *>(reinterpret_cast<char *>(pool) + 256);
    const int nmc = p.G.M[0] * p.G.M[1] * p.G.M[2];
    majorant_mask_kernel<<<(unsigned)((p.maskWords + 7) / 8), 256, 0, stream>>>(p.G.maj, nmc, p.maskWords, mask);
    st = check_launch("majorant_mask_kernel");
    q.maskSrc = mask;
  }
  if (st == GBV_OK) {
    (p.counters ? kCount : kPlain)<<<(unsigned)blocks, kThreads, smem, stream>>>(q, nullptr, nullptr, 0, pool);
    st = check_launch("render_kernel");
  }
  const gbv_status fst = check_cuda(cudaFreeAsync(pool, stream), "cudaFreeAsync(tile pool)");
  return st != GBV_OK ? st : fst;
}

// Launch settings resolved from a gbv_render_config (gbv_render_ex): the
// resident 288-thread blocks per SM the registers are capped for (4: 36
// warps per SM at 56 registers; 5 blocks give 45 warps at 40 registers and
// spill more), and the shared-memory staging mode.  The traversal settings
// (skip, threshold) and the profile switch travel in RenderParams.
struct LaunchChoice {
  int occ = 4;
  int stage = GBV_STAGE_DEFAULT;
  int mode = GBV_RENDER_PERSISTENT;
};

// Shared-memory staging (same results either way).  GBV_STAGE_DEFAULT: the
// bitmask of non-zero majorants, one bit per macrocell, when it takes at
// most 8 KB per block (64 Ki macrocells; 4 KB for the 32^3 grid of the 512^3
// frame): the empty-cell test of the traversal becomes a shared-memory load
// (measured +1.8%); with an env map of at most 1024 rows also the row terms
// of its pdf (8 bytes a row).  GBV_STAGE_ALL also stages the env-map cdf_y
// and the per-row pivots of cdf_x (up to 64 KB per block; measured slower:
// the shared memory comes out of L1, which spills and CDF loads use).
// GBV_STAGE_NONE stages nothing.
inline void plan_staging(RenderParams &p, int stage) {
  const long long nmc = (long long)p.G.M[0] * p.G.M[1] * p.G.M[2];
  const bool any = stage != GBV_STAGE_NONE, all = stage == GBV_STAGE_ALL;
  p.maskMode = stage == GBV_STAGE_BALLOT ? 1 : 0;
  const int budget = (all ? 64 : 8) * 1024 / 4;
  int used = 0;
  p.maskWords = 0;
  p.cdfYOff = p.pivOff = p.rowOff = -1;
  p.pivPerRow = 0;
  p.maskSrc = nullptr;
  if (any && nmc > 0 && p.hasVolume && (((nmc + 31) / 32 + 3) & ~3ll) <= budget) {
    p.maskWords = (int)(((nmc + 31) / 32 + 3) & ~3ll);  // whole 16-byte units (one bulk copy)
    used = p.maskWords;
  }
  if (any && p.hasEnv && p.env.H >= 1 && p.env.H <= 1024) {
    used = (used + 1) & ~1;  // float2 entries
    p.rowOff = used;
    used += 2 * p.env.H;
  }
  if (all && p.hasEnv && p.env.W >= 2) {
    if (used + p.env.H <= budget) {
      p.cdfYOff = used;
      used += p.env.H;
    }
    const int per = (p.env.W - 1 + 31) / 32;  // segments holding entries 0..W-2
    if ((long long)used + (long long)p.env.H * per <= budget) {
      p.pivOff = used;
      p.pivPerRow = per;
      used += p.env.H * per;
    }
  }
}

template <class Store>
inline gbv_status launch_render(RenderParams p, const Store &store, cudaStream_t stream, const LaunchChoice &lc) {
  plan_staging(p, lc.stage);
  if (!p.counters) p.profile = 0;
  if (lc.occ <= 4 || p.isoOn) return launch_render_t<Store, 4>(p, store, stream);
  if (lc.occ >= 6) return launch_render_t<Store, 6>(p, store, stream);
  return launch_render_t<Store, 5>(p, store, stream);
}

template <class Store>
inline gbv_status launch_render_noalloc(RenderParams p, const Store &store, cudaStream_t stream, int *pool) {
  // fixed launch settings (results do not depend on them): 4 resident
  // blocks per SM, the default traversal settings, no shared-memory staging
  p.skip = kSkipDefault;
  p.threshold = kThresholdDefault;
  p.maskWords = 0;
  p.cdfYOff = p.pivOff = p.rowOff = -1;
  p.pivPerRow = 0;
  p.profile = 0;
  int dev = 0, sms = 0, perSM = 0;
  RenderKernelFn kCount, kPlain;
  render_kernels<Store, 4>(p, kCount, kPlain);
  gbv_status st = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (st == GBV_OK) st = check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  if (st == GBV_OK)
    st = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kCount, kThreads, 0),
                    "render_kernel: occupancy");
  if (st != GBV_OK) return st;
  const long long tiles = warp_tile_count(p);
  const long long warpsPerBlock = kThreads / 32;
  long long blocks = (long long)sms * (perSM > 0 ? perSM : 1);
  const long long needed = (tiles + warpsPerBlock - 1) / warpsPerBlock;
  if (blocks > needed) blocks = needed;
  if (blocks < 1) blocks = 1;
  st = check_cuda(cudaMemsetAsync(pool, 0, sizeof(int), stream), "gbv_render_noalloc: clearing the tile pool");
  if (st != GBV_OK) return st;
  (p.counters ? kCount : kPlain)<<<(unsigned)blocks, kThreads, 0, stream>>>(p, nullptr, nullptr, 0, pool);
  return check_launch("render_kernel (noalloc)");
}

}  // namespace gbv

struct gbv_batch {
  int count;
  int format, layout;
  gbv::RenderParams *d_items;  // device copy of the per-item parameters
  long long *d_tileStart;      // prefix sums of the items' 8x4 tile counts
  int *d_pool;                 // tile-pool counter
  long long totalTiles;
  int occ, threshold, skip;
  int device;
};

namespace gbv {

template <class Store>
inline gbv_status batch_launch(const gbv_batch *b, RenderParams L, cudaStream_t stream) {
  int sms = 0, perSM = 0;
  gbv_status st = check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device), "SM count");
  if (st != GBV_OK) return st;
  const long long warpsPerBlock = kThreads / 32;
  st = check_cuda(cudaMemsetAsync(b->d_pool, 0, sizeof(int), stream), "gbv_batch_render: pool");
  if (st != GBV_OK) return st;
#define GBV_BATCH_LAUNCH(OCC)                                                                              \
  {                                                                                                        \
    st = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, render_kernel<Store, OCC, true, true>, \
                                                                  kThreads, 0),                            \
                    "render_kernel (batch): occupancy");                                                   \
    if (st != GBV_OK) return st;                                                                           \
    long long blocks = (long long)sms * (perSM > 0 ? perSM : 1);                                           \
    const long long needed = (b->totalTiles + warpsPerBlock - 1) / warpsPerBlock;                         \
    if (blocks > needed) blocks = needed;                                                                  \
    if (blocks < 1) blocks = 1;                                                                            \
    if (L.counters)                                                                                        \
      render_kernel<Store, OCC, true, true><<<(unsigned)blocks, kThreads, 0, stream>>>(                    \
          L, b->d_items, b->d_tileStart, b->count, b->d_pool);                                             \
    else                                                                                                   \
      render_kernel<Store, OCC, true, false><<<(unsigned)blocks, kThreads, 0, stream>>>(                   \
          L, b->d_items, b->d_tileStart, b->count, b->d_pool);                                             \
  }
  switch (b->occ) {
    case 4: GBV_BATCH_LAUNCH(4) break;
    case 6: GBV_BATCH_LAUNCH(6) break;
    default: GBV_BATCH_LAUNCH(5) break;
  }
#undef GBV_BATCH_LAUNCH
  return check_launch("render_kernel (batch)");
}

#define GBV_DECLARE_STORE_LAUNCHERS(NAME)                                                        \
  gbv_status render_launch_##NAME(const RenderParams &p, cudaStream_t s, const LaunchChoice &lc); \
  gbv_status render_launch_noalloc_##NAME(const RenderParams &p, cudaStream_t s, int *pool);    \
  gbv_status batch_launch_##NAME(const gbv_batch *b, const RenderParams &L, cudaStream_t s);

GBV_DECLARE_STORE_LAUNCHERS(linear)
GBV_DECLARE_STORE_LAUNCHERS(f32)
GBV_DECLARE_STORE_LAUNCHERS(f16)
GBV_DECLARE_STORE_LAUNCHERS(bf16)
GBV_DECLARE_STORE_LAUNCHERS(u8)
GBV_DECLARE_STORE_LAUNCHERS(nvdb)

}  // namespace gbv
