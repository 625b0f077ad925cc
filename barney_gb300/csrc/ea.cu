// ea.cu -- fixed-step emission-absorption march and its path-replay adjoint.
//
// The reference renderer has no such form (it only delta-tracks); this march
// reuses its field sampler (StructuredData.h:104-115 with the CPU backend's
// trilinear filter) and transfer-function map (TransferFunction.h:66-86).
// Definition, shared with the CPU oracle:
//   ray: the perspective camera's pixel-centre ray; [t0,t1] from the box test
//   against the field's world bounds (tmin 0, tmax 1e30);
//   n = ceil((t1-t0)/dt) steps at t_i = t0+(i+.5)dt (skipped once >= t1);
//   x_i = sigma_i dt, alpha_i = -expm1(-x_i), T_i = exp(-tau_i) with a
//   Neumaier-compensated optical depth tau_i = sum_{k<i} x_k;
//   C = sum T_i alpha_i rgb_i, A = -expm1(-tau_n).
// Adjoint (no stored per-step state): dC/dx_j = rgb_j T_{j+1} - (C - C_{<=j}),
// dA/dx_j = T_n, dC/drgb_j = T_j alpha_j.
#include <cuda_runtime.h>
#include "gbv_volume.cuh"
#include "gbv_internal.h"

namespace gbv {

void commit_camera(const float pos[3], const float dir[3], const float up[3], float fovy, vec3 &lens00,
                   vec3 &dir00, vec3 &du, vec3 &dv);
bool make_field_geom(const gbv_scene *s, FieldGeom &F);

constexpr int kMaxViewsPerLaunch = 32;
// Steps per ray are bounded: the host rejects a step for which the field's
// box diagonal would take more than kEAMaxSteps - 16 steps, and the device
// clamps every ray's step count to kEAMaxSteps (never binding for an
// accepted step, whose chord is at most the diagonal).
constexpr int kEAMaxSteps = 1 << 24;
__device__ __forceinline__ int ea_step_count(float chord, float dt) {
  const float q = ceilf(chord / dt);
  return q < (float)kEAMaxSteps ? (int)q : kEAMaxSteps;
}

struct EAViewDev {
  vec3 lens00, dir00, du, dv;
  int W, H;
  long long offset;  // pixel offset of the view's image
};
struct EAParams {
  FieldGeom F;
  StoreLinearF32 store;  // linear FP32 field (the adjoint and FP64 modes read this)
  // brick-corner field of the forward march (any format), see ea_store
  const void *vox;
  const float2 *so;
  BrickGeom brick;
  XF xf;
  float dt;
  int numViews;
  EAViewDev views[kMaxViewsPerLaunch];
};

template <typename R> struct V3T { R x, y, z; };

__device__ __forceinline__ bool ea_ray(const EAParams &p, const EAViewDev &v, int ix, int iy, vec3 &org, vec3 &dir,
                                       float &t0, float &t1, int &n) {
  float image_u = ((float)ix + .5f) / (float)v.W;
  float image_v = ((float)iy + .5f) / (float)v.H;
  float aspect = (float)v.W / (float)v.H;
  vec3 d = v.dir00 + (1.f * aspect * (image_u - .5f)) * v.du + (1.f * (image_v - .5f)) * v.dv;
  dir = normalize(d);
  org = v.lens00;
  t0 = 0.f;
  t1 = 1e30f;
  if (!box_test(org, dir, t0, t1, p.F.boundsLo, p.F.boundsHi)) return false;
  if (!(t1 > t0)) return false;
  n = ea_step_count(t1 - t0, p.dt);
  return true;
}

template <class Store> __device__ __forceinline__ Store ea_store(const EAParams &p);
template <> __device__ __forceinline__ StoreLinearF32 ea_store<StoreLinearF32>(const EAParams &p) { return p.store; }
// brick stores read through L1 (neighbouring rays and consecutive steps share cells)
#define GBV_EA_BRICK_STORE(FMT)                                                                           \
  template <> __device__ __forceinline__ StoreBrickCorners<FMT, true> ea_store<StoreBrickCorners<FMT, true>>( \
      const EAParams &p) {                                                                                \
    return StoreBrickCorners<FMT, true>{p.vox, p.so, p.brick};                                            \
  }
GBV_EA_BRICK_STORE(GBV_VOXEL_F32)
GBV_EA_BRICK_STORE(GBV_VOXEL_F16)
GBV_EA_BRICK_STORE(GBV_VOXEL_BF16)
GBV_EA_BRICK_STORE(GBV_VOXEL_U8_SCALED)
#undef GBV_EA_BRICK_STORE

// FP32 forward; the voxels come from any store (a brick-corner FP32 store
// samples the same values as the linear one)
template <class Store>
__global__ void __launch_bounds__(128) ea_forward_kernel(const EAParams p, float4 *__restrict__ out) {
  const Store store = ea_store<Store>(p);
  const EAViewDev &v = p.views[blockIdx.z];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ix = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
  const int iy = blockIdx.y * 8 + (warp >> 1) * 4 + (lane >> 3);
  if (ix >= v.W || iy >= v.H) return;
  vec3 org, dir;
  float t0, t1;
  int n;
  float4 res = make_float4(0.f, 0.f, 0.f, 0.f);
  if (ea_ray(p, v, ix, iy, org, dir, t0, t1, n)) {
    float tau = 0.f, comp = 0.f, C0 = 0.f, C1 = 0.f, C2 = 0.f;
    for (int i = 0; i < n; i++) {
      const float t = t0 + ((float)i + .5f) * p.dt;
      if (t >= t1) break;
      const vec3 P = org + t * dir;
      const vec4 m = sample_and_map(p.F, store, p.xf, P);
      const float x = m.w * p.dt;
      const float T = expf(-(tau + comp));
      const float alpha = -expm1f(-x);
      const float w = T * alpha;
      C0 += w * m.x;
      C1 += w * m.y;
      C2 += w * m.z;
      const float tn = tau + x;
      if (fabsf(tau) >= fabsf(x)) comp += (tau - tn) + x;
      else comp += (x - tn) + tau;
      tau = tn;
    }
    res = make_float4(C0, C1, C2, -expm1f(-(tau + comp)));
  }
  out[v.offset + (long long)iy * v.W + ix] = res;
}

// FP64 forward (finite-difference check mode)
__device__ __forceinline__ double sample_field_f64(const FieldGeom &F, const StoreLinearF32 &S, double Px, double Py,
                                                   double Pz) {
  double rx = (Px - (double)F.origin.x) * (double)F.rcpSpacing.x;
  double ry = (Py - (double)F.origin.y) * (double)F.rcpSpacing.y;
  double rz = (Pz - (double)F.origin.z) * (double)F.rcpSpacing.z;
  if (rx < 0.0 || ry < 0.0 || rz < 0.0) return __longlong_as_double(0x7ff8000000000000ll);
  if (rx >= (double)F.C[0] || ry >= (double)F.C[1] || rz >= (double)F.C[2])
    return __longlong_as_double(0x7ff8000000000000ll);
  double tc[3] = {rx + .5, ry + .5, rz + .5};
  int i0[3], i1[3];
  double f[3];
  for (int a = 0; a < 3; a++) {
    int N = F.N[a];
    if (tc[a] - .5 <= 0.0) { i0[a] = i1[a] = 0; f[a] = 0.0; }
    else if (tc[a] - .5 >= (double)(N - 1)) { i0[a] = i1[a] = N - 1; f[a] = 0.0; }
    else {
      f[a] = (tc[a] - .5) - (double)(int)(tc[a] - .5);
      i0[a] = (int)(tc[a] - .5);
      i1[a] = i0[a] + 1;
    }
  }
  float c[8];
  S.corners(i0[0], i1[0], i0[1], i1[1], i0[2], i1[2], c);
  auto l = [](double t, double a, double b) { return (1.0 - t) * a + t * b; };
  double v00 = l(f[0], c[0], c[1]), v01 = l(f[0], c[2], c[3]);
  double v10 = l(f[0], c[4], c[5]), v11 = l(f[0], c[6], c[7]);
  return l(f[2], l(f[1], v00, v01), l(f[1], v10, v11));
}

__global__ void __launch_bounds__(128) ea_forward_f64_kernel(const EAParams p, double4 *__restrict__ out) {
  const EAViewDev &v = p.views[blockIdx.z];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ix = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
  const int iy = blockIdx.y * 8 + (warp >> 1) * 4 + (lane >> 3);
  if (ix >= v.W || iy >= v.H) return;
  vec3 orgf, dirf;
  float t0f, t1f;
  int nf;
  double4 res = make_double4(0., 0., 0., 0.);
  if (ea_ray(p, v, ix, iy, orgf, dirf, t0f, t1f, nf)) {
    // the box test of the double march runs in double, as the oracle's does
    double o[3] = {orgf.x, orgf.y, orgf.z}, d[3] = {dirf.x, dirf.y, dirf.z};
    double lo[3] = {p.F.boundsLo.x, p.F.boundsLo.y, p.F.boundsLo.z};
    double hi[3] = {p.F.boundsHi.x, p.F.boundsHi.y, p.F.boundsHi.z};
    double t0 = 0.0, t1 = (double)1e30f, tn_[3], tf_[3];
    for (int a = 0; a < 3; a++) {
      double r = 1.0 / d[a];
      double a0 = (lo[a] - o[a]) * r, a1 = (hi[a] - o[a]) * r;
      tn_[a] = (a1 < a0) ? a1 : a0;
      tf_[a] = (a0 < a1) ? a1 : a0;
    }
    double tnear = mx(mx(tn_[0], tn_[1]), tn_[2]), tfar = mn(mn(tf_[0], tf_[1]), tf_[2]);
    t0 = mx(t0, tnear);
    t1 = mn(t1, tfar);
    if (t0 <= t1 && t1 > t0) {
      const double dt = (double)p.dt;
      const double q = ceil((t1 - t0) / dt);
      const int n = q < (double)kEAMaxSteps ? (int)q : kEAMaxSteps;
      double tau = 0., comp = 0., C0 = 0., C1 = 0., C2 = 0.;
      for (int i = 0; i < n; i++) {
        const double t = t0 + ((double)i + .5) * dt;
        if (t >= t1) break;
        double s = sample_field_f64(p.F, p.store, o[0] + t * d[0], o[1] + t * d[1], o[2] + t * d[2]);
        double r = 0., g = 0., b = 0., sig = 0.;
        if (!isnan(s)) {
          double f = (s - (double)p.xf.lo) / (double)p.xf.span;
          f = clampv(f, 0.0, 1.0);
          f *= (double)(p.xf.n - 1);
          int idx = clampv((int)f, 0, p.xf.n - 2);
          f -= (double)idx;
          float4 v0 = __ldg(p.xf.v + idx), v1 = __ldg(p.xf.v + idx + 1);
          r = (1. - f) * v0.x + f * v1.x;
          g = (1. - f) * v0.y + f * v1.y;
          b = (1. - f) * v0.z + f * v1.z;
          sig = ((1. - f) * v0.w + f * v1.w) * (double)p.xf.baseDensity;
        }
        const double x = sig * dt;
        const double T = exp(-(tau + comp));
        const double w = T * -expm1(-x);
        C0 += w * r;
        C1 += w * g;
        C2 += w * b;
        const double tn = tau + x;
        if (fabs(tau) >= fabs(x)) comp += (tau - tn) + x;
        else comp += (x - tn) + tau;
        tau = tn;
      }
      res = make_double4(C0, C1, C2, -expm1(-(tau + comp)));
    }
  }
  out[v.offset + (long long)iy * v.W + ix] = res;
}

// Warp-aggregated flush of 8 per-corner (or per-TF-entry) gradient sums.
// Lanes that flush in the same step and hold the same key are grouped with
// __match_any_sync; the group's lowest lane gathers the others' sums by
// shuffles and issues the 8 atomics once.  Called by all 32 lanes.
// off(k) gives the destination index of sum k (evaluated by the leader only).
template <class Off>
__device__ __forceinline__ void flush8(float *__restrict__ dst, bool flush, unsigned long long key, Off off,
                                       const float v[8]) {
  const int lane = threadIdx.x & 31;
  const unsigned fm = __ballot_sync(0xffffffffu, flush);
  if (!flush) return;
  const unsigned peers = __match_any_sync(fm, key);
  const int leader = __ffs(peers) - 1;
  unsigned rem = (lane == leader) ? (peers & ~(1u << lane)) : 0u;
  const int maxRounds = (int)__reduce_max_sync(fm, (unsigned)__popc(rem));
  float acc[8];
#pragma unroll
  for (int k = 0; k < 8; k++) acc[k] = v[k];
  for (int r = 0; r < maxRounds; r++) {
    const int src = rem ? (__ffs(rem) - 1) : lane;
    const bool take = rem != 0u;
    if (rem) rem &= rem - 1u;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const float o = __shfl_sync(fm, v[k], src);
      if (take) acc[k] += o;
    }
  }
  if (lane == leader) {
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (acc[k] != 0.f) atomicAdd(dst + off(k), acc[k]);
  }
}

// FP32 adjoint by path replay.  Consecutive steps of a ray mostly stay in
// the same cell and TF segment, so each lane keeps running sums for its
// current stencil and TF segment and flushes them (warp-aggregated) only
// when either changes.  Lanes run in lockstep up to the warp's longest march
// (one extra iteration without steps flushes the last sums) so the flushes
// see all 32 lanes.
template <int MinBlocks>
__global__ void __launch_bounds__(128, MinBlocks) ea_backward_kernel(const EAParams p, const float4 *__restrict__ img,
                                                          const float4 *__restrict__ gimg, float *__restrict__ gvox,
                                                          float *__restrict__ gtf) {
  extern __shared__ float s_gtf[];  // tf_n*4, block-private TF gradient
  const int ntf = 4 * p.xf.n;
  for (int i = threadIdx.x; i < ntf; i += blockDim.x) s_gtf[i] = 0.f;
  __syncthreads();
  const EAViewDev &v = p.views[blockIdx.z];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int ix = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
  const int iy = blockIdx.y * 8 + (warp >> 1) * 4 + (lane >> 3);
  const bool inside = ix < v.W && iy < v.H;
  vec3 org(0.f), dir(0.f, 0.f, 1.f);
  float t0 = 0.f, t1 = 0.f;
  int n = 0;
  float4 C = make_float4(0.f, 0.f, 0.f, 0.f), g = C;
  if (inside) {
    const long long pix = v.offset + (long long)iy * v.W + ix;
    if (ea_ray(p, v, ix, iy, org, dir, t0, t1, n)) {
      C = img[pix];
      g = gimg[pix];
    } else {
      n = 0;
    }
  }
  const int nMax = (int)__reduce_max_sync(0xffffffffu, (unsigned)max(n, 0));
  const float Tn = 1.f - C.w;
  const float gs = (float)(p.xf.n - 1) / p.xf.span;
  const size_t sy = (size_t)p.F.N[0], sz = (size_t)p.F.N[0] * p.F.N[1];
  const float bd = p.xf.baseDensity;
  float A0 = 0.f, A1 = 0.f, A2 = 0.f;
  // transmittance before the current step; the replay advances it as
  // T_{i+1} = T_i - T_i alpha_i (alpha from expm1, so 1-alpha keeps full
  // absolute precision): one transcendental per step
  float T = 1.f;
  bool alive = inside && n > 0;
  // running sums: voxel stencil (key = 8 * base voxel + which axes are not
  // clamped) and TF segment (key = idx)
  long long vKey = -1;
  float vAcc[8];
  int tIdx = -1;
  float tAcc[8];
#pragma unroll
  for (int k = 0; k < 8; k++) { vAcc[k] = 0.f; tAcc[k] = 0.f; }
  for (int i = 0; i <= nMax; i++) {
    // this step's contributions (none past the end of the lane's march)
    bool have = false;
    long long key = -1;
    int idx = -1;
    float fx = 0.f, fy = 0.f, fz = 0.f, dLds = 0.f, f = 0.f, dr = 0.f, dg = 0.f, db = 0.f, dsb = 0.f;
    if (alive && i < n) {
      const float t = t0 + ((float)i + .5f) * p.dt;
      if (t >= t1) {
        alive = false;
      } else {
        const vec3 P = org + t * dir;
        vec3 rel = (P - p.F.origin) * p.F.rcpSpacing;
        const bool in = !(rel.x < 0.f || rel.y < 0.f || rel.z < 0.f || rel.x >= (float)p.F.C[0] ||
                          rel.y >= (float)p.F.C[1] || rel.z >= (float)p.F.C[2]);
        if (in) {
          const vec3 tc = rel + vec3(.5f);
          int x0, x1, y0, y1, z0, z1;
          lerp_coords(p.F.N[0], tc.x, x0, x1, fx);
          lerp_coords(p.F.N[1], tc.y, y0, y1, fy);
          lerp_coords(p.F.N[2], tc.z, z0, z1, fz);
          float c[8];
          p.store.corners(x0, x1, y0, y1, z0, z1, c);
          const float v00 = lerp_l(fx, c[0], c[1]), v01 = lerp_l(fx, c[2], c[3]);
          const float v10 = lerp_l(fx, c[4], c[5]), v11 = lerp_l(fx, c[6], c[7]);
          const float sv = lerp_l(fz, lerp_l(fy, v00, v01), lerp_l(fy, v10, v11));
          f = (sv - p.xf.lo) / p.xf.span;
          const bool clamped = !(f > 0.f && f < 1.f);
          f = clampv(f, 0.f, 1.f);
          f *= (float)(p.xf.n - 1);
          idx = clampv((int)f, 0, p.xf.n - 2);
          f -= (float)idx;
          const float4 e0 = __ldg(p.xf.v + idx), e1 = __ldg(p.xf.v + idx + 1);
          const float r = (1.f - f) * e0.x + f * e1.x, gg = (1.f - f) * e0.y + f * e1.y,
                      b = (1.f - f) * e0.z + f * e1.z;
          const float sig = ((1.f - f) * e0.w + f * e1.w) * bd;
          const float x = sig * p.dt;
          const float w = T * -expm1f(-x);
          A0 += w * r;
          A1 += w * gg;
          A2 += w * b;
          const float Tnext = T - w;
          float dLdx = g.w * Tn;
          dLdx += g.x * (r * Tnext - (C.x - A0));
          dLdx += g.y * (gg * Tnext - (C.y - A1));
          dLdx += g.z * (b * Tnext - (C.z - A2));
          T = Tnext;
          const float dLdsig = dLdx * p.dt;
          dr = g.x * w;
          dg = g.y * w;
          db = g.z * w;
          dsb = dLdsig * bd;
          if (!clamped) {
            dLds = dLdsig * bd * (e1.w - e0.w) * gs;
            dLds += dr * (e1.x - e0.x) * gs + dg * (e1.y - e0.y) * gs + db * (e1.z - e0.z) * gs;
            const size_t base = (size_t)x0 + sy * y0 + sz * z0;
            key = 8 * (long long)base + (x1 != x0 ? 1 : 0) + (y1 != y0 ? 2 : 0) + (z1 != z0 ? 4 : 0);
            have = true;
          }
        }
      }
    }
    // voxel stencil: flush the running sums when the stencil changes
    const bool vFlush = vKey >= 0 && (key != vKey);
    flush8(gvox, vFlush, (unsigned long long)vKey,
           [&](int k) {
             const size_t base = (size_t)(vKey >> 3);
             const int m = (int)(vKey & 7) & k;
             return base + ((m & 1) ? 1 : 0) + ((m & 2) ? sy : 0) + ((m & 4) ? sz : 0);
           },
           vAcc);
    if (vFlush || vKey < 0) {
      vKey = have ? key : -1;
#pragma unroll
      for (int k = 0; k < 8; k++) vAcc[k] = 0.f;
    }
    if (have) {
      const float wx0 = 1.f - fx, wy0 = 1.f - fy, wz0 = 1.f - fz;
      vAcc[0] += dLds * wx0 * wy0 * wz0;
      vAcc[1] += dLds * fx * wy0 * wz0;
      vAcc[2] += dLds * wx0 * fy * wz0;
      vAcc[3] += dLds * fx * fy * wz0;
      vAcc[4] += dLds * wx0 * wy0 * fz;
      vAcc[5] += dLds * fx * wy0 * fz;
      vAcc[6] += dLds * wx0 * fy * fz;
      vAcc[7] += dLds * fx * fy * fz;
    }
    // TF segment: same scheme, into the block's shared-memory gradient
    const bool tFlush = tIdx >= 0 && idx != tIdx;
    flush8(s_gtf, tFlush, (unsigned long long)tIdx, [&](int k) { return 4 * tIdx + k; }, tAcc);
    if (tFlush || tIdx < 0) {
      tIdx = idx;
#pragma unroll
      for (int k = 0; k < 8; k++) tAcc[k] = 0.f;
    }
    if (idx >= 0) {
      tAcc[0] += dr * (1.f - f);
      tAcc[1] += dg * (1.f - f);
      tAcc[2] += db * (1.f - f);
      tAcc[3] += dsb * (1.f - f);
      tAcc[4] += dr * f;
      tAcc[5] += dg * f;
      tAcc[6] += db * f;
      tAcc[7] += dsb * f;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < ntf; i += blockDim.x)
    if (s_gtf[i] != 0.f) atomicAdd(gtf + i, s_gtf[i]);
}

// forward_any_store: the caller is the forward march, which also reads
// brick-corner stores (any format); the adjoint and the FP64 march read the
// linear FP32 field only.
static gbv_status ea_prepare(const gbv_scene *s, float step, EAParams &p, bool forward_any_store = false) {
  if (!s || !s->d_voxels || !s->d_tf || s->tf_n < 2)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "ea: scene lacks voxels or transfer function");
  const bool linear = s->layout == GBV_LAYOUT_LINEAR && s->format == GBV_VOXEL_F32;
  const bool bricks = s->layout == GBV_LAYOUT_BRICK_CORNERS && s->format >= GBV_VOXEL_F32 &&
                      s->format <= GBV_VOXEL_U8_SCALED;
  if (!linear && !(forward_any_store && bricks))
    return set_error(GBV_ERROR_UNSUPPORTED, forward_any_store
                                                ? "ea: unknown voxel layout or format"
                                                : "ea: the adjoint and FP64 marches read an FP32 linear field");
  if (bricks && s->format == GBV_VOXEL_U8_SCALED && !s->d_scale_offset)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "ea: U8 voxels need the scale/offset table");
  if (!(step > 0.f)) return set_error(GBV_ERROR_INVALID_ARGUMENT, "ea: step must be positive");
  if (s->dims[0] < 2 || s->dims[1] < 2 || s->dims[2] < 2)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "ea: a field needs at least 2 voxels per axis");
  make_field_geom(s, p.F);
  {
    const double dx = (double)p.F.boundsHi.x - p.F.boundsLo.x, dy = (double)p.F.boundsHi.y - p.F.boundsLo.y,
                 dz = (double)p.F.boundsHi.z - p.F.boundsLo.z;
    const double diag = sqrt(dx * dx + dy * dy + dz * dz);
    if (!(diag / (double)step <= (double)(kEAMaxSteps - 16)))
      return set_error(GBV_ERROR_INVALID_ARGUMENT,
                       "ea: step too small for the field (a ray could take more than 2^24 steps)");
  }
  p.store = StoreLinearF32{reinterpret_cast<const float *>(s->d_voxels), s->dims[0], s->dims[1]};
  p.vox = s->d_voxels;
  p.so = reinterpret_cast<const float2 *>(s->d_scale_offset);
  if (bricks) {
    int l[3];
    if (!resolve_brick_shape(s->brick_log2, l))
      return set_error(GBV_ERROR_INVALID_ARGUMENT, "brick_log2: each 1..6 (0 = 3), sum at most 15");
    p.brick = make_brick_geom(s->dims, l);
  }
  p.xf.v = reinterpret_cast<const float4 *>(s->d_tf);
  p.xf.n = s->tf_n;
  p.xf.lo = s->domain[0];
  p.xf.span = s->domain[1] - s->domain[0];
  p.xf.baseDensity = s->base_density;
  p.dt = step;
  return GBV_OK;
}

// Runs `fn(params, maxW, maxH)` for chunks of at most kMaxViewsPerLaunch views.
template <typename F>
static gbv_status for_view_chunks(EAParams &p, const gbv_ea_view *views, int num_views, F &&fn) {
  long long offset = 0;
  for (int base = 0; base < num_views; base += kMaxViewsPerLaunch) {
    int cnt = min(kMaxViewsPerLaunch, num_views - base);
    int maxW = 0, maxH = 0;
    for (int k = 0; k < cnt; k++) {
      const gbv_ea_view &v = views[base + k];
      if (v.width <= 0 || v.height <= 0) return set_error(GBV_ERROR_INVALID_ARGUMENT, "ea: empty view");
      EAViewDev &d = p.views[k];
      commit_camera(v.pos, v.dir, v.up, v.fovy, d.lens00, d.dir00, d.du, d.dv);
      d.W = v.width;
      d.H = v.height;
      d.offset = offset;
      offset += (long long)v.width * v.height;
      maxW = max(maxW, v.width);
      maxH = max(maxH, v.height);
    }
    p.numViews = cnt;
    gbv_status st = fn(p, cnt, maxW, maxH);
    if (st != GBV_OK) return st;
  }
  return GBV_OK;
}

}  // namespace gbv

using namespace gbv;

extern "C" {

gbv_status gbv_ea_render(const gbv_scene *s, const gbv_ea_view *views, int num_views, float step, float *d_images,
                         void *stream) {
  EAParams p;
  gbv_status st = ea_prepare(s, step, p, true);
  if (st != GBV_OK) return st;
  if (!views || num_views <= 0 || !d_images) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_ea_render: views");
  const int layout = s->layout, format = s->format;
  return for_view_chunks(p, views, num_views, [&](EAParams &q, int cnt, int maxW, int maxH) {
    dim3 grid((maxW + 15) / 16, (maxH + 7) / 8, cnt);
    float4 *out = reinterpret_cast<float4 *>(d_images);
    cudaStream_t cs = (cudaStream_t)stream;
    if (layout == GBV_LAYOUT_LINEAR) ea_forward_kernel<StoreLinearF32><<<grid, 128, 0, cs>>>(q, out);
    else if (format == GBV_VOXEL_F32) ea_forward_kernel<StoreBrickCorners<GBV_VOXEL_F32, true>><<<grid, 128, 0, cs>>>(q, out);
    else if (format == GBV_VOXEL_F16) ea_forward_kernel<StoreBrickCorners<GBV_VOXEL_F16, true>><<<grid, 128, 0, cs>>>(q, out);
    else if (format == GBV_VOXEL_BF16)
      ea_forward_kernel<StoreBrickCorners<GBV_VOXEL_BF16, true>><<<grid, 128, 0, cs>>>(q, out);
    else ea_forward_kernel<StoreBrickCorners<GBV_VOXEL_U8_SCALED, true>><<<grid, 128, 0, cs>>>(q, out);
    return check_launch("ea_forward_kernel");
  });
}

gbv_status gbv_ea_render_f64(const gbv_scene *s, const gbv_ea_view *views, int num_views, float step,
                             double *d_images, void *stream) {
  EAParams p;
  gbv_status st = ea_prepare(s, step, p);
  if (st != GBV_OK) return st;
  if (!views || num_views <= 0 || !d_images) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_ea_render_f64: views");
  return for_view_chunks(p, views, num_views, [&](EAParams &q, int cnt, int maxW, int maxH) {
    dim3 grid((maxW + 15) / 16, (maxH + 7) / 8, cnt);
    ea_forward_f64_kernel<<<grid, 128, 0, (cudaStream_t)stream>>>(q, reinterpret_cast<double4 *>(d_images));
    return check_launch("ea_forward_f64_kernel");
  });
}

gbv_status gbv_ea_backward_ex(const gbv_scene *s, const gbv_ea_view *views, int num_views, float step,
                              const float *d_images, const float *d_grad_images, float *d_grad_scalars,
                              float *d_grad_tf, int blocks_per_sm, void *stream) {
  EAParams p;
  gbv_status st = ea_prepare(s, step, p);
  if (st != GBV_OK) return st;
  if (!views || num_views <= 0 || !d_images || !d_grad_images || !d_grad_scalars || !d_grad_tf)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_ea_backward: null pointer");
  if (blocks_per_sm != 0 && blocks_per_sm != 4 && blocks_per_sm != 6 && blocks_per_sm != 8)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_ea_backward_ex: blocks_per_sm is 4, 6 or 8 (0: 6)");
  size_t smem = (size_t)4 * s->tf_n * sizeof(float);
  if (smem > 48 * 1024) return set_error(GBV_ERROR_UNSUPPORTED, "gbv_ea_backward: transfer function above 3072 entries");
  // resident 128-thread blocks per SM the adjoint's registers are capped
  // for (default 6: 80 registers, no spills)
  const int occ = blocks_per_sm ? blocks_per_sm : 6;
  return for_view_chunks(p, views, num_views, [&](EAParams &q, int cnt, int maxW, int maxH) {
    dim3 grid((maxW + 15) / 16, (maxH + 7) / 8, cnt);
    const float4 *img = reinterpret_cast<const float4 *>(d_images);
    const float4 *gimg = reinterpret_cast<const float4 *>(d_grad_images);
    cudaStream_t cs = (cudaStream_t)stream;
    if (occ == 8) ea_backward_kernel<8><<<grid, 128, smem, cs>>>(q, img, gimg, d_grad_scalars, d_grad_tf);
    else if (occ == 6) ea_backward_kernel<6><<<grid, 128, smem, cs>>>(q, img, gimg, d_grad_scalars, d_grad_tf);
    else ea_backward_kernel<4><<<grid, 128, smem, cs>>>(q, img, gimg, d_grad_scalars, d_grad_tf);
    return check_launch("ea_backward_kernel");
  });
}

gbv_status gbv_ea_backward(const gbv_scene *s, const gbv_ea_view *views, int num_views, float step,
                           const float *d_images, const float *d_grad_images, float *d_grad_scalars,
                           float *d_grad_tf, void *stream) {
  return gbv_ea_backward_ex(s, views, num_views, step, d_images, d_grad_images, d_grad_scalars, d_grad_tf, 0,
                            stream);
}

}  // extern "C"
