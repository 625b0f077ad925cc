// iso.cu -- ray queries against an iso-surface of the structured field.
//
// MCIsoSurfaceAccel::isProg (barney/volume/MCAccelerator.h:338-567): the
// macrocell DDA of the volume path (dda::dda3, DDA.h:65-206), but each cell
// is tested against the iso value with its scalar range (not a majorant),
// and a cell whose range holds it is cut into 10 sub-steps; the first
// sub-step whose end samples bracket the iso value gives the hit t by linear
// interpolation.  The normal is the central difference of the field at
// +-delta per axis, one-sided where a sample falls outside the field
// (iso_search, shared with the frame render).  The query returns t, the hit
// point and the unit normal; the frame render adds the material (opacity,
// Lambertian) and the surface shading (gbv_scene.iso).
#include "render_kernel.cuh"

namespace gbv {

bool make_field_geom(const gbv_scene *s, FieldGeom &F);

struct IsoParams {
  FieldGeom F;
  MCGridDev G;  // G.maj unused; ranges below
  vec3 rcpMc;
  const float2 *ranges;
  float iso;
  float delta;  // normal finite-difference step
  const void *vox;
  const float2 *so;
  BrickGeom brick;
};

template <class Store> __device__ __forceinline__ Store iso_store(const IsoParams &p);
template <> __device__ __forceinline__ StoreLinearF32 iso_store<StoreLinearF32>(const IsoParams &p) {
  return StoreLinearF32{reinterpret_cast<const float *>(p.vox), p.F.N[0], p.F.N[1]};
}
#define GBV_ISO_BRICK_STORE(FMT)                                                                             \
  template <> __device__ __forceinline__ StoreBrickCorners<FMT> iso_store<StoreBrickCorners<FMT>>(          \
      const IsoParams &p) {                                                                                  \
    return StoreBrickCorners<FMT>{p.vox, p.so, p.brick};                                                     \
  }
GBV_ISO_BRICK_STORE(GBV_VOXEL_F32)
GBV_ISO_BRICK_STORE(GBV_VOXEL_F16)
GBV_ISO_BRICK_STORE(GBV_VOXEL_BF16)
GBV_ISO_BRICK_STORE(GBV_VOXEL_U8_SCALED)
#undef GBV_ISO_BRICK_STORE

// rays: two float4 per ray, (org.xyz, tmax) and (dir.xyz, unused).
// hits: two float4 per ray, (t, P.xyz) and (N.xyz, 1) on a hit, else all 0.
template <class Store>
__global__ void __launch_bounds__(128) iso_kernel(const IsoParams p, const float4 *__restrict__ rays, long long n,
                                                  float4 *__restrict__ hits) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const Store store = iso_store<Store>(p);
  const float4 r0 = rays[2 * k], r1 = rays[2 * k + 1];
  const float tmax = r0.w;
  float4 h0 = make_float4(0.f, 0.f, 0.f, 0.f), h1 = h0;
  Traversal T;
  RNGSeed seed;
  seed.state = 0;
  Ctr<false> cnt;
  // box test, zero-direction guard and DDA set-up, as for a volume ray
  if (trace_begin(p.F, p.G, p.rcpMc, vec3(r0.x, r0.y, r0.z), vec3(r1.x, r1.y, r1.z), tmax, seed, T, cnt)) {
    float t;
    vec3 N;
    if (iso_search(p.F, store, p.G, p.ranges, p.iso, p.delta, T, tmax, t, N)) {
      const vec3 P = T.org + t * T.dir;
      h0 = make_float4(t, P.x, P.y, P.z);
      h1 = make_float4(N.x, N.y, N.z, 1.f);
    }
  }
  hits[2 * k] = h0;
  hits[2 * k + 1] = h1;
}

}  // namespace gbv

using namespace gbv;

extern "C" gbv_status gbv_iso_intersect(const gbv_scene *s, const float *d_ranges, float iso_value,
                                        const float *d_rays, long long num_rays, float *d_hits, void *stream) {
  if (!s || !s->d_voxels || !d_ranges || !d_rays || !d_hits || num_rays < 0 || s->cells_per_mc <= 0)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_iso_intersect: null pointer or bad size");
  if (s->dims[0] < 2 || s->dims[1] < 2 || s->dims[2] < 2)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_iso_intersect: a field needs at least 2 voxels per axis");
  const bool linear = s->layout == GBV_LAYOUT_LINEAR && s->format == GBV_VOXEL_F32;
  const bool bricks = s->layout == GBV_LAYOUT_BRICK_CORNERS && s->format >= GBV_VOXEL_F32 &&
                      s->format <= GBV_VOXEL_U8_SCALED;
  if (!linear && !bricks) return set_error(GBV_ERROR_UNSUPPORTED, "gbv_iso_intersect: unknown layout or format");
  if (s->format == GBV_VOXEL_U8_SCALED && !s->d_scale_offset)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_iso_intersect: U8 voxels need the scale/offset table");
  if (num_rays == 0) return GBV_OK;
  IsoParams p;
  make_field_geom(s, p.F);
  int M[3];
  gbv_status st = gbv_mc_dims(s->dims, s->cells_per_mc, M);
  if (st != GBV_OK) return st;
  p.G.maj = nullptr;
  for (int i = 0; i < 3; i++) p.G.M[i] = M[i];
  p.G.origin = p.F.boundsLo;
  p.G.spacing = vec3((float)s->cells_per_mc) * vec3(s->spacing[0], s->spacing[1], s->spacing[2]);
  p.rcpMc = rcp(p.G.spacing);
  p.ranges = reinterpret_cast<const float2 *>(d_ranges);
  p.iso = iso_value;
  // MCAccelerator.h:476-479: delta = |bounds size| * .1 / (Mx + My + Mz)
  const vec3 size = p.F.boundsHi - p.F.boundsLo;
  p.delta = sqrtf(dot(size, size)) * .1f / (float)(M[0] + M[1] + M[2]);
  p.vox = s->d_voxels;
  p.so = reinterpret_cast<const float2 *>(s->d_scale_offset);
  if (bricks) {
    int l[3];
    if (!resolve_brick_shape(s->brick_log2, l))
      return set_error(GBV_ERROR_INVALID_ARGUMENT, "brick_log2: each 1..6 (0 = 3), sum at most 15");
    p.brick = make_brick_geom(s->dims, l);
  }
  const unsigned blocks = (unsigned)((num_rays + 127) / 128);
  cudaStream_t cs = (cudaStream_t)stream;
  const float4 *r = reinterpret_cast<const float4 *>(d_rays);
  float4 *h = reinterpret_cast<float4 *>(d_hits);
  if (linear) iso_kernel<StoreLinearF32><<<blocks, 128, 0, cs>>>(p, r, num_rays, h);
  else if (s->format == GBV_VOXEL_F32) iso_kernel<StoreBrickCorners<GBV_VOXEL_F32>><<<blocks, 128, 0, cs>>>(p, r, num_rays, h);
  else if (s->format == GBV_VOXEL_F16) iso_kernel<StoreBrickCorners<GBV_VOXEL_F16>><<<blocks, 128, 0, cs>>>(p, r, num_rays, h);
  else if (s->format == GBV_VOXEL_BF16) iso_kernel<StoreBrickCorners<GBV_VOXEL_BF16>><<<blocks, 128, 0, cs>>>(p, r, num_rays, h);
  else iso_kernel<StoreBrickCorners<GBV_VOXEL_U8_SCALED>><<<blocks, 128, 0, cs>>>(p, r, num_rays, h);
  return check_launch("iso_kernel");
}
