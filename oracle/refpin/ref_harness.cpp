// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// The reference pin: the reference renderer's own headers and sources for
// the structured-volume path, compiled unchanged from the reference tree by
// the recipe in oracle/Makefile (target `ref`, output oracle/_ref/), against
// a project-written restatement of the owl math library (oracle/refpin/shim,
// the owl submodule is empty) and a stub of the embree API header (no embree
// function is called), and exposed as C functions.  tests/test_oracle_refpin.py
// drives these and the CPU oracle with the same inputs and compares them bit
// for bit; tests/golden/make_ref_golden.py stores their outputs as fixtures.
// Nothing here is shipped or measured; the product never links it.
//
// Compiled from the reference (unchanged):
//   barney/common/barney-common.h   RNGSeed, Random2, hash
//   barney/volume/Volume.h          fastLog, Woodcock::sampleRange,
//                                   Volume::DD::sampleAndMap
//   barney/volume/TransferFunction.h  TransferFunction::DD::map, majorant
//   barney/volume/DDA.h             dda::dda3
//   barney/volume/StructuredData.{h,cu}  StructuredDataSampler::DD::sample,
//                                   StructuredData_computeMCs
//   barney/volume/MCAccelerator.h   MCVolumeAccel::isProg
//   barney/render/Ray.h             boxTest, Ray::setVolumeHit
//   barney/common/math.h            linear_to_srgb, make_8bit, make_rgba
//   rtcore/embree/Texture.cpp       TextureData, TextureSamplerT::tex3D
//   rtcore/embree/Float16.cpp       float32ToFloat16, float16ToFloat32
//   barney/volume/MCAccelerator.h   MCIsoSurfaceAccel::isProg
//   barney/material/DeviceMaterial.h, AnariMatte.h  createBSDF, setHit
//   barney/packedBSDF/Lambertian.h  eval, pdf, scatter
//   barney/render/DG.h              cosineSampleHemisphere, EvalRes
// Restated here (glue of the embree backend, no arithmetic of the path):
//   TraceInterface::transformNormal/PointFromObjectToWorldSpace (embree
//   Device.cpp:26-35: xfmVector(objectToWorldXfm->l, v), xfmPoint(
//   *objectToWorldXfm, v)); the trace set-up that rtcore/embree/Group.cpp:
//   34-78 does before calling isProg (tmin 0, tmax = ray.tMax, the
//   instance's index, geometry 0, primitive 0, identity instance transform).
// ref_shade.cpp (the shading step and env-map tables, also built for the
// multi-scatter configuration) and ref_gen.cpp (camera commit and ray
// generation) are the pin's other two parts.
// The owl math the reference calls (vec, box, frame, xfmVector ...) is the
// shim's restatement: the owl submodule is absent, so what depends on it --
// the Lambertian scatter direction through frame() -- is pinned only by
// restatement.
#include "barney/common/barney-common.h"
#include "barney/common/math.h"
#include "barney/volume/DDA.h"
#include "barney/volume/Volume.h"
#include "barney/volume/StructuredData.cu"
#include "barney/geometry/IsoSurface.h"
#include "barney/material/DeviceMaterial.h"
#include "rtcore/embree/Texture.h"
#include "rtcore/embree/ComputeInterface.h"
#include "rtcore/embree/TraceInterface.h"
#include "rtcore/embree/Float16.h"

using namespace BARNEY_NS;

namespace rtc {
namespace embree {
// embree Device.cpp:26-35
vec3f TraceInterface::transformNormalFromObjectToWorldSpace(vec3f v) const { return xfmVector(objectToWorldXfm->l, v); }
vec3f TraceInterface::transformPointFromObjectToWorldSpace(vec3f v) const { return xfmPoint(*objectToWorldXfm, v); }
}  // namespace embree
}  // namespace rtc

namespace {

TransferFunction::DD make_xf(const float *tf, int n, float lo, float hi, float base_density) {
  TransferFunction::DD xf;
  xf.values = (rtc::float4 *)tf;
  xf.domain = range1f{lo, hi};
  xf.baseDensity = base_density;
  xf.numValues = n;
  return xf;
}

// The structured field's LINEAR texture as StructuredData::setObject makes
// it (barney/volume/StructuredData.cu:154-173, barney/common/Texture.cpp:
// 94-105): FLOAT texels, CLAMP on every axis, unnormalised coordinates.
struct Field {
  rtc::embree::TextureData *data = nullptr;
  rtc::embree::Texture *linear = nullptr;
  Field(const float *scalars, const int dims[3]) {
    data = new rtc::embree::TextureData(nullptr, vec3i(dims[0], dims[1], dims[2]), rtc::FLOAT, scalars);
    rtc::TextureDesc desc;
    desc.filterMode = rtc::FILTER_MODE_LINEAR;
    desc.normalizedCoords = false;
    for (int i = 0; i < 3; i++) desc.addressMode[i] = rtc::CLAMP;
    linear = data->createTexture(desc);
  }
  ~Field() {
    delete linear->sampler;
    delete linear;
    delete data;
  }
  // StructuredDataSampler::getDD (StructuredData.cu:97-106)
  StructuredDataSampler::DD sampler(const int dims[3], const float origin[3], const float spacing[3]) const {
    StructuredDataSampler::DD dd;
    dd.texObj = linear->getDD();
    dd.cellGridOrigin = vec3f(origin[0], origin[1], origin[2]);
    dd.cellGridSpacing = vec3f(spacing[0], spacing[1], spacing[2]);
    dd.numCells = vec3i(dims[0] - 1, dims[1] - 1, dims[2] - 1);
    return dd;
  }
};

}  // namespace

#pragma GCC visibility push(default)
extern "C" {

int ref_pin_version(void) { return 1; }

// Random2(a, b) and n draws (barney-common.h:65-112)
void ref_rng_sequence(uint32_t a, uint32_t b, int n, float *out) {
  Random2 r(a, b);
  for (int i = 0; i < n; i++) out[i] = r();
}

// Random2(seed, hash) (32- or 64-bit hash) and n draws; the seed's state
// after the construction goes to *new_seed_state
void ref_rng_from_seed(uint64_t seed_state, uint64_t h, int use_u64, int n, float *out, uint64_t *new_seed_state) {
  RNGSeed s;
  s.state = seed_state;
  if (use_u64) {
    Random2 r(s, (uint64_t)h);
    for (int i = 0; i < n; i++) out[i] = r();
  } else {
    Random2 r(s, (uint32_t)h);
    for (int i = 0; i < n; i++) out[i] = r();
  }
  *new_seed_state = s.state;
}

// RNGSeed::seed(a, b) (barney-common.h:66-72): the state it leaves
uint64_t ref_rng_seed_state(uint32_t a, uint32_t b) {
  RNGSeed s;
  s.seed(a, b);
  return s.state;
}

uint64_t ref_hash3(uint32_t a, uint32_t b, uint32_t c) { return hash(a, b, c); }

float ref_fast_log(float f) { return fastLog(f); }

uint16_t ref_float_to_half(float f) { return float32ToFloat16(f); }
float ref_half_to_float(uint16_t h) { return float16ToFloat32(h); }

// TransferFunction::DD::map for n scalars -> n RGBA
void ref_tf_map(const float *tf, int tf_n, float lo, float hi, float base_density, const float *s, int n,
                float *rgba) {
  const TransferFunction::DD xf = make_xf(tf, tf_n, lo, hi, base_density);
  for (int i = 0; i < n; i++) {
    const vec4f v = xf.map(s[i]);
    rgba[4 * i + 0] = v.x;
    rgba[4 * i + 1] = v.y;
    rgba[4 * i + 2] = v.z;
    rgba[4 * i + 3] = v.w;
  }
}

// TransferFunction::DD::majorant for n (lower, upper) ranges
void ref_tf_majorant(const float *tf, int tf_n, float lo, float hi, float base_density, const float *ranges, int n,
                     float *out) {
  const TransferFunction::DD xf = make_xf(tf, tf_n, lo, hi, base_density);
  for (int i = 0; i < n; i++) out[i] = xf.majorant(range1f{ranges[2 * i], ranges[2 * i + 1]});
}

// dda::dda3 over a grid of grid[3] cells: the cells it visits with their
// (t0, t1), at most max_cells; returns the number visited
int ref_dda(const float org[3], const float dir[3], float t_max, const int grid[3], int max_cells, int *cells,
            float *t01) {
  int count = 0;
  dda::dda3(vec3f(org[0], org[1], org[2]), vec3f(dir[0], dir[1], dir[2]), t_max,
            vec3ui((uint32_t)grid[0], (uint32_t)grid[1], (uint32_t)grid[2]),
            [&](const vec3i &cell, float t0, float t1) -> bool {
              if (count >= max_cells) return false;
              cells[3 * count + 0] = cell.x;
              cells[3 * count + 1] = cell.y;
              cells[3 * count + 2] = cell.z;
              t01[2 * count + 0] = t0;
              t01[2 * count + 1] = t1;
              count++;
              return true;
            },
            false);
  return count;
}

// StructuredDataSampler::DD::sample (NaN outside the cell grid) at n points
void ref_sample_points(const float *scalars, const int dims[3], const float origin[3], const float spacing[3],
                       const float *P, int n, float *out) {
  Field f(scalars, dims);
  const StructuredDataSampler::DD dd = f.sampler(dims, origin, spacing);
  for (int i = 0; i < n; i++) out[i] = dd.sample(vec3f(P[3 * i], P[3 * i + 1], P[3 * i + 2]));
}

// Volume::DD::sampleAndMap at n points -> RGBA
void ref_sample_and_map(const float *scalars, const int dims[3], const float origin[3], const float spacing[3],
                        const float *tf, int tf_n, float lo, float hi, float base_density, const float *P, int n,
                        float *rgba) {
  Field f(scalars, dims);
  Volume::DD<StructuredDataSampler> vol;
  vol.sfSampler = f.sampler(dims, origin, spacing);
  vol.xf = make_xf(tf, tf_n, lo, hi, base_density);
  for (int i = 0; i < n; i++) {
    const vec4f v = vol.sampleAndMap(vec3f(P[3 * i], P[3 * i + 1], P[3 * i + 2]));
    rgba[4 * i + 0] = v.x;
    rgba[4 * i + 1] = v.y;
    rgba[4 * i + 2] = v.z;
    rgba[4 * i + 3] = v.w;
  }
}

// One ray through the structured volume: MCVolumeAccel<StructuredDataSampler>
// ::isProg (MCAccelerator.h:569-708) as the embree backend calls it for the
// volume's user geometry (tmin 0, tmax = ray.tMax, instance 0, geometry 0,
// identity instance transform).  majorants: per macrocell of
// ceil((dims-1)/cells_per_mc) per axis (StructuredData::buildMCs,
// StructuredData.cu:70-95).  On a hit returns 1 with *t_hit, the hit point
// P[3] and the phase function's albedo[3] as Ray::setVolumeHit stores them;
// *seed_state carries the ray's RNG seed in and out.
int ref_trace_ray(const float *scalars, const int dims[3], const float origin[3], const float spacing[3],
                  int cells_per_mc, const float *majorants, const float *tf, int tf_n, float lo, float hi,
                  float base_density, const float org[3], const float dir[3], float tmax, uint64_t *seed_state,
                  float *t_hit, float P[3], float albedo[3]) {
  Field f(scalars, dims);
  MCVolumeAccel<StructuredDataSampler>::DD dd;
  // StructuredData::commit (StructuredData.cu:176-180)
  const vec3f gridOrigin(origin[0], origin[1], origin[2]), gridSpacing(spacing[0], spacing[1], spacing[2]);
  const vec3i numCells(dims[0] - 1, dims[1] - 1, dims[2] - 1);
  dd.volume.sfCommon.worldBounds.lower = gridOrigin;
  dd.volume.sfCommon.worldBounds.upper = gridOrigin + gridSpacing * vec3f(numCells);
  dd.volume.sfSampler = f.sampler(dims, origin, spacing);
  dd.volume.xf = make_xf(tf, tf_n, lo, hi, base_density);
  dd.volume.userID = 0;
  // StructuredData::buildMCs (StructuredData.cu:73-76)
  const vec3i mcDims = divRoundUp(numCells, vec3i(cells_per_mc));
  dd.mcGrid.scalarRanges = nullptr;
  dd.mcGrid.dims = mcDims;
  dd.mcGrid.gridOrigin = dd.volume.sfCommon.worldBounds.lower;
  dd.mcGrid.gridSpacing = vec3f((float)cells_per_mc) * gridSpacing;
  dd.mcGrid.majorants = const_cast<float *>(majorants);

  render::Ray ray;
  std::memset((void *)&ray, 0, sizeof(ray));
  ray.org = vec3f(org[0], org[1], org[2]);
  ray.dir = vec3f(dir[0], dir[1], dir[2]);
  ray.tMax = tmax;
  ray.rngSeed.state = *seed_state;
  ray.bsdfType = PackedBSDF::NONE;

  render::OptixGlobals globals;
  std::memset((void *)&globals, 0, sizeof(globals));
  globals.hitIDs = nullptr;

  embree_for_barney::RTCRay er;
  er.org_x = ray.org.x; er.org_y = ray.org.y; er.org_z = ray.org.z; er.tnear = 0.f;
  er.dir_x = ray.dir.x; er.dir_y = ray.dir.y; er.dir_z = ray.dir.z; er.time = 0.f;
  er.tfar = ray.tMax;
  er.mask = ~0u; er.id = 0; er.flags = 0;
  const affine3f identity{LinearSpace3f(vec3f(1.f, 0.f, 0.f), vec3f(0.f, 1.f, 0.f), vec3f(0.f, 0.f, 1.f)),
                          vec3f(0.f)};
  const int instIDs[1] = {0};
  rtc::embree::TraceInterface ti;
  std::memset((void *)&ti, 0, sizeof(ti));
  ti.isec_t = INFINITY;
  ti.instIdx = 0;
  ti.geomID = 0;
  ti.primID = 0;
  ti.worldOrigin = ray.org;
  ti.worldDirection = ray.dir;
  ti.prd = &ray;
  ti.instIDs = instIDs;
  ti.geomData = &dd;
  ti.lpData = &globals;
  ti.objectToWorldXfm = &identity;
  ti.worldToObjectXfm = &identity;
  ti.embreeRay = &er;
  MCVolumeAccel<StructuredDataSampler>::isProg(ti);
  *seed_state = ray.rngSeed.state;
  if (ray.bsdfType == PackedBSDF::NONE) return 0;
  *t_hit = ray.tMax;
  P[0] = ray.P.x; P[1] = ray.P.y; P[2] = ray.P.z;
  const render::packedBSDF::Phase &phase = (const render::packedBSDF::Phase &)ray.hitBSDF;
  albedo[0] = phase.albedo.x; albedo[1] = phase.albedo.y; albedo[2] = phase.albedo.z;
  return 1;
}

// One ray against an iso-surface of the structured field:
// MCIsoSurfaceAccel<StructuredDataSampler>::isProg (MCAccelerator.h:338-567)
// as the embree backend calls it for the iso-surface's user geometry (tmin
// 0, tmax = ray.tMax, geometry 0, primitive 0, instance `inst`, identity
// instance transform), with one AnariMatte material of constant color and
// opacity (DeviceMaterial::setHit, AnariMatte::DD::createBSDF).  ranges: the
// field's macrocell scalar ranges, (lower, upper) per macrocell.  On a hit
// returns 1 with *t_hit, P[3], the normal as Ray::setHit stores it (three
// halfs) and the Lambertian's albedo (xyz) and alpha (w); *seed_state carries
// the ray's RNG seed in and out.
int ref_iso_hit(const float *scalars, const int dims[3], const float origin[3], const float spacing[3],
                int cells_per_mc, const float *ranges, float iso, const float color[4], float opacity, int inst,
                const float org[3], const float dir[3], float tmax, uint64_t *seed_state, float *t_hit, float P[3],
                uint16_t N[3], float albedo[4]) {
  Field f(scalars, dims);
  MCIsoSurfaceAccel<StructuredDataSampler>::DD dd;
  std::memset((void *)&dd, 0, sizeof(dd));
  const vec3f gridOrigin(origin[0], origin[1], origin[2]), gridSpacing(spacing[0], spacing[1], spacing[2]);
  const vec3i numCells(dims[0] - 1, dims[1] - 1, dims[2] - 1);
  dd.isoSurface.sfCommon.worldBounds.lower = gridOrigin;
  dd.isoSurface.sfCommon.worldBounds.upper = gridOrigin + gridSpacing * vec3f(numCells);
  dd.isoSurface.sfSampler = f.sampler(dims, origin, spacing);
  dd.isoSurface.isoValue = iso;
  dd.isoSurface.materialID = 0;
  dd.isoSurface.userID = 0;
  dd.mcGrid.scalarRanges = (range1f *)const_cast<float *>(ranges);
  dd.mcGrid.dims = divRoundUp(numCells, vec3i(cells_per_mc));
  dd.mcGrid.gridOrigin = dd.isoSurface.sfCommon.worldBounds.lower;
  dd.mcGrid.gridSpacing = vec3f((float)cells_per_mc) * gridSpacing;

  // AnariMatte::getDD with VALUE parameters (Material.h:19-47, Material.cpp:37-52)
  render::DeviceMaterial mat;
  std::memset((void *)&mat, 0, sizeof(mat));
  mat.type = render::DeviceMaterial::TYPE_AnariMatte;
  mat.anariMatte.color.type = render::PossiblyMappedParameter::VALUE;
  mat.anariMatte.color.value = rtc::float4{color[0], color[1], color[2], color[3]};
  mat.anariMatte.opacity.type = render::PossiblyMappedParameter::VALUE;
  mat.anariMatte.opacity.value = rtc::float4{opacity, 0.f, 0.f, 1.f};

  render::Ray ray;
  std::memset((void *)&ray, 0, sizeof(ray));
  ray.org = vec3f(org[0], org[1], org[2]);
  ray.dir = vec3f(dir[0], dir[1], dir[2]);
  ray.tMax = tmax;
  ray.rngSeed.state = *seed_state;
  ray.bsdfType = PackedBSDF::NONE;

  render::OptixGlobals globals;
  std::memset((void *)&globals, 0, sizeof(globals));
  globals.hitIDs = nullptr;
  globals.world.materials = &mat;
  globals.world.samplers = nullptr;

  embree_for_barney::RTCRay er;
  er.org_x = ray.org.x; er.org_y = ray.org.y; er.org_z = ray.org.z; er.tnear = 0.f;
  er.dir_x = ray.dir.x; er.dir_y = ray.dir.y; er.dir_z = ray.dir.z; er.time = 0.f;
  er.tfar = ray.tMax;
  er.mask = ~0u; er.id = 0; er.flags = 0;
  const affine3f identity{LinearSpace3f(vec3f(1.f, 0.f, 0.f), vec3f(0.f, 1.f, 0.f), vec3f(0.f, 0.f, 1.f)),
                          vec3f(0.f)};
  std::vector<int> instIDs(inst + 1);
  for (int i = 0; i <= inst; i++) instIDs[i] = i;
  rtc::embree::TraceInterface ti;
  std::memset((void *)&ti, 0, sizeof(ti));
  ti.isec_t = INFINITY;
  ti.instIdx = inst;
  ti.geomID = 0;
  ti.primID = 0;
  ti.worldOrigin = ray.org;
  ti.worldDirection = ray.dir;
  ti.prd = &ray;
  ti.instIDs = instIDs.data();
  ti.geomData = &dd;
  ti.lpData = &globals;
  ti.objectToWorldXfm = &identity;
  ti.worldToObjectXfm = &identity;
  ti.embreeRay = &er;
  MCIsoSurfaceAccel<StructuredDataSampler>::isProg(ti);
  *seed_state = ray.rngSeed.state;
  if (ray.bsdfType == PackedBSDF::NONE) return 0;
  *t_hit = ray.tMax;
  P[0] = ray.P.x; P[1] = ray.P.y; P[2] = ray.P.z;
  const uint16_t *nh = (const uint16_t *)&ray.N;
  N[0] = nh[0]; N[1] = nh[1]; N[2] = nh[2];
  const render::packedBSDF::Lambertian &lam = (const render::packedBSDF::Lambertian &)ray.hitBSDF;
  albedo[0] = lam.albedo.x; albedo[1] = lam.albedo.y; albedo[2] = lam.albedo.z;
  albedo[3] = lam.alpha;
  return 1;
}

// The Lambertian BSDF an AnariMatte material of constant color makes
// (AnariMatte.h:50-62, packedBSDF/Lambertian.h), at a surface point with
// normal Ng (dg.Ng = dg.Ns, as shadeRays.cu:625-629 sets them) seen from
// wo: eval and pdf toward wi, then one scatter drawing from Random2(a, b).
// out: eval value[3], eval pdf, pdf(wi), scatter dir[3], scatter pdf,
// scatter f_r[3].
void ref_lambertian(const float color[4], const float Ng[3], const float wo[3], const float wi[3], uint32_t a,
                    uint32_t b, float out[12]) {
  render::AnariMatte::DD m;
  std::memset((void *)&m, 0, sizeof(m));
  m.color.type = render::PossiblyMappedParameter::VALUE;
  m.color.value = rtc::float4{color[0], color[1], color[2], color[3]};
  m.opacity.type = render::PossiblyMappedParameter::VALUE;
  m.opacity.value = rtc::float4{1.f, 0.f, 0.f, 1.f};
  render::HitAttributes hit;
  const PackedBSDF bsdf = m.createBSDF(hit, nullptr, false);
  render::DG dg;
  dg.Ng = vec3f(Ng[0], Ng[1], Ng[2]);
  dg.Ns = dg.Ng;
  dg.wo = vec3f(wo[0], wo[1], wo[2]);
  dg.P = vec3f(0.f);
  dg.insideMedium = false;
  const vec3f w(wi[0], wi[1], wi[2]);
  const render::EvalRes e = bsdf.eval(dg, w);
  out[0] = e.value.x; out[1] = e.value.y; out[2] = e.value.z; out[3] = e.pdf;
  out[4] = bsdf.pdf(dg, w);
  Random2 r(a, b);
  render::ScatterResult s;
  bsdf.scatter(s, dg, r);
  out[5] = s.dir.x; out[6] = s.dir.y; out[7] = s.dir.z; out[8] = s.pdf;
  out[9] = s.f_r.x; out[10] = s.f_r.y; out[11] = s.f_r.z;
}

// StructuredData::buildMCs (StructuredData.cu:29-61, 70-95): the macrocell
// scalar ranges of a structured field, cellsPerMC = 8, read through the
// field's NEAREST texture (StructuredData::setObject, :153-172: CLAMP on
// every axis, unnormalised coordinates), StructuredData_computeMCs run for
// every macrocell; ranges: 2 floats per macrocell, x fastest
void ref_mc_ranges(const float *scalars, const int dims[3], float *ranges) {
  rtc::embree::TextureData data(nullptr, vec3i(dims[0], dims[1], dims[2]), rtc::FLOAT, scalars);
  rtc::TextureDesc desc;
  desc.filterMode = rtc::FILTER_MODE_POINT;
  desc.normalizedCoords = false;
  for (int i = 0; i < 3; i++) desc.addressMode[i] = rtc::CLAMP;
  rtc::embree::Texture *nn = data.createTexture(desc);
  const vec3i numCells(dims[0] - 1, dims[1] - 1, dims[2] - 1);
  const vec3i mcDims = divRoundUp(numCells, vec3i(cellsPerMC));
  MCGrid::DD grid;
  std::memset((void *)&grid, 0, sizeof(grid));
  grid.dims = mcDims;
  grid.scalarRanges = (range1f *)ranges;
  rtc::embree::ComputeInterface ci;
  std::memset((void *)&ci, 0, sizeof(ci));
  ci.blockDim = vec3ui(1, 1, 1);
  const int n = mcDims.x * mcDims.y * mcDims.z;
  for (int t = 0; t < n; t++) {
    ci.blockIdx = vec3ui(t, 0, 0);
    StructuredData_computeMCs(ci, grid, vec3i(dims[0], dims[1], dims[2]), nn->getDD());
  }
  delete nn->sampler;
  delete nn;
}

// linear_to_srgb and the 8-bit packing of the frame-buffer read
// (common/math.h:52-116) for n RGBA pixels; srgb = 0: make_rgba of the
// linear values, 1: of their sRGB transform
void ref_rgba8(const float *rgba, int n, int srgb, uint32_t *out) {
  for (int i = 0; i < n; i++) {
    vec4f c(rgba[4 * i], rgba[4 * i + 1], rgba[4 * i + 2], rgba[4 * i + 3]);
    if (srgb) {
      c.x = linear_to_srgb(c.x);
      c.y = linear_to_srgb(c.y);
      c.z = linear_to_srgb(c.z);
    }
    out[i] = make_rgba(c);
  }
}

}  // extern "C"
#pragma GCC visibility pop
