// ref_shade.cpp -- TEST INFRASTRUCTURE ONLY.
//
// The reference pin's shading step (see ref_harness.cpp for how the pin is
// built): the reference's own code, compiled unchanged from the reference
// tree --
//   barney/kernels/shadeRays.cu  bounce() with sampleLights, sampleDirLights,
//                                sampleEnvLight, radianceFromEnv, safe_eps
//   barney/light/EnvMap.{h,cu}   EnvMapLight::DD::sample and ::pdf, and the
//                                importance-table kernels ComputeWeights_xy,
//                                ComputeCDFs_doLine, Normalize_cdf_y
//   barney/packedBSDF/Phase.h, Lambertian.h, barney/material/AnariMatte.h
//   rtcore/embree/Texture.cpp    the env map's 2D texture
// -- exposed as C functions on the records of oracle/gbv_oracle.h
// (orc_shade_world, orc_shade_path).  oracle/Makefile builds this file twice:
// with the configuration of the default build (single scattering,
// SCI_VIS_MODE) into _ref/libbarney_ref.so and with
// BARNEY_USE_MULTI_SCATTERING=1 into _ref/libbarney_ref_ms.so, as the
// reference's CMake option selects one or the other at compile time.
// Restated here: only the set-up of the records the kernels receive --
// World::DD, Renderer::DD, EnvMapLight::DD (as EnvMapLight::getDD fills it
// from the given tables and transforms), the texture as barney::Texture
// creates a 2D texture (dims (W, H, 0), normalized coordinates, linear
// filter, the app's address modes), the incoming Ray (setVolumeHit, or
// setHit with the material's BSDF) and PathState, and the per-thread
// ComputeInterface of the table kernels.
#include <cstring>
#include <memory>
#include "barney/kernels/shadeRays.cu"
#include "barney/light/EnvMap.cu"
#include "barney/material/DeviceMaterial.h"
#include "../gbv_oracle.h"

using namespace BARNEY_NS;

namespace {

struct EnvTexture {
  std::unique_ptr<rtc::embree::TextureData> data;
  rtc::embree::Texture *tex = nullptr;
  EnvTexture(const float *texels, int W, int H, const int addr[2]) {
    // barney::Texture for bnTexture2DCreate (barney/common/Texture.cpp:84-110,
    // barney/api/barney.cu:288-315)
    data.reset(new rtc::embree::TextureData(nullptr, vec3i(W, H, 0), rtc::FLOAT4, texels));
    rtc::TextureDesc desc;
    desc.filterMode = rtc::FILTER_MODE_LINEAR;
    desc.addressMode[0] = (rtc::AddressMode)addr[0];
    desc.addressMode[1] = (rtc::AddressMode)addr[1];
    tex = data->createTexture(desc);
  }
  ~EnvTexture() {
    if (tex) {
      delete tex->sampler;
      delete tex;
    }
  }
};

linear3f lin(const float m[9]) {
  return linear3f(vec3f(m[0], m[1], m[2]), vec3f(m[3], m[4], m[5]), vec3f(m[6], m[7], m[8]));
}

}  // namespace

#pragma GCC visibility push(default)
extern "C" {

// 1 for the multi-scatter build of this library, 0 for the default build
int ref_shade_multi_scatter(void) { return BARNEY_USE_MULTI_SCATTERING; }

// EnvMapLight::computeCDFs (barney/light/EnvMap.cu:181-238): the per-texel
// weights, the per-row CDFs with the rows' weights, and the normalized row
// CDF, each kernel run for every thread index of its launch in turn
void ref_env_cdfs(const float *texels, const int dims[2], const int addr[2], float *cdf_y, float *cdf_x) {
  EnvTexture t(texels, dims[0], dims[1], addr);
  const vec2i d(dims[0], dims[1]);
  rtc::embree::ComputeInterface ci;
  std::memset((void *)&ci, 0, sizeof(ci));
  ci.blockDim = vec3ui(1, 1, 1);
  ci.gridDim = vec3ui(1, 1, 1);
  ComputeWeights_xy weights = {cdf_x, t.tex->getDD(), d};
  for (int iy = 0; iy < d.y; iy++)
    for (int ix = 0; ix < d.x; ix++) {
      ci.threadIdx = vec3ui(ix, iy, 0);
      weights.run(ci);
    }
  ComputeCDFs_doLine lines = {cdf_y, cdf_x, d};
  for (int y = 0; y < d.y; y++) {
    ci.threadIdx = vec3ui(y, 0, 0);
    lines.run(ci);
  }
  Normalize_cdf_y norm = {cdf_y, cdf_x, d};
  ci.threadIdx = vec3ui(0, 0, 0);
  norm.run(ci);
}

// bounce() as _shadeRays calls it (shadeRays.cu:881-941: the shadow ray
// starts invalid, tMax = -1) for the path *io at depth `depth`
void ref_bounce(const orc_shade_world *w, int depth, orc_shade_path *io, orc_shade_path *sh, float fragment[3]) {
  using namespace render;
  World::DD world;
  std::memset((void *)&world, 0, sizeof(world));
  DirLight::DD dl[4];
  const int nd = w->num_dir_lights < 0 ? 0 : (w->num_dir_lights > 4 ? 4 : w->num_dir_lights);
  for (int i = 0; i < nd; i++) {
    dl[i].direction = vec3f(w->dir_light_dir[i][0], w->dir_light_dir[i][1], w->dir_light_dir[i][2]);
    dl[i].color = vec3f(w->dir_light_color[i][0], w->dir_light_color[i][1], w->dir_light_color[i][2]);
    dl[i].radiance = w->dir_light_radiance[i];
  }
  world.numDirLights = nd;
  world.dirLights = dl;
  std::unique_ptr<EnvTexture> env;
  if (w->env_texels) {
    env.reset(new EnvTexture(w->env_texels, w->env_dims[0], w->env_dims[1], w->env_addr));
    EnvMapLight::DD &e = world.envMapLight;
    e.texture = env->tex->getDD();
    e.dims = vec2i(w->env_dims[0], w->env_dims[1]);
    e.scale = w->env_scale;
    e.toWorld = lin(w->env_to_world);
    e.toLocal = lin(w->env_to_local);
    e.cdf_y = w->env_cdf_y;
    e.allCDFs_x = w->env_cdf_x;
  }
  Renderer::DD renderer;
  std::memset((void *)&renderer, 0, sizeof(renderer));
  renderer.ambientRadiance = w->ambient_radiance;
  renderer.pathsPerPixel = 1;
#if BARNEY_USE_MULTI_SCATTERING
  renderer.maxVolumeBounces = w->max_volume_bounces;
  renderer.volumeMultiScatter = w->volume_multi_scatter;
#endif

  Ray ray;
  std::memset((void *)&ray, 0, sizeof(ray));
  ray.org = vec3f(io->org[0], io->org[1], io->org[2]);
  ray.dir = vec3f(io->dir[0], io->dir[1], io->dir[2]);
  ray.tMax = io->tmax;
  ray.rngSeed.state = io->seed;
  ray.bsdfType = PackedBSDF::NONE;
  ray.isShadowRay = io->shadow != 0;
  ray.missColor = bn_float4{io->miss_color[0], io->miss_color[1], io->miss_color[2], io->miss_color[3]};
  const vec3f P(io->P[0], io->P[1], io->P[2]);
  if (io->hit == 1) {
    const vec3f rgb(io->rgb[0], io->rgb[1], io->rgb[2]);
#if BARNEY_USE_MULTI_SCATTERING
    ray.setVolumeHit(P, io->tmax, rgb, io->g, io->scattering_albedo);
#else
    ray.setVolumeHit(P, io->tmax, rgb);
#endif
  } else if (io->hit == 2) {
    AnariMatte::DD m;
    std::memset((void *)&m, 0, sizeof(m));
    m.color.type = PossiblyMappedParameter::VALUE;
    m.color.value = rtc::float4{io->color[0], io->color[1], io->color[2], io->color[3]};
    m.opacity.type = PossiblyMappedParameter::VALUE;
    m.opacity.value = rtc::float4{io->opacity, 0.f, 0.f, 1.f};
    HitAttributes hit;
    ray.setHit(P, vec3f(io->N[0], io->N[1], io->N[2]), io->tmax, m.createBSDF(hit, nullptr, false));
  }
  PathState st;
  std::memset((void *)&st, 0, sizeof(st));
  uint16_t *tp = (uint16_t *)&st.throughput;
  tp[0] = io->tp[0]; tp[1] = io->tp[1]; tp[2] = io->tp[2];
  st.misWeight = io->mis;
  st.numDiffuseBounces = io->diffuse_bounces;
#if BARNEY_USE_MULTI_SCATTERING
  st.numVolumeBounces = io->volume_bounces;
#endif
  Ray shadowRay;
  PathState shadowState;
  std::memset((void *)&shadowRay, 0, sizeof(shadowRay));
  std::memset((void *)&shadowState, 0, sizeof(shadowState));
  shadowRay.tMax = -1.f;
  vec3f frag = 0.f;
  bounce(0, world, renderer, frag, ray, st, shadowRay, shadowState, depth);
  fragment[0] = frag.x; fragment[1] = frag.y; fragment[2] = frag.z;
  io->org[0] = ray.org.x; io->org[1] = ray.org.y; io->org[2] = ray.org.z;
  io->dir[0] = ray.dir.x; io->dir[1] = ray.dir.y; io->dir[2] = ray.dir.z;
  io->tmax = ray.tMax;
  io->seed = ray.rngSeed.state;
  io->hit = ray.hadHit() ? (ray.bsdfType == PackedBSDF::TYPE_Lambertian ? 2 : 1) : 0;
  io->tp[0] = tp[0]; io->tp[1] = tp[1]; io->tp[2] = tp[2];
  io->mis = st.misWeight;
  io->diffuse_bounces = st.numDiffuseBounces;
#if BARNEY_USE_MULTI_SCATTERING
  io->volume_bounces = st.numVolumeBounces;
#endif
  std::memset((void *)sh, 0, sizeof(*sh));
  sh->tmax = -1.f;
  if (shadowRay.tMax > 0.f) {
    sh->org[0] = shadowRay.org.x; sh->org[1] = shadowRay.org.y; sh->org[2] = shadowRay.org.z;
    sh->dir[0] = shadowRay.dir.x; sh->dir[1] = shadowRay.dir.y; sh->dir[2] = shadowRay.dir.z;
    sh->tmax = shadowRay.tMax;
    sh->seed = shadowRay.rngSeed.state;
    sh->shadow = shadowRay.isShadowRay ? 1 : 0;
    const uint16_t *stp = (const uint16_t *)&shadowState.throughput;
    sh->tp[0] = stp[0]; sh->tp[1] = stp[1]; sh->tp[2] = stp[2];
    sh->mis = shadowState.misWeight;
  }
}

}  // extern "C"
#pragma GCC visibility pop
