// render.cu -- host entry points of the frame render: parameter set-up
// (camera, lights, env map, macrocell grid) and dispatch to the kernels of
// the scene's voxel store (render_store_*.cu).
#include <cstdio>
#include "render_kernel.cuh"

namespace gbv {
static M3 inverse3(const M3 &m) {
  vec3 a = cross(m.vy, m.vz), b = cross(m.vz, m.vx), c = cross(m.vx, m.vy);
  float det = dot(m.vx, a);
  float r = 1.f / det;
  M3 t;
  t.vx = vec3(a.x, b.x, c.x) * r;
  t.vy = vec3(a.y, b.y, c.y) * r;
  t.vz = vec3(a.z, b.z, c.z) * r;
  return t;
}

bool make_field_geom(const gbv_scene *s, FieldGeom &F) {
  for (int i = 0; i < 3; i++) {
    F.N[i] = s->dims[i];
    F.C[i] = s->dims[i] - 1;
  }
  F.origin = vec3(s->origin[0], s->origin[1], s->origin[2]);
  vec3 spacing(s->spacing[0], s->spacing[1], s->spacing[2]);
  F.rcpSpacing = rcp(spacing);
  F.boundsLo = F.origin;
  F.boundsHi = F.origin + spacing * vec3((float)F.C[0], (float)F.C[1], (float)F.C[2]);
  return true;
}

void commit_camera(const float pos[3], const float dir[3], const float up[3], float fovy, vec3 &lens00,
                   vec3 &dir00, vec3 &du, vec3 &dv) {
  // PerspectiveCamera::set3f("direction") normalizes; commit() (Camera.cu:83-97)
  vec3 direction = normalize(vec3(dir[0], dir[1], dir[2]));
  vec3 vup(up[0], up[1], up[2]);
  vec3 d00 = normalize(direction);
  vec3 ddu = normalize(cross(d00, vup));
  vec3 ddv = normalize(cross(ddu, d00));
  d00 = d00 * (float)(1.f / (2.0f * tanf((0.5f * fovy) * (float)M_PI / 180.0f)));
  lens00 = vec3(pos[0], pos[1], pos[2]);
  dir00 = d00;
  du = ddu;
  dv = ddv;
}

static gbv_status fill_params(const gbv_scene *s, RenderParams &p) {
  p.xf.v = reinterpret_cast<const float4 *>(s->d_tf);
  p.xf.n = s->tf_n;
  p.xf.lo = s->domain[0];
  p.xf.span = s->domain[1] - s->domain[0];
  p.xf.baseDensity = s->base_density;
  p.G.maj = s->d_majorants;
  if (s->layout == GBV_LAYOUT_NANOVDB) {
    // NanoVDBData::commit and ::buildMCs (barney/volume/NanoVDB.cu:70-92,
    // 193-232): world bounds from the grid, macrocells over them
    if (!s->nanovdb) return set_error(GBV_ERROR_INVALID_ARGUMENT, "NanoVDB scene without its parsed grid");
    const gbv_nanovdb_info &nv = *s->nanovdb;
    memset(&p.F, 0, sizeof(p.F));
    p.F.boundsLo = vec3(nv.world_lo[0], nv.world_lo[1], nv.world_lo[2]);
    p.F.boundsHi = vec3(nv.world_hi[0], nv.world_hi[1], nv.world_hi[2]);
    p.F.origin = p.F.boundsLo;
    for (int i = 0; i < 3; i++) p.G.M[i] = nv.mc_dims[i];
    p.G.origin = p.F.boundsLo;
    p.G.spacing = (p.F.boundsHi - p.F.boundsLo) * rcp(vec3((float)nv.mc_dims[0], (float)nv.mc_dims[1],
                                                           (float)nv.mc_dims[2]));
    p.nvdb = make_nvdb_grid(s->d_voxels, nv);
  } else {
    make_field_geom(s, p.F);
    int M[3];
    gbv_status st = gbv_mc_dims(s->dims, s->cells_per_mc, M);
    if (st != GBV_OK) return st;
    for (int i = 0; i < 3; i++) p.G.M[i] = M[i];
    p.G.origin = p.F.boundsLo;
    p.G.spacing = vec3((float)s->cells_per_mc) * vec3(s->spacing[0], s->spacing[1], s->spacing[2]);
  }
  p.rcpMc = rcp(p.G.spacing);
  p.vox = s->d_voxels;
  p.so = reinterpret_cast<const float2 *>(s->d_scale_offset);
  {
    int l[3];
    if (!resolve_brick_shape(s->brick_log2, l))
      return set_error(GBV_ERROR_INVALID_ARGUMENT, "brick_log2: each 1..6 (0 = 3), sum at most 15");
    p.brick = make_brick_geom(s->dims, l);
  }
  commit_camera(s->cam_pos, s->cam_dir, s->cam_up, s->fovy, p.lens00, p.dir00, p.du, p.dv);
  p.numDir = s->num_dir_lights < 0 ? 0 : (s->num_dir_lights > 4 ? 4 : s->num_dir_lights);
  for (int i = 0; i < p.numDir; i++) {
    p.dir[i].direction = normalize(vec3(s->dir_light_dir[i][0], s->dir_light_dir[i][1], s->dir_light_dir[i][2]));
    p.dir[i].color = vec3(s->dir_light_color[i][0], s->dir_light_color[i][1], s->dir_light_color[i][2]);
    p.dir[i].radiance = s->dir_light_radiance[i];
  }
  p.hasEnv = s->d_env_texels != nullptr;
  if (p.hasEnv) {
    if (!s->d_env_cdf_x || !s->d_env_cdf_y || s->env_dims[0] <= 0 || s->env_dims[1] <= 0)
      return set_error(GBV_ERROR_INVALID_ARGUMENT, "env map needs texels, both CDF tables and positive dims");
    EnvDev &e = p.env;
    e.tex = reinterpret_cast<const float4 *>(s->d_env_texels);
    e.cdf_y = s->d_env_cdf_y;
    e.cdf_x = s->d_env_cdf_x;
    e.W = s->env_dims[0];
    e.H = s->env_dims[1];
    e.addr[0] = s->env_addr[0];
    e.addr[1] = s->env_addr[1];
    e.scale = s->env_scale;
    // EnvMap.cu:164-179
    vec3 up(s->env_up[0], s->env_up[1], s->env_up[2]);
    vec3 dir(s->env_dir[0], s->env_dir[1], s->env_dir[2]);
    e.toWorld.vz = -normalize(up);
    e.toWorld.vy = -normalize(cross(e.toWorld.vz, dir));
    e.toWorld.vx = normalize(cross(e.toWorld.vy, e.toWorld.vz));
    e.toLocal = inverse3(e.toWorld);
  }
  p.bg = make_float4(s->bg_color[0], s->bg_color[1], s->bg_color[2], s->bg_color[3]);
  p.ambient = s->ambient_radiance;
  p.multi = s->multi_scatter;
  p.volMS = s->volume_multi_scatter;
  p.maxVB = s->max_volume_bounces;
  p.aniso = s->anisotropy;
  p.scatAlb = s->scattering_albedo;
  p.rank = 0;
  p.numRanks = 1;
  p.capFlag = nullptr;
  // the world's instances (gbv_iso_surface): the volume's and the
  // iso-surface's stream hashes and their order
  p.hasVolume = s->d_majorants != nullptr;
  if (!p.hasVolume) p.G.maj = nullptr;
  if (s->volume_instance < 0) return set_error(GBV_ERROR_INVALID_ARGUMENT, "volume_instance must be >= 0");
  p.volHash = fnv_hash3((uint32_t)s->volume_instance, 0, 0);
  p.isoOn = s->iso != nullptr;
  p.isoFirst = 0;
  p.isoValue = p.isoDelta = 0.f;
  p.isoAlpha = 1.f;
  p.isoRanges = nullptr;
  p.isoAlbedo = vec3(0.f);
  p.isoHash = 0;
  p.depth = s->d_depth;
  p.primId = s->d_prim_id;
  p.instId = s->d_inst_id;
  p.objId = s->d_obj_id;
  p.volInst = s->volume_instance;
  p.volUser = s->volume_user_id;
  p.isoInst = p.isoUser = -1;
  if (p.isoOn) {
    const gbv_iso_surface &iso = *s->iso;
    if (!iso.d_ranges) return set_error(GBV_ERROR_INVALID_ARGUMENT, "iso-surface without macrocell ranges");
    if (iso.instance < 0 || (p.hasVolume && iso.instance == s->volume_instance))
      return set_error(GBV_ERROR_INVALID_ARGUMENT,
                       "iso-surface instance must be >= 0 and differ from the volume's");
    p.isoFirst = !p.hasVolume || iso.instance < s->volume_instance;
    p.isoHash = fnv_hash3((uint32_t)iso.instance, 0, 0);
    p.isoInst = iso.instance;
    p.isoUser = iso.user_id;
    p.isoValue = iso.iso_value;
    p.isoRanges = reinterpret_cast<const float2 *>(iso.d_ranges);
    // MCAccelerator.h:476-479: delta = |bounds size| * .1 / (Mx + My + Mz)
    const vec3 size = p.F.boundsHi - p.F.boundsLo;
    p.isoDelta = sqrtf(dot(size, size)) * .1f / (float)(p.G.M[0] + p.G.M[1] + p.G.M[2]);
    // AnariMatte::DD::createBSDF (AnariMatte.h:50-62) with VALUE parameters
    // (PossiblyMappedParameter::DD::eval, Material.h:101-106: a NaN value
    // reads as (0, 0, 0, 1); opacity is (opacity, 0, 0, 1))
    float c[4] = {iso.color[0], iso.color[1], iso.color[2], iso.color[3]};
    if (c[0] != c[0]) {
      c[0] = c[1] = c[2] = 0.f;
      c[3] = 1.f;
    }
    const float opacity = iso.opacity != iso.opacity ? 0.f : iso.opacity;
    const float reflectance = .85f;
    p.isoAlbedo = reflectance * vec3(c[0], c[1], c[2]) * kOneOverPi;
    p.isoAlpha = c[3] * opacity;
  }
  return GBV_OK;
}

// A scene's field, and its volume unless an iso-surface stands alone
// (gbv_scene.iso with d_majorants == 0).
static bool scene_complete(const gbv_scene *s) {
  if (!s->d_voxels || (s->layout != GBV_LAYOUT_NANOVDB && s->cells_per_mc <= 0)) return false;
  const bool volume = s->d_majorants != nullptr || s->iso == nullptr;
  return !volume || (s->d_majorants && s->d_tf && s->tf_n >= 2);
}

}  // namespace gbv

using namespace gbv;

namespace gbv {

// Launch settings of a gbv_render_config (zero fields: defaults); false if
// a field is out of range.
static bool resolve_config(const gbv_render_config *c, RenderParams &p, LaunchChoice &lc) {
  p.skip = kSkipDefault;
  p.threshold = kThresholdDefault;
  p.profile = 0;
  lc = LaunchChoice();
  if (!c) return true;
  if (c->blocks_per_sm != 0 && (c->blocks_per_sm < 4 || c->blocks_per_sm > 6)) return false;
  if (c->threshold_pct < 0 || c->threshold_pct > 100) return false;
  if (c->skip_cells < 0 || c->skip_cells > 1024) return false;
  if (c->stage < GBV_STAGE_DEFAULT || c->stage > GBV_STAGE_BALLOT) return false;
  if (c->profile != 0 && c->profile != 1) return false;
  if (c->mode != GBV_RENDER_PERSISTENT && c->mode != GBV_RENDER_WAVEFRONT) return false;
  if (c->reserved[0] || c->reserved[1]) return false;
  lc.mode = c->mode;
  if (c->blocks_per_sm) lc.occ = c->blocks_per_sm;
  lc.stage = c->stage;
  if (c->threshold_pct) p.threshold = c->threshold_pct;
  else if (c->mode == GBV_RENDER_WAVEFRONT) p.threshold = 25;
  if (c->skip_cells) p.skip = c->skip_cells;
  p.profile = c->profile;
  return true;
}

static gbv_status render_frame(const char *fn, const gbv_scene *s, float *d_accum, int width, int height,
                               int accum_id_start, int spp, int rank, int num_ranks, unsigned long long *d_counters,
                               void *stream, int *d_cap_flag = nullptr, const gbv_render_config *config = nullptr) {
  char msg[160];
  if (!s || !d_accum || width <= 0 || height <= 0 || spp < 0 || accum_id_start < 0) {
    snprintf(msg, sizeof msg, "%s: null pointer or non-positive size", fn);
    return set_error(GBV_ERROR_INVALID_ARGUMENT, msg);
  }
  if (num_ranks < 1 || rank < 0 || rank >= num_ranks) {
    snprintf(msg, sizeof msg, "%s: rank must be in [0, num_ranks) and num_ranks >= 1", fn);
    return set_error(GBV_ERROR_INVALID_ARGUMENT, msg);
  }
  if (!scene_complete(s)) {
    snprintf(msg, sizeof msg, "%s: scene lacks voxels, majorants or a transfer function", fn);
    return set_error(GBV_ERROR_INVALID_ARGUMENT, msg);
  }
  if (s->layout == GBV_LAYOUT_LINEAR && s->format != GBV_VOXEL_F32) {
    snprintf(msg, sizeof msg, "%s: the linear layout holds FP32 voxels only", fn);
    return set_error(GBV_ERROR_UNSUPPORTED, msg);
  }
  if (s->format == GBV_VOXEL_U8_SCALED && !s->d_scale_offset) {
    snprintf(msg, sizeof msg, "%s: U8 voxels need the brick scale/offset table", fn);
    return set_error(GBV_ERROR_INVALID_ARGUMENT, msg);
  }
  RenderParams p;
  LaunchChoice lc;
  if (!resolve_config(config, p, lc)) {
    snprintf(msg, sizeof msg, "%s: launch config out of range (blocks 4..6, threshold 0..100, skip 0..1024, stage 0..3, mode 0..1)",
             fn);
    return set_error(GBV_ERROR_INVALID_ARGUMENT, msg);
  }
  if (s->iso && lc.mode == GBV_RENDER_WAVEFRONT) {
    snprintf(msg, sizeof msg, "%s: the wavefront mode renders volume-only worlds", fn);
    return set_error(GBV_ERROR_UNSUPPORTED, msg);
  }
  if ((s->d_depth || s->d_prim_id || s->d_inst_id || s->d_obj_id) && lc.mode == GBV_RENDER_WAVEFRONT) {
    snprintf(msg, sizeof msg, "%s: the wavefront mode writes no auxiliary channels", fn);
    return set_error(GBV_ERROR_UNSUPPORTED, msg);
  }
  if (spp == 0) return GBV_OK;
  gbv_status st = fill_params(s, p);
  if (st != GBV_OK) return st;
  p.W = width;
  p.H = height;
  p.accum = reinterpret_cast<float4 *>(d_accum);
  p.accumIdStart = accum_id_start;
  p.spp = spp;
  p.counters = d_counters;
  p.capFlag = d_cap_flag;
  p.rank = rank;
  p.numRanks = num_ranks;
  if (warp_tile_count(p) == 0) return GBV_OK;  // a rank that owns no tile
  if (warp_tile_count(p) >= (1ll << 31) - (1ll << 24)) {
    snprintf(msg, sizeof msg, "%s: more 8x4-pixel tiles than the 32-bit tile counter holds", fn);
    return set_error(GBV_ERROR_INVALID_ARGUMENT, msg);
  }
  cudaStream_t cs = (cudaStream_t)stream;
  if (s->layout == GBV_LAYOUT_LINEAR) return render_launch_linear(p, cs, lc);
  if (s->layout == GBV_LAYOUT_NANOVDB) return render_launch_nvdb(p, cs, lc);
  if (s->layout != GBV_LAYOUT_BRICK_CORNERS) {
    snprintf(msg, sizeof msg, "%s: unknown layout", fn);
    return set_error(GBV_ERROR_UNSUPPORTED, msg);
  }
  switch (s->format) {
    case GBV_VOXEL_F32: return render_launch_f32(p, cs, lc);
    case GBV_VOXEL_F16: return render_launch_f16(p, cs, lc);
    case GBV_VOXEL_BF16: return render_launch_bf16(p, cs, lc);
    case GBV_VOXEL_U8_SCALED: return render_launch_u8(p, cs, lc);
  }
  snprintf(msg, sizeof msg, "%s: unknown voxel format", fn);
  return set_error(GBV_ERROR_UNSUPPORTED, msg);
}

// gbv_render without event counting whose loop-cap events store 1 in
// *d_cap_flag (the bn* frame path: frame statistics only when asked for).
gbv_status render_cap_flagged(const gbv_scene *s, float *d_accum, int width, int height, int accum_id_start,
                              int spp, int *d_cap_flag, void *stream) {
  return render_frame("bnRender", s, d_accum, width, height, accum_id_start, spp, 0, 1, nullptr, stream,
                      d_cap_flag);
}

}  // namespace gbv

extern "C" gbv_status gbv_render(const gbv_scene *s, float *d_accum, int width, int height, int accum_id_start,
                                 int spp, unsigned long long *d_counters, void *stream) {
  return render_frame("gbv_render", s, d_accum, width, height, accum_id_start, spp, 0, 1, d_counters, stream);
}

extern "C" gbv_status gbv_render_ex(const gbv_scene *s, float *d_accum, int width, int height, int accum_id_start,
                                    int spp, unsigned long long *d_counters, const gbv_render_config *config,
                                    void *stream) {
  return render_frame("gbv_render_ex", s, d_accum, width, height, accum_id_start, spp, 0, 1, d_counters, stream,
                      nullptr, config);
}

extern "C" gbv_status gbv_render_tiles(const gbv_scene *s, float *d_accum, int width, int height,
                                       int accum_id_start, int spp, int rank, int num_ranks,
                                       unsigned long long *d_counters, void *stream) {
  return render_frame("gbv_render_tiles", s, d_accum, width, height, accum_id_start, spp, rank, num_ranks,
                      d_counters, stream);
}

extern "C" gbv_status gbv_tile_partition(int width, int height, int rank, int num_ranks, int *num_tiles,
                                         int *tile_lower) {
  if (width <= 0 || height <= 0 || num_ranks < 1 || rank < 0 || rank >= num_ranks || !num_tiles)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_tile_partition: bad size, rank or null count");
  const long long n = owned_ref_tiles(width, height, rank, num_ranks);
  if (n > (1ll << 31) - 1) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_tile_partition: too many tiles");
  *num_tiles = (int)n;
  if (tile_lower) {
    const long long tilesX = ((long long)width + kRefTile - 1) / kRefTile;
    for (long long k = 0; k < n; k++) {
      const long long id = (long long)rank + k * num_ranks;
      tile_lower[2 * k] = (int)(id % tilesX) * kRefTile;
      tile_lower[2 * k + 1] = (int)(id / tilesX) * kRefTile;
    }
  }
  return GBV_OK;
}

// ===========================================================================
// gbv_render_noalloc: the same frame render with no device allocation.
//
// Some callers cannot let a library allocate device memory while they
// render: an application that hands out all HBM from its own pre-sized pool
// and requires libraries to work inside the buffers it passes them, or a
// real-time viewer that forbids allocation and free calls on its frame
// path (gbv_render takes its one scratch word from cudaMallocAsync and
// returns it with cudaFreeAsync, which draw on the device's memory pool).
// This entry point takes that scratch word from a file-scope device array
// instead.
// ===========================================================================
namespace gbv {

// The persistent kernel's only scratch: the tile-pool counter (one 32-bit
// word).  Every GPU that loads this library holds this array until the
// process exits.  All calls share it and it keeps the last call's value, so
// each call clears it first; calls that overlap on the GPU (for example on
// two streams) race on it.
static __device__ __align__(256) int g_noalloc_tile_pool[1];
constexpr long long kNoAllocMaxTiles = 1ll << 30;

// Device address of the scratch on the current device.  Host code may not
// use the array's name as a device address, so every call looks the address
// up (cudaGetSymbolAddress allocates nothing); a device reset between calls,
// which reloads this library's device code at possibly new addresses, is
// therefore harmless.  The first lookup on a device (or after a reset) may
// load the device code there, which is why the first call on a device
// belongs before any stream capture.
static gbv_status noalloc_scratch(int **out) {
  void *ptr = nullptr;
  gbv_status st = check_cuda(cudaGetSymbolAddress(&ptr, g_noalloc_tile_pool), "gbv_render_noalloc: cudaGetSymbolAddress");
  if (st != GBV_OK) return st;
  *out = static_cast<int *>(ptr);
  return GBV_OK;
}


}  // namespace gbv

extern "C" gbv_status gbv_render_noalloc(const gbv_scene *s, float *d_accum, int width, int height,
                                         int accum_id_start, int spp, unsigned long long *d_counters,
                                         void *stream) {
  if (!s || !d_accum || width <= 0 || height <= 0 || spp < 0 || accum_id_start < 0)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_render_noalloc: null pointer or non-positive size");
  // the scratch is one 32-bit counter of 8x4-pixel tiles; every warp may take
  // one tile past the end, so the frame's tiles must leave room for them
  const long long tiles = (((long long)width + 7) / 8) * (((long long)height + 3) / 4);
  if (tiles > kNoAllocMaxTiles)
    return set_error(GBV_ERROR_INVALID_ARGUMENT,
                     "gbv_render_noalloc: frame exceeds the 2^30 tiles of 8x4 pixels its 32-bit tile counter holds");
  if (!scene_complete(s))
    return set_error(GBV_ERROR_INVALID_ARGUMENT,
                     "gbv_render_noalloc: scene lacks voxels, majorants or a transfer function");
  if (s->layout == GBV_LAYOUT_LINEAR && s->format != GBV_VOXEL_F32)
    return set_error(GBV_ERROR_UNSUPPORTED, "gbv_render_noalloc: the linear layout holds FP32 voxels only");
  if (s->format == GBV_VOXEL_U8_SCALED && !s->d_scale_offset)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_render_noalloc: U8 voxels need the brick scale/offset table");
  if (spp == 0) return GBV_OK;
  int *pool = nullptr;
  gbv_status st = noalloc_scratch(&pool);
  if (st != GBV_OK) return st;
  RenderParams p;
  st = fill_params(s, p);
  if (st != GBV_OK) return st;
  p.W = width;
  p.H = height;
  p.accum = reinterpret_cast<float4 *>(d_accum);
  p.accumIdStart = accum_id_start;
  p.spp = spp;
  p.counters = d_counters;
  cudaStream_t cs = (cudaStream_t)stream;
  if (s->layout == GBV_LAYOUT_LINEAR) return render_launch_noalloc_linear(p, cs, pool);
  if (s->layout == GBV_LAYOUT_NANOVDB) return render_launch_noalloc_nvdb(p, cs, pool);
  if (s->layout != GBV_LAYOUT_BRICK_CORNERS)
    return set_error(GBV_ERROR_UNSUPPORTED, "gbv_render_noalloc: unknown layout");
  switch (s->format) {
    case GBV_VOXEL_F32: return render_launch_noalloc_f32(p, cs, pool);
    case GBV_VOXEL_F16: return render_launch_noalloc_f16(p, cs, pool);
    case GBV_VOXEL_BF16: return render_launch_noalloc_bf16(p, cs, pool);
    case GBV_VOXEL_U8_SCALED: return render_launch_noalloc_u8(p, cs, pool);
  }
  return set_error(GBV_ERROR_UNSUPPORTED, "gbv_render_noalloc: unknown voxel format");
}

// ===========================================================================
// Batched rendering: many independent scenes of uneven sizes in one
// persistent launch.  All items share a voxel format and layout.
// ===========================================================================


extern "C" gbv_status gbv_batch_create(const gbv_scene *scenes, float *const *d_accums, const int *widths,
                                       const int *heights, int count, gbv_batch **out) {
  if (!scenes || !d_accums || !widths || !heights || count <= 0 || !out)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_batch_create: bad argument");
  *out = nullptr;
  std::vector<RenderParams> items(count);
  std::vector<long long> starts(count + 1, 0);
  for (int i = 0; i < count; i++) {
    const gbv_scene *s = scenes + i;
    if (!s->d_voxels || !s->d_majorants || !s->d_tf || s->tf_n < 2 ||
        (s->layout != GBV_LAYOUT_NANOVDB && s->cells_per_mc <= 0) || !d_accums[i] ||
        widths[i] <= 0 || heights[i] <= 0)
      return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_batch_create: an item lacks data or has an empty frame");
    if (s->format != scenes[0].format || s->layout != scenes[0].layout)
      return set_error(GBV_ERROR_UNSUPPORTED, "gbv_batch_create: items must share voxel format and layout");
    if (s->iso) return set_error(GBV_ERROR_UNSUPPORTED, "gbv_batch_create: batches render volume-only worlds");
    if (s->d_depth || s->d_prim_id || s->d_inst_id || s->d_obj_id)
      return set_error(GBV_ERROR_UNSUPPORTED, "gbv_batch_create: batches write no auxiliary channels");
    if (s->layout == GBV_LAYOUT_LINEAR && s->format != GBV_VOXEL_F32)
      return set_error(GBV_ERROR_UNSUPPORTED, "gbv_batch_create: the linear layout holds FP32 voxels only");
    if (s->format == GBV_VOXEL_U8_SCALED && !s->d_scale_offset)
      return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_batch_create: U8 voxels need the brick scale table");
    gbv_status st = fill_params(s, items[i]);
    if (st != GBV_OK) return st;
    RenderParams &p = items[i];
    p.W = widths[i];
    p.H = heights[i];
    p.accum = reinterpret_cast<float4 *>(d_accums[i]);
    p.maskWords = 0;
    p.cdfYOff = p.pivOff = p.rowOff = -1;
    p.pivPerRow = 0;
    starts[i + 1] = starts[i] + (((long long)p.W + 7) / 8) * (((long long)p.H + 3) / 4);
  }
  if (starts[count] >= (1ll << 31) - (1ll << 20))
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_batch_create: more tiles than the 32-bit tile counter holds");
  gbv_batch *b = new gbv_batch();
  b->count = count;
  b->format = scenes[0].format;
  b->layout = scenes[0].layout;
  b->totalTiles = starts[count];
  b->occ = 4;
  b->threshold = kThresholdDefault;
  b->skip = kSkipDefault;
  gbv_status st = check_cuda(cudaGetDevice(&b->device), "gbv_batch_create: cudaGetDevice");
  if (st == GBV_OK) st = check_cuda(cudaMalloc((void **)&b->d_items, sizeof(RenderParams) * count), "gbv_batch_create");
  if (st == GBV_OK)
    st = check_cuda(cudaMalloc((void **)&b->d_tileStart, sizeof(long long) * (count + 1)), "gbv_batch_create");
  if (st == GBV_OK) st = check_cuda(cudaMalloc((void **)&b->d_pool, sizeof(int)), "gbv_batch_create");
  if (st == GBV_OK)
    st = check_cuda(cudaMemcpy(b->d_items, items.data(), sizeof(RenderParams) * count, cudaMemcpyHostToDevice),
                    "gbv_batch_create: upload");
  if (st == GBV_OK)
    st = check_cuda(cudaMemcpy(b->d_tileStart, starts.data(), sizeof(long long) * (count + 1),
                               cudaMemcpyHostToDevice),
                    "gbv_batch_create: upload");
  if (st != GBV_OK) {
    gbv_batch_destroy(b);
    return st;
  }
  *out = b;
  return GBV_OK;
}

extern "C" gbv_status gbv_batch_set_launch(gbv_batch *b, int blocks_per_sm, int threshold_pct, int skip_cells) {
  if (!b || blocks_per_sm < 4 || blocks_per_sm > 6 || threshold_pct < 1 || threshold_pct > 100 || skip_cells < 1)
    return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_batch_set_launch: blocks 4..6, threshold 1..100, skip >= 1");
  b->occ = blocks_per_sm;
  b->threshold = threshold_pct;
  b->skip = skip_cells;
  return GBV_OK;
}

extern "C" gbv_status gbv_batch_render(gbv_batch *b, int accum_id_start, int spp, unsigned long long *d_counters,
                                       void *stream) {
  if (!b || spp < 0 || accum_id_start < 0) return set_error(GBV_ERROR_INVALID_ARGUMENT, "gbv_batch_render: bad argument");
  if (spp == 0) return GBV_OK;
  RenderParams L;
  memset(&L, 0, sizeof(L));
  L.accumIdStart = accum_id_start;
  L.spp = spp;
  L.counters = d_counters;
  L.skip = b->skip;
  L.threshold = b->threshold;
  L.maskWords = 0;
  L.cdfYOff = L.pivOff = L.rowOff = -1;
  L.profile = 0;
  cudaStream_t cs = (cudaStream_t)stream;
  if (b->layout == GBV_LAYOUT_LINEAR) return batch_launch_linear(b, L, cs);
  if (b->layout == GBV_LAYOUT_NANOVDB) return batch_launch_nvdb(b, L, cs);
  switch (b->format) {
    case GBV_VOXEL_F32: return batch_launch_f32(b, L, cs);
    case GBV_VOXEL_F16: return batch_launch_f16(b, L, cs);
    case GBV_VOXEL_BF16: return batch_launch_bf16(b, L, cs);
    case GBV_VOXEL_U8_SCALED: return batch_launch_u8(b, L, cs);
  }
  return set_error(GBV_ERROR_UNSUPPORTED, "gbv_batch_render: unknown voxel format");
}

extern "C" gbv_status gbv_batch_destroy(gbv_batch *b) {
  if (!b) return GBV_OK;
  if (b->d_items) cudaFree(b->d_items);
  if (b->d_tileStart) cudaFree(b->d_tileStart);
  if (b->d_pool) cudaFree(b->d_pool);
  delete b;
  return GBV_OK;
}
