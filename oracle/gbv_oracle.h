/* gbv_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * C interface of the CPU oracle: a restatement of the reference renderer's
 * embree (CPU) backend for the structured-volume path (Barney 1.1.8).  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * this library.  It is the checker, never the product.
 *
 * Pinned by the reference's own code: the reference ships no golden vectors
 * for this path and cannot be built as a whole here, but its sources for the
 * path compile unchanged against a restated owl and a stubbed embree API
 * (oracle/refpin, `make ref`); the RNG, fastLog, float/half, the transfer
 * function, the field sampler, sampleAndMap, the per-ray volume isProg, the
 * iso-surface isProg with a matte material, the Lambertian BSDF, the
 * shading step bounce() of both scattering builds, the env-map importance
 * tables, the sRGB packing and the NanoVDB field code agree with this oracle
 * bit for bit (tests/test_oracle_refpin.py).  Ray generation is pinned by
 * known-answer tests and a second, pure-Python restatement of the scalar
 * kernels (tests/golden/make_golden.py).
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_scene {
  /* structured field (StructuredData: "dims", "gridOrigin", "gridSpacing") */
  const float *scalars;      /* x-fastest, dims[0]*dims[1]*dims[2] */
  int   dims[3];
  float origin[3];
  float spacing[3];
  /* macrocells */
  int   cells_per_mc;        /* 8 in the reference; 16 for the 512^3 scene */
  const float *majorants;    /* optional; if null the oracle builds its own */
  /* transfer function (TransferFunction::set) */
  const float *tf;           /* n x RGBA */
  int   tf_n;
  float domain[2];
  float base_density;        /* "densityAt1" */
  /* volume params of the multi-scatter build (Volume.h:158-159) */
  float anisotropy;
  float scattering_albedo;
  /* perspective camera parameters (Camera.cu PerspectiveCamera) */
  float cam_pos[3], cam_dir[3], cam_up[3];
  float fovy;
  /* directional lights (DirLight), at most 4 */
  int   num_dir_lights;
  float dir_light_dir[4][3];
  float dir_light_color[4][3];
  float dir_light_radiance[4];
  /* env-map light (EnvMapLight); env_texels == 0 means "no env map" */
  const float *env_texels;   /* RGBA float, env_dims[0] x env_dims[1] */
  int   env_dims[2];
  int   env_addr[2];         /* 0 wrap, 1 clamp, 2 border, 3 mirror */
  float env_dir[3], env_up[3];
  float env_scale;
  /* renderer */
  float bg_color[4];
  float ambient_radiance;
  int   multi_scatter;       /* 0: default build (SCI_VIS_MODE), 1: multi-scatter build */
  int   volume_multi_scatter;
  int   max_volume_bounces;
  /* frame */
  int   width, height;
  /* 1: sample the field as the library's U8 brick store holds it -- per
     8^3-cell scale brick, u8 = round(255 (v - min) / (max - min)) over its
     9^3 voxels, dequantized as min + (max - min)/255 * u8 per cell corner --
     and bound macrocells by the dequantized corners (the library's own
     storage form; the reference has none) */
  int   u8_scaled;
  /* 0: the path's sines, cosines, arc cosines and arc tangents are libm's
     (sinf, cosf, acosf, atan2f), as in the reference's CPU backend.  1: they
     use the bounded methods of the library's device code
     (orc_bounded_sincos, orc_bounded_angles): the scattering azimuth, the
     env-map CDF rows, the env light sample's angles and pdf, and the env
     lookups' theta and phi.  Then nothing else differs and frames with
     multiple scattering and an env map are comparable bit for bit. */
  int   bounded_math;
  /* a NanoVDB float grid (format 32) in host memory; when set it is the
     field (scalars, dims, origin, spacing and cells_per_mc are not used):
     the reference's NanoVDB field (barney/volume/NanoVDB.{h,cu}) */
  const unsigned char *nanovdb;
  unsigned long long nanovdb_bytes;
  /* an iso-surface geometry over the same field (IsoSurface,
     barney/geometry/IsoSurface.{h,cpp}) with a matte material (AnariMatte,
     barney/material/AnariMatte.h); iso_enabled = 0: none.  The world's
     instances are intersected in ascending order of their RTC instance
     index (ModelSlot::flattenInstancesForDevice appends a group's
     user-geometry group before its volumes), and each one's hash(instance,
     0, 0) seeds its random stream. */
  int   iso_enabled;
  float iso_value;
  float iso_color[4];        /* AnariMatte "color" (set3f: alpha 1) */
  float iso_opacity;         /* AnariMatte "opacity" */
  int   iso_instance;
  int   volume_instance;
  int   no_volume;           /* 1: the world holds the iso-surface only */
  /* the geometries' "userID" (the object ID of their hits) and auxiliary
     frame channels (host memory, width*height each, or 0): the reference's
     aux tiles written at a pixel's primary-ray shading (shadeRays.cu:
     1003-1023) from its closest hit's IDs (MCAccelerator.h:552-565,
     685-700) */
  int   volume_user_id, iso_user_id;
  float *aux_depth;
  int   *aux_prim_id, *aux_inst_id, *aux_obj_id;
} orc_scene;

typedef struct orc_stats {
  uint64_t density_samples;  /* sampleAndMap evaluations */
  uint64_t mc_visits;        /* DDA cells with a non-zero majorant */
  uint64_t rays;             /* traced rays */
} orc_stats;

/* --- scalar kernels, exposed for known-answer tests --- */
void  orc_rng_sequence(uint32_t a, uint32_t b, int n, float *out);
void  orc_rng_from_seed(uint64_t seed_state, uint64_t hash, int use_u64, int n,
                        float *out, uint64_t *new_seed_state);
uint64_t orc_rng_seed_state(uint32_t a, uint32_t b);  /* RNGSeed::seed(a, b) from the default state */
uint64_t orc_hash3(uint32_t a, uint32_t b, uint32_t c);
float orc_fast_log(float f);
uint16_t orc_float_to_half(float f);
float orc_half_to_float(uint16_t h);
void  orc_sample_points(const orc_scene *s, const float *P, int n, float *out);
void  orc_tf_map(const orc_scene *s, const float *scalars, int n, float *rgba);

/* --- macrocell build (StructuredData_computeMCs + mapMCs) --- */
/* macrocell grid of the scene's field: dims, and for NanoVDB fields the
   world bounds (lower xyz, upper xyz) the grid spans */
void  orc_scene_mc_grid(const orc_scene *s, int mc_dims[3], float world[6]);
void  orc_mc_dims(const int dims[3], int cells_per_mc, int mc_dims[3]);
void  orc_mc_ranges(const float *scalars, const int dims[3], int cells_per_mc,
                    float *ranges /* 2 per MC */);
/* sine and cosine of each x[i] (x in [-pi/4, 2 pi + pi/4]), and arc cosine
   of x[i] (x in [-1, 1]) with arc tangent of y[i]/x[i], by the bounded
   methods of orc_scene.bounded_math */
void orc_bounded_sincos(const float *x, long long n, float *sn, float *cs);
void orc_bounded_angles(const float *y, const float *x, long long n, float *acos_x, float *atan2_yx);

/* ranges of the scene's field in its storage form (orc_scene.u8_scaled) */
void  orc_scene_mc_ranges(const orc_scene *s, float *ranges /* 2 per MC */);
void  orc_majorants(const float *ranges, int num_mc, const float *tf, int tf_n,
                    float lo, float hi, float base_density, float *out);

/* --- one ray through the volume (MCVolumeAccel::isProg) --- */
int   orc_trace_ray(const orc_scene *s, const float org[3], const float dir[3],
                    float tmax, uint64_t *seed_state, float *t_hit, float rgb[3]);

/* --- iso-surface ray query (MCIsoSurfaceAccel::isProg); ranges: per-MC
       (min, max) or null; out: t, P[3], N[3]; returns 1 on a hit --- */
int   orc_iso_intersect(const orc_scene *s, const float *ranges, float iso,
                        const float org[3], const float dir[3], float tmax,
                        float out[7]);

/* The iso-surface isProg with a constant-color AnariMatte material for one
   ray (instance `inst`, geometry 0, primitive 0): 1 on a hit with t, P, the
   normal's halfs and the Lambertian's albedo (xyz) and alpha (w); the ray's
   RNG seed state in and out. */
int   orc_iso_hit(const orc_scene *s, const float *ranges, float iso, const float color[4],
                  float opacity, int inst, const float org[3], const float dir[3], float tmax,
                  uint64_t *seed_state, float *t_hit, float P[3], uint16_t N[3], float albedo[4]);
/* The AnariMatte Lambertian at normal Ng seen from wo: eval value[3], eval
   pdf, pdf toward wi, then a scatter from Random2(a, b): dir[3], pdf, f_r[3]. */
void  orc_lambertian(const float color[4], const float Ng[3], const float wo[3], const float wi[3],
                     uint32_t a, uint32_t b, float out[12]);

/* --- one shading step, bounce() (shadeRays.cu:477-878), on a given world
       and path: the records the reference pin (ref_bounce) shares --- */
typedef struct orc_shade_world {
  int   num_dir_lights;            /* DirLight::DD: unit direction, colour, radiance */
  float dir_light_dir[4][3];
  float dir_light_color[4][3];
  float dir_light_radiance[4];
  const float *env_texels;         /* RGBA float env map, or 0: none */
  int   env_dims[2];
  int   env_addr[2];
  float env_to_world[9], env_to_local[9];  /* EnvMapLight::DD toWorld/toLocal: columns vx, vy, vz */
  float env_scale;
  const float *env_cdf_y, *env_cdf_x;      /* its importance tables */
  float ambient_radiance;
  int   volume_multi_scatter, max_volume_bounces;  /* multi-scatter build */
} orc_shade_world;

typedef struct orc_shade_path {
  float org[3], dir[3], tmax;      /* on a hit: tmax = the hit's t */
  uint64_t seed;                   /* ray.rngSeed */
  int   hit;                       /* 0 none; 1 volume (Phase of rgb); 2 surface (AnariMatte Lambertian) */
  float P[3];
  float rgb[3];                    /* volume hit: the sampled colour */
  float g, scattering_albedo;      /* volume hit, multi-scatter build */
  float N[3];                      /* surface hit: unit normal (stored in half precision) */
  float color[4], opacity;         /* surface hit: the matte material */
  int   shadow;                    /* isShadowRay */
  uint16_t tp[3];                  /* PathState throughput (halfs) */
  uint16_t pad;
  float mis;
  int   diffuse_bounces, volume_bounces;
  float miss_color[4];
} orc_shade_path;

/* bounce() of the default (multi = 0) or the multi-scatter build (multi = 1)
   at path depth `depth`: updates *ray (dead: tmax = -1), fills *shadow
   (none: tmax = -1) and fragment[3]; libm sines and cosines. */
void  orc_bounce(const orc_shade_world *w, int multi, int depth, orc_shade_path *ray,
                 orc_shade_path *shadow, float fragment[3]);

/* PerspectiveCamera::commit: dir_00, dir_du, dir_dv, lens_00 (12 floats) */
void  orc_camera_commit(const float pos[3], const float dir[3], const float up[3], float fovy,
                        float out[12]);
/* _generateRays for pass accum_id of a W x H frame with background bg (w < 0:
   the gradient): per pixel, row-major, org[3], dir[3], tMax, missColor[4]
   and the ray's seed state; returns the count of pixels whose path state is
   not (throughput 1, misWeight 0) */
int   orc_generate(const float pos[3], const float dir[3], const float up[3], float fovy, int W, int H,
                   int accum_id, const float bg[4], float *out, uint64_t *seeds);

/* --- full render: bnRender's generate/trace/shade loop for `spp`
       consecutive accumulation passes starting at accum_id_start.
       accum: width*height RGBA, row-major, y=0 the bottom row.
       use_double: evaluate everything downstream of the RNG in double.
       rows: render only rows [row0, row1) (row1<=0 means all). --- */
void  orc_render(const orc_scene *s, float *accum, int accum_id_start, int spp,
                 int use_double, int nthreads, int row0, int row1,
                 orc_stats *stats);

/* --- frame-buffer read (linearizeColorAndNormalKernel); format:
       0 float4, 1 RGBA8, 2 sRGB RGBA8 --- */
void  orc_tonemap(const float *accum, int width, int height, int accum_id,
                  int format, void *out);

/* --- env map importance tables (EnvMap.cu computeCDFs) --- */
void  orc_env_cdfs(const float *texels, const int dims[2], const int addr[2],
                   float *cdf_y, float *cdf_x);

/* --- fixed-step emission-absorption (project-defined form) --- */
typedef struct orc_ea_view {
  float pos[3], dir[3], up[3];
  float fovy;
  int   width, height;
} orc_ea_view;

void  orc_ea_render(const orc_scene *s, const orc_ea_view *views, int num_views,
                    float step, int use_double, int nthreads, float *images);
/* gradient of L = sum(w * image) with respect to voxels and TF entries, in
   FP64; d_images holds w (dL/dimage). */
void  orc_ea_backward(const orc_scene *s, const orc_ea_view *views,
                      int num_views, float step, const float *d_images,
                      int nthreads, double *d_scalars, double *d_tf);

#ifdef __cplusplus
}
#endif
