/* gbvol.h -- low-level C-ABI of the GB300 structured-volume path.
 *
 * Plain pointers and sizes only.  Pointers named d_* are device (HBM)
 * pointers on the current CUDA device; `stream` is a cudaStream_t passed as
 * void* (0 = legacy default stream).  Every entry point returns a gbv_status
 * and never throws; gbv_last_error() gives the message of the last failure on
 * the calling thread.
 *
 * These entry points are what the reference's internal volume seam would bind
 * for this path (one per reference kernel / launcher); the barney-compatible
 * bn* surface in barney_gb300.h is built on top of them.
 */
#ifndef GBVOL_H
#define GBVOL_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gbv_status {
  GBV_OK = 0,
  GBV_ERROR_INVALID_ARGUMENT = 1,
  GBV_ERROR_CUDA = 2,
  GBV_ERROR_OUT_OF_MEMORY = 3,
  /* a device loop hit its iteration cap; results of that launch are partial */
  GBV_ERROR_LIMIT = 4,
  GBV_ERROR_UNSUPPORTED = 5
} gbv_status;

/* voxel storage formats */
enum {
  GBV_VOXEL_F32 = 0,
  GBV_VOXEL_F16 = 1,
  GBV_VOXEL_BF16 = 2,
  GBV_VOXEL_U8_SCALED = 3 /* uint8 with a float (scale, offset) per 8^3 cells */
};
/* voxel layouts */
enum {
  GBV_LAYOUT_LINEAR = 0,        /* x-fastest scalars, FP32 only (the reference's texel array) */
  GBV_LAYOUT_BRICK_CORNERS = 1, /* bricks of cells (8^3 unless shaped); each cell stores its 8 corner voxels */
  GBV_LAYOUT_NANOVDB = 2        /* a NanoVDB float grid buffer (gbv_nanovdb_parse) */
};
/* frame-buffer read formats (BNDataType subset) */
enum { GBV_FB_FLOAT4 = 0, GBV_FB_RGBA8 = 1, GBV_FB_RGBA8_SRGB = 2 };
/* texture address modes (BNTextureAddressMode order) */
enum { GBV_ADDR_WRAP = 0, GBV_ADDR_CLAMP = 1, GBV_ADDR_BORDER = 2, GBV_ADDR_MIRROR = 3 };

const char *gbv_last_error(void);
int gbv_version(void);

/* ------------------------------------------------------------------------
 * Macrocells.
 * ------------------------------------------------------------------------ */

/* Macrocell grid dimensions: ceil((dims-1)/cells_per_mc) per axis.
   Replaces StructuredData::buildMCs's mcDims computation
   (barney/volume/StructuredData.cu:73). */
gbv_status gbv_mc_dims(const int dims[3], int cells_per_mc, int mc_dims[3]);

/* Per-macrocell scalar range (min, max) over the (cells_per_mc+1)^3 voxel
   footprint of each macrocell, from an FP32 x-fastest scalar array.
   d_ranges: 2 floats per macrocell, x-fastest.
   Replaces StructuredData_computeMCs (barney/volume/StructuredData.cu:29-61)
   and MCGrid::clearCells (barney/volume/MCGrid.cu:63-91). */
gbv_status gbv_build_mc_ranges(const float *d_scalars, const int dims[3],
                               int cells_per_mc, float *d_ranges, void *stream);

/* Per-macrocell scalar range taken from a brick-corner store (any format):
   min/max of the dequantized corner voxels of the macrocell's cells, i.e.
   the values its trilinear samples can interpolate.  For FP32 stores this
   equals gbv_build_mc_ranges; for FP16/BF16/U8 stores it bounds the stored
   (rounded) values, which the FP32 source may not.
   Replaces StructuredData_computeMCs (barney/volume/StructuredData.cu:29-61)
   for quantized voxels. */
gbv_status gbv_build_mc_ranges_from_store(const void *d_voxels,
                                          const float *d_scale_offset,
                                          int format, const int dims[3],
                                          int cells_per_mc, float *d_ranges,
                                          void *stream);

/* Majorant of each macrocell = the transfer function's maximum opacity over
   its range times base_density.  Bit-identical to the reference's FP32.
   d_tf: tf_n RGBA float entries.
   Replaces mapMCs / TransferFunction::DD::majorant
   (barney/volume/MCGrid.cu:94-116, barney/volume/TransferFunction.h:91-116). */
gbv_status gbv_map_majorants(const float *d_ranges, int num_mc,
                             const float *d_tf, int tf_n, float domain_lo,
                             float domain_hi, float base_density,
                             float *d_majorants, void *stream);

/* ------------------------------------------------------------------------
 * Voxel storage.
 * ------------------------------------------------------------------------ */

/* Bytes needed for the brick-corner store of a volume (voxels; for
   GBV_VOXEL_U8_SCALED also *scale_offset_bytes for the scale table). */
gbv_status gbv_brick_store_bytes(const int dims[3], int format,
                                 size_t *voxel_bytes, size_t *scale_offset_bytes);

/* Re-lays an FP32 x-fastest volume as 8^3-cell bricks in `format`; each
   cell stores its 8 corner voxels (one vector load per trilinear sample).
   U8: one float (scale, offset) per 8^3 cells, u8 = round(255 (v - min) /
   (max - min)) over their 9^3 voxels.
   Replaces the texel upload of StructuredData::setObject("textureData")
   (barney/volume/StructuredData.cu:154-173, rtcore/cudaCommon/TextureData.cu:59-75). */
gbv_status gbv_build_brick_store(const float *d_scalars, const int dims[3],
                                 int format, void *d_voxels,
                                 float *d_scale_offset, void *stream);

/* The same with a chosen brick shape: brick_log2[i] = log2 of the brick
   edge in cells along axis i, each 1..6 (0 or a null pointer: 3) and at most
   15 in sum.  The shape changes only the order of cells in HBM (locality),
   never a sampled value: U8 scales stay per 8^3 cells.  A scene rendering
   such a store sets gbv_scene.brick_log2 to the same shape.  No counterpart
   in the reference (its texels are a cudaArray or an x-fastest array). */
gbv_status gbv_brick_store_bytes_shaped(const int dims[3], int format,
                                        const int brick_log2[3],
                                        size_t *voxel_bytes,
                                        size_t *scale_offset_bytes);
gbv_status gbv_build_brick_store_shaped(const float *d_scalars, const int dims[3],
                                        int format, const int brick_log2[3],
                                        void *d_voxels, float *d_scale_offset,
                                        void *stream);
gbv_status gbv_build_mc_ranges_from_store_shaped(const void *d_voxels,
                                                 const float *d_scale_offset,
                                                 int format, const int dims[3],
                                                 const int brick_log2[3],
                                                 int cells_per_mc, float *d_ranges,
                                                 void *stream);

/* Normalised 8- or 16-bit unsigned texels (bits = 8 or 16) to FP32 scalars
   v / 255 or v / 65535, on the device.  Replaces the normalised-float texture
   reads of integer texel formats (rtcore/cudaCommon/TextureData.cu:34-39,
   rtcore/embree/Texture.cpp:216-225) for BN_UFIXED8 / BN_UFIXED16 fields. */
gbv_status gbv_normalize_texels(const void *d_texels, int bits, long long n,
                                float *d_scalars, void *stream);

/* ------------------------------------------------------------------------
 * NanoVDB fields: one NanoVDB grid of value type Float (format version 32,
 * the buffer nanovdb::GridHandle holds), resident on the device as is.
 * ------------------------------------------------------------------------ */
typedef struct gbv_nanovdb_info {
  /* from the grid buffer */
  unsigned long long bytes;      /* the grid's size in bytes */
  long long root_offset;         /* byte offset of the root node */
  unsigned int root_tiles;       /* root table size */
  float background;              /* value of unset voxels */
  float inv_map[9], map_offset[3]; /* world -> index: inv_map x (P - map_offset), single precision */
  int index_lo[3], index_hi[3];  /* index bbox of the active values (inclusive) */
  float world_lo[3], world_hi[3];/* world bbox (single precision) */
  double voxel_size[3];
  /* macrocells: ceil(index bbox size / 16) per axis (NanoVDBData::buildMCs) */
  int mc_dims[3];
  /* nanovdb::GridType of the values: 1 Float, 13 Fp4, 14 Fp8, 15 Fp16, 16 FpN */
  int grid_type;
} gbv_nanovdb_info;

/* Parses and checks a NanoVDB grid held in HOST memory (h_grid, `bytes`
   long): magic number, format version 32, a value type the reference's
   NanoVDB field reads (Float, Fp4, Fp8, Fp16, FpN; barney/volume/NanoVDB.h:
   23-28), the size the header states, and every node of the tree inside the
   buffer on 32-byte alignment, FpN leaves with bit widths of at most 16 (the
   device follows the child offsets unchecked, so a grid is parsed before it
   is used on the device).  Replaces
   NanoVDBData::commit (barney/volume/NanoVDB.cu:193-232). */
gbv_status gbv_nanovdb_parse(const void *h_grid, size_t bytes, gbv_nanovdb_info *info);

/* Per-macrocell scalar range (min, max) of a NanoVDB grid on the device:
   macrocell m covers the index box lo + (m*size)/mc .. lo + ((m+1)*size)/mc
   + 1, both ends inclusive, and takes every value the grid returns there
   (active, inactive, tile or background).  d_ranges: 2 floats per
   macrocell, x-fastest, info->mc_dims macrocells.  Replaces
   NanoVDBData_computeMCs (barney/volume/NanoVDB.cu:28-60). */
gbv_status gbv_nanovdb_mc_ranges(const void *d_grid, const gbv_nanovdb_info *info, float *d_ranges,
                                 void *stream);

/* The field's sampler at n world points (d_points: 3 floats each) into
   d_values: NanoVDBDataSampler::DD::sample (barney/volume/NanoVDB.h:100-129),
   the same function the renderer samples with. */
gbv_status gbv_nanovdb_sample(const void *d_grid, const gbv_nanovdb_info *info, const float *d_points,
                              long long n, float *d_values, void *stream);

/* ------------------------------------------------------------------------
 * Scene description for rendering (device pointers where marked d_).
 * ------------------------------------------------------------------------ */
/* An iso-surface of the scene's field with a matte material: the
   "iso_surface" geometry (IsoSurface, barney/geometry/IsoSurface.{h,cpp}:
   "isoValue") and the "matte" material (AnariMatte,
   barney/material/AnariMatte.{h,cpp}: "color", "opacity"), rendered as the
   reference's surface path does (MCIsoSurfaceAccel::isProg,
   barney/volume/MCAccelerator.h:338-567; the surface branch of
   barney/kernels/shadeRays.cu:541-878 with the material's Lambertian).  The
   world's instances are intersected in ascending order of their RTC
   instance index (ModelSlot::flattenInstancesForDevice,
   barney/ModelSlot.cpp:129-155, lists a group's user geometries before its
   volumes), each one's random stream seeded with hash(instance, 0, 0).
   The persistent mode of gbv_render/gbv_render_ex/gbv_render_tiles and
   gbv_render_noalloc render it; the wavefront mode and batches do not. */
typedef struct gbv_iso_surface {
  float iso_value;
  /* the field's macrocell scalar ranges, (lower, upper) per macrocell, as
     gbv_build_mc_ranges (or gbv_nanovdb_mc_ranges) writes them */
  const float *d_ranges;
  float color[4];         /* AnariMatte color, RGBA (a color set as 3 floats has alpha 1) */
  float opacity;          /* AnariMatte opacity */
  int instance;           /* RTC instance index of the geometry's group */
  int user_id;            /* the geometry's "userID": objID of its hits */
} gbv_iso_surface;

typedef struct gbv_scene {
  /* structured field */
  const void *d_voxels;          /* per layout/format */
  const float *d_scale_offset;   /* U8_SCALED only */
  int format, layout;
  int dims[3];
  float origin[3], spacing[3];
  /* macrocells (from gbv_map_majorants) */
  const float *d_majorants;
  int cells_per_mc;
  /* transfer function */
  const float *d_tf;
  int tf_n;
  float domain[2];
  float base_density;
  float anisotropy, scattering_albedo;
  /* perspective camera parameters */
  float cam_pos[3], cam_dir[3], cam_up[3];
  float fovy;
  /* directional lights (at most 4) */
  int num_dir_lights;
  float dir_light_dir[4][3];
  float dir_light_color[4][3];
  float dir_light_radiance[4];
  /* env-map light: d_env_texels == 0 means none */
  const float *d_env_texels;     /* RGBA float */
  const float *d_env_cdf_y;      /* env_dims[1] */
  const float *d_env_cdf_x;      /* env_dims[0]*env_dims[1] */
  int env_dims[2];
  int env_addr[2];
  float env_dir[3], env_up[3];
  float env_scale;
  /* renderer */
  float bg_color[4];
  float ambient_radiance;
  int multi_scatter;             /* 0 default build (single scatter), 1 multi-scatter build */
  int volume_multi_scatter;
  int max_volume_bounces;
  /* brick shape of a GBV_LAYOUT_BRICK_CORNERS store (as passed to
     gbv_build_brick_store_shaped; {0,0,0} = 8^3 cells) */
  int brick_log2[3];
  /* GBV_LAYOUT_NANOVDB: the parsed grid (host memory); d_voxels is the grid
     buffer on the device, d_majorants has nanovdb->mc_dims macrocells, and
     dims, origin, spacing and cells_per_mc are not used (the grid's own
     index bbox, world bbox and macrocells are) */
  const gbv_nanovdb_info *nanovdb;
  /* an iso-surface of the field (host memory), or 0.  With an iso-surface,
     d_majorants == 0 means the world holds no volume (d_tf is then not
     used either). */
  const gbv_iso_surface *iso;
  int volume_instance;   /* RTC instance index of the volume's group (0 without an iso-surface) */
  int volume_user_id;    /* the volume's "userID": objID of its hits */
  /* Auxiliary frame channels (device memory, width*height entries each, row
     by row; 0 = not wanted), written from each pixel's primary ray as the
     reference's shading step writes its aux tiles (barney/kernels/
     shadeRays.cu:1003-1023, the hit IDs of MCAccelerator.h:552-565,
     685-700): on pass 0 depth = the primary ray's tMax (its hit distance,
     or 1e30 on a miss) and the closest hit's primitive (0), instance (its
     RTC instance index) and object IDs (its userID), -1 on a miss; on
     later passes depth = min(depth, tMax) and the IDs stay.  Persistent
     mode only (gbv_render, gbv_render_ex, gbv_render_tiles,
     gbv_render_noalloc). */
  float *d_depth;
  int *d_prim_id, *d_inst_id, *d_obj_id;
} gbv_scene;

/* Counters written by gbv_render when d_counters != 0 (uint64 each):
   [0] density samples, [1] macrocells entered with a non-zero majorant,
   [2] rays traced, [3] loop-cap events, [4] macrocells crossed (all),
   [5..7] SM cycles spent starting traces, traversing and shading, summed
   over warps, [8] traversal iterations of warps and [9] tracing lanes
   summed over them, [10] shading passes of warps and [11] shaded lanes
   summed over them ([5..11] only when gbv_render_ex's config asks for a
   profile, else 0). */
enum { GBV_COUNTER_SAMPLES = 0, GBV_COUNTER_MC_VISITS = 1, GBV_COUNTER_RAYS = 2,
       GBV_COUNTER_CAPS = 3, GBV_COUNTER_CELLS = 4, GBV_COUNTER_CYCLES_START = 5,
       GBV_COUNTER_CYCLES_TRAVERSE = 6, GBV_COUNTER_CYCLES_SHADE = 7,
       GBV_COUNTER_TRAVERSE_ITERS = 8, GBV_COUNTER_TRAVERSE_LANES = 9,
       GBV_COUNTER_SHADE_PASSES = 10, GBV_COUNTER_SHADE_LANES = 11,
       GBV_NUM_COUNTERS = 12 };

/* Env-map importance tables (d_cdf_y: H floats, d_cdf_x: W*H floats) from
   RGBA float texels.  Replaces EnvMapLight::computeCDFs
   (barney/light/EnvMap.cu:61-137, 181-238). */
gbv_status gbv_env_build_cdfs(const float *d_texels, int width, int height,
                              const int addr[2], float *d_cdf_y, float *d_cdf_x,
                              void *stream);

/* Renders `spp` accumulation passes (accumIDs accum_id_start ..
   accum_id_start+spp-1) into d_accum (width*height RGBA float, row-major,
   row 0 the bottom row), accumulating as the reference does: the first pass
   of a fresh frame (accum_id_start == 0) overwrites.  d_counters: optional,
   GBV_NUM_COUNTERS uint64 (accumulated, not cleared).
   Replaces Context::renderTiles' generate/trace/shade loop
   (barney/Context.cpp:142-185; barney/kernels/generateRays.cu:44-243,
   traceRays.dev.cu:20-52, shadeRays.cu:881-1041;
   barney/volume/MCAccelerator.h:569-708). */
gbv_status gbv_render(const gbv_scene *scene, float *d_accum, int width,
                      int height, int accum_id_start, int spp,
                      unsigned long long *d_counters, void *stream);

/* Launch settings of the render kernel.  They change speed, never results:
   every setting renders the identical frame.  A zero field takes its
   default, so a zero-initialised struct (or a null pointer) is the default
   launch.
   blocks_per_sm: resident 288-thread blocks per SM the registers are capped
     for: 4 (default; 56 registers), 5 or 6.
   threshold_pct: a warp keeps traversing while at least this percentage of
     its busy lanes is still tracing (1..100, default 20).
   skip_cells: cell tests and Woodcock distance draws a lane makes per
     traversal iteration before the warp samples (1..1024, default 6).
   stage: shared-memory staging, GBV_STAGE_DEFAULT (the bitmask of non-zero
     majorants, at most 8 KB, computed once per launch in HBM and copied to
     each block by one bulk copy, and the env map's per-row pdf terms),
     GBV_STAGE_NONE, GBV_STAGE_ALL (also the env map's CDF tables, up to
     64 KB per block) or GBV_STAGE_BALLOT (the default staging, with each
     block building the bitmask from the majorants by warp ballots).
   profile: 1 = per-phase cycle and lane counts into d_counters[5..11]
     (needs d_counters; persistent mode only).
   mode: GBV_RENDER_PERSISTENT (one persistent kernel renders every pass)
     or GBV_RENDER_WAVEFRONT (per step, a trace kernel over a queue of rays
     and a shade kernel over the active pixels, with the path state in HBM;
     scratch of about 200 bytes per pixel from the stream's memory pool).
     In wavefront mode threshold_pct is the share of a trace warp's lanes
     that must be idle before it takes new rays (default 25) and
     blocks_per_sm is ignored. */
enum { GBV_STAGE_DEFAULT = 0, GBV_STAGE_NONE = 1, GBV_STAGE_ALL = 2, GBV_STAGE_BALLOT = 3 };
enum { GBV_RENDER_PERSISTENT = 0, GBV_RENDER_WAVEFRONT = 1 };
typedef struct gbv_render_config {
  int blocks_per_sm;
  int threshold_pct;
  int skip_cells;
  int stage;
  int profile;
  int mode;
  int reserved[2]; /* zero */
} gbv_render_config;

/* gbv_render with explicit launch settings (config may be null).  No
   counterpart in the reference (whose launches are fixed). */
gbv_status gbv_render_ex(const gbv_scene *scene, float *d_accum, int width,
                         int height, int accum_id_start, int spp,
                         unsigned long long *d_counters,
                         const gbv_render_config *config, void *stream);

/* Frame partition across ranks (one GPU each), as the reference's tiled
   frame buffer does it: the frame is cut into 32x32-pixel tiles, row-major,
   and rank r of num_ranks owns tiles r, r + num_ranks, r + 2*num_ranks, ...
   gbv_tile_partition (host only) gives the number of tiles rank `rank` owns
   and, if tile_lower is not null, each tile's lower-left pixel (x, y) in
   that order.  Replaces TiledFB::resize's numActiveTilesThisGPU and
   setTileCoordsKernel (barney/fb/TiledFB.cu:226-255). */
gbv_status gbv_tile_partition(int width, int height, int rank, int num_ranks,
                              int *num_tiles, int *tile_lower);

/* gbv_render restricted to the tiles rank `rank` of num_ranks owns: those
   pixels of d_accum (the full width*height frame) are written exactly as
   gbv_render writes them; all other pixels are left untouched.  A rank that
   owns no tile returns at once.  The owners' tiles together are the frame;
   gathering them to one rank is the caller's exchange step (the reference's
   LocalFB::gatherColorChannel / DistFB, barney/fb/LocalFB.cpp:60-70).
   Replaces the per-device part of Context::renderTiles
   (barney/Context.cpp:142-185) on a multi-device context. */
gbv_status gbv_render_tiles(const gbv_scene *scene, float *d_accum, int width,
                            int height, int accum_id_start, int spp, int rank,
                            int num_ranks, unsigned long long *d_counters,
                            void *stream);

/* The compressed tile format of the gather (DistFB's CompressedColorTile,
   barney/fb/DistFB.h:43-48): per 32x32 tile, 1024 uint32 RGBA8 (rgb divided
   by the pixel's largest channel, alpha unscaled) followed by 1024 uint16
   half-precision scales (that largest channel), gbv_compressed_tile_bytes()
   = 6144 bytes per tile.
   gbv_compress_tiles writes the tiles rank `rank` of num_ranks owns
   (gbv_tile_partition order) of the frame d_accum (width*height RGBA float
   accumulation, accum_id passes) to d_tiles; gbv_unpack_tiles writes that
   rank's tiles from d_tiles into d_out (width*height float4, RGBA8 or sRGB
   RGBA8, GBV_FB_*), leaving other pixels alone.  Replace CompressTiles and
   UnpackTiles (barney/fb/DistFB.cu:25-108). */
size_t gbv_compressed_tile_bytes(void);
gbv_status gbv_compress_tiles(const float *d_accum, int width, int height,
                              int accum_id, int rank, int num_ranks,
                              void *d_tiles, void *stream);
gbv_status gbv_unpack_tiles(const void *d_tiles, int width, int height,
                            int rank, int num_ranks, int format, void *d_out,
                            void *stream);

/* gbv_render without any device allocation, for callers that may not
   allocate device memory while they render (an application that hands out
   all HBM from its own pre-sized pool, or a real-time viewer that forbids
   allocation calls on its frame path).  No counterpart in the reference.
   Same arguments and results as gbv_render.  Its one word of scratch (the
   persistent kernel's tile-pool counter) lives in a file-scope device array
   of 4 bytes that every GPU loading this library keeps until exit, instead
   of a cudaMallocAsync/cudaFreeAsync pair.  Every call looks up that
   array's device address on the current device (cudaGetSymbolAddress, which
   allocates nothing), so a device reset between calls is harmless; the first
   call on a device (or after a reset) may load the library's device code
   there, so make it before any stream capture.  All calls share the word and each
   call clears it before its launch, so calls that overlap on the GPU (for
   example on two streams) race.  Frames above 2^30 tiles of 8x4 pixels are
   rejected with GBV_ERROR_INVALID_ARGUMENT. */
gbv_status gbv_render_noalloc(const gbv_scene *scene, float *d_accum, int width,
                              int height, int accum_id_start, int spp,
                              unsigned long long *d_counters, void *stream);

/* Batched rendering: many independent scenes of uneven sizes (each with its
   own field, TF, camera, lights and frame) rendered by one persistent launch
   whose warps take 8x4-pixel tiles from all items.  No counterpart in the
   reference (which renders one model per bnRender).
   gbv_batch_create uploads the items' parameters (allocates and copies; call
   it outside stream capture); gbv_batch_render is one memset and one kernel
   launch on `stream`, so a capture of it replays as a CUDA graph;
   gbv_batch_set_launch sets the launch shape (resident 288-thread blocks per
   SM, 4 to 6, default 4; traversal threshold %, default 20; cell tests and
   Woodcock distance draws per lane and traversal iteration, default 6),
   which changes speed, never results.  Items must share the voxel format and
   layout; each item's frame accumulates exactly as gbv_render would. */
typedef struct gbv_batch gbv_batch;
gbv_status gbv_batch_create(const gbv_scene *scenes, float *const *d_accums,
                            const int *widths, const int *heights, int count,
                            gbv_batch **out);
gbv_status gbv_batch_set_launch(gbv_batch *batch, int blocks_per_sm,
                                int threshold_pct, int skip_cells);
gbv_status gbv_batch_render(gbv_batch *batch, int accum_id_start, int spp,
                            unsigned long long *d_counters, void *stream);
gbv_status gbv_batch_destroy(gbv_batch *batch);

/* Frame-buffer read: d_accum * (1/accum_id) into d_out as float4, RGBA8 or
   sRGB RGBA8.  Replaces linearizeColorAndNormalKernel
   (barney/fb/TiledFB.cu:13-50) with LocalFB::gatherColorChannel's
   accumScale (barney/fb/LocalFB.cpp:60-70). */
gbv_status gbv_tonemap(const float *d_accum, int width, int height,
                       int accum_id, int format, void *d_out, void *stream);

/* ------------------------------------------------------------------------
 * Fixed-step emission-absorption march and its adjoint (no counterpart in
 * the reference, which only delta-tracks).
 * ------------------------------------------------------------------------ */
typedef struct gbv_ea_view {
  float pos[3], dir[3], up[3];
  float fovy;
  int width, height;
} gbv_ea_view;

/* Renders num_views views into d_images (views packed back to back, each
   width*height RGBA float).  FP32 interpolation and transmittance with
   compensated optical depth.  The field is FP32 LINEAR or a brick-corner
   store of any format and brick shape (FP16/BF16/U8 voxels are widened to
   FP32 before interpolation). */
gbv_status gbv_ea_render(const gbv_scene *scene, const gbv_ea_view *views,
                         int num_views, float step, float *d_images,
                         void *stream);
/* Same march in FP64 (finite-difference check mode); d_images are doubles.
   The field must be FP32 LINEAR. */
gbv_status gbv_ea_render_f64(const gbv_scene *scene, const gbv_ea_view *views,
                             int num_views, float step, double *d_images,
                             void *stream);
/* Adjoint by path replay: given the forward images and dL/dimage, adds
   dL/dvoxel into d_grad_scalars (FP32, x-fastest, dims) and dL/dTF into
   d_grad_tf (tf_n*4).  The scene's field must be FP32 LINEAR. */
gbv_status gbv_ea_backward(const gbv_scene *scene, const gbv_ea_view *views,
                           int num_views, float step, const float *d_images,
                           const float *d_grad_images, float *d_grad_scalars,
                           float *d_grad_tf, void *stream);
/* gbv_ea_backward with the adjoint kernel's resident 128-thread blocks per
   SM chosen: 4, 6 (the default, also for 0) or 8.  Speed only; the
   gradients are the same up to the order of floating-point atomics. */
gbv_status gbv_ea_backward_ex(const gbv_scene *scene, const gbv_ea_view *views,
                              int num_views, float step, const float *d_images,
                              const float *d_grad_images, float *d_grad_scalars,
                              float *d_grad_tf, int blocks_per_sm, void *stream);

/* Every EA entry point rejects (GBV_ERROR_INVALID_ARGUMENT, before any
   launch) a step for which a ray along the field's box diagonal would take
   more than 2^24 steps. */

/* ------------------------------------------------------------------------
 * Iso-surface ray queries.
 * ------------------------------------------------------------------------ */

/* For each of num_rays rays, the first crossing of the scene field's
   iso_value, found as the reference's iso-surface geometry finds it: the
   macrocell DDA, cells whose scalar range (d_ranges, from
   gbv_build_mc_ranges or gbv_build_mc_ranges_from_store) holds the value cut
   into 10 sub-steps, linear interpolation inside the first bracketing
   sub-step, and a central-difference normal.  Any voxel layout, format and
   brick shape of the scene.
   d_rays: two float4 per ray, (org.xyz, tmax) and (dir.xyz, unused).
   d_hits: two float4 per ray, (t, P.xyz) and (N.xyz, 1) on a hit (N unit
   length), all zero on a miss.
   Replaces MCIsoSurfaceAccel::isProg up to the hit record
   (barney/volume/MCAccelerator.h:338-503); the material, opacity and hit-ID
   parts of it belong to the surface path, which is not on this path. */
gbv_status gbv_iso_intersect(const gbv_scene *scene, const float *d_ranges,
                             float iso_value, const float *d_rays,
                             long long num_rays, float *d_hits, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GBVOL_H */
