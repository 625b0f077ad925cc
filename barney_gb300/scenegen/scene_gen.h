/* scene_gen.h -- seeded synthetic structured volumes (host memory, no GPU).
 *
 * Input generation for tests, the bench and the CPU baseline; not part of
 * the renderer's C-ABI (include/).  Built as libgbv_scenegen.so.
 */
#ifndef GBV_SCENE_GEN_H
#define GBV_SCENE_GEN_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Blob-plus-noise volume: clamp(sum_i a_i exp(-|x-c_i|^2/(2 s_i^2))
   + U[0,noise] + fBm, 0, 1) on the unit cube, x-fastest, FP32, written to
   `out` (dims[0]*dims[1]*dims[2] floats).  nthreads <= 0: one per host core.
   Returns 0, or 1 for a bad argument (dims below 2, negative counts, null
   pointers). */
int sg_blob_volume(const int dims[3], int num_blobs, uint64_t seed,
                   float noise_amplitude, int fbm_octaves, float fbm_amplitude,
                   int nthreads, float *out);

/* A NanoVDB float grid (format 32.7 memory layout) of a dense x-fastest
   array placed at index `origin`, world = voxel_size * index + translation;
   voxels equal to `background` are inactive.  *out receives a malloc'd
   buffer of *bytes bytes (release with sg_free).  Returns 0, 1 for a bad
   argument, 2 when no voxel is active, 3 when memory runs out. */
int sg_nanovdb_from_dense(const float *values, const int dims[3], const int origin[3],
                          float background, double voxel_size, const double translation[3],
                          void **out, size_t *bytes);
/* The same grid with values of nanovdb::GridType grid_type: 1 Float, 13 Fp4,
   14 Fp8, 15 Fp16 or 16 FpN, quantized as NanoVDB's builder does with
   dithering off; tolerance: the absolute error an FpN leaf's bit width is
   chosen for (negative: the builder's default for a fog volume, 0.01). */
int sg_nanovdb_from_dense_typed(const float *values, const int dims[3], const int origin[3],
                                float background, double voxel_size, const double translation[3],
                                int grid_type, float tolerance, void **out, size_t *bytes);
void sg_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
