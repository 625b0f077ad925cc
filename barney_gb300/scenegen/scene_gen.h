/* scene_gen.h -- seeded synthetic structured volumes (host memory, no GPU).
 *
 * Input generation for tests, the bench and the CPU baseline; not part of
 * the renderer's C-ABI (include/).  Built as libgbv_scenegen.so.
 */
#ifndef GBV_SCENE_GEN_H
#define GBV_SCENE_GEN_H
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

#ifdef __cplusplus
}
#endif
#endif
