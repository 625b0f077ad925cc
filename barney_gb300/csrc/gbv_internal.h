// gbv_internal.h -- helpers shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>
#include "../../include/gbvol.h"

namespace gbv {

// Records `msg` as the calling thread's last error and returns `st`.
gbv_status set_error(gbv_status st, const char *msg);
// Converts a pending CUDA launch error into a status.
gbv_status check_launch(const char *what);
gbv_status check_cuda(cudaError_t e, const char *what);

// The device view of a parsed NanoVDB grid whose buffer is at d_grid
// (nanovdb.cu).
struct NvdbGrid;
NvdbGrid make_nvdb_grid(const void *d_grid, const gbv_nanovdb_info &info);

// gbv_render without event counting whose loop-cap events store 1 in
// *d_cap_flag (render.cu; the bn* frame path).
gbv_status render_cap_flagged(const gbv_scene *s, float *d_accum, int width, int height, int accum_id_start,
                              int spp, int *d_cap_flag, void *stream);

// Number of bricks of 2^l[i] cells per axis of a volume with `dims` voxels
// (l == nullptr: 8^3-cell bricks).
inline void brick_counts(const int dims[3], int nb[3], const int *l = nullptr) {
  for (int i = 0; i < 3; i++) {
    const int cells = dims[i] - 1, edge = 1 << (l ? l[i] : 3);
    nb[i] = cells <= 0 ? 0 : (cells + edge - 1) / edge;
  }
}

// Brick shape of a brick-corner layout: log2 of the brick edge per axis,
// each 1..6 (2..64 cells) and at most 15 in sum (32768 cells per brick).
// A null pointer or a 0 entry selects 3 (8 cells).  Returns false if a value
// is outside that range.
inline bool resolve_brick_shape(const int *in, int out[3]) {
  for (int i = 0; i < 3; i++) {
    const int v = in ? in[i] : 0;
    out[i] = v == 0 ? 3 : v;
    if (out[i] < 1 || out[i] > 6) return false;
  }
  return out[0] + out[1] + out[2] <= 15;
}

}  // namespace gbv
