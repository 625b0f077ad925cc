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

// Number of 8^3-cell bricks per axis of a volume with `dims` voxels.
inline void brick_counts(const int dims[3], int nb[3]) {
  for (int i = 0; i < 3; i++) {
    int cells = dims[i] - 1;
    nb[i] = cells <= 0 ? 0 : (cells + 7) / 8;
  }
}

}  // namespace gbv
