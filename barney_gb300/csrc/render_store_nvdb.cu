// render_store_nvdb.cu -- the render kernels of the StoreNanoVDB voxel store
// (one translation unit per store so the builds run in parallel).
#include "render_wavefront.cuh"

namespace gbv {
GBV_STORE_LAUNCHERS(nvdb, StoreNanoVDB)
}  // namespace gbv
