// render_store_f16.cu -- the render kernels of the StoreBrickCorners<GBV_VOXEL_F16> voxel store
// (one translation unit per store so the builds run in parallel).
#include "render_wavefront.cuh"

namespace gbv {
GBV_STORE_LAUNCHERS(f16, StoreBrickCorners<GBV_VOXEL_F16>)
}  // namespace gbv
