// render_store_f32.cu -- the render kernels of the StoreBrickCorners<GBV_VOXEL_F32> voxel store
// (one translation unit per store so the builds run in parallel).
#include "render_wavefront.cuh"

namespace gbv {
GBV_STORE_LAUNCHERS(f32, StoreBrickCorners<GBV_VOXEL_F32>)
}  // namespace gbv
