// render_store_u8.cu -- the render kernels of the StoreBrickCorners<GBV_VOXEL_U8_SCALED> voxel store
// (one translation unit per store so the builds run in parallel).
#include "render_wavefront.cuh"

namespace gbv {
GBV_STORE_LAUNCHERS(u8, StoreBrickCorners<GBV_VOXEL_U8_SCALED>)
}  // namespace gbv
