// render_store_bf16.cu -- the render kernels of the StoreBrickCorners<GBV_VOXEL_BF16> voxel store
// (one translation unit per store so the builds run in parallel).
#include "render_wavefront.cuh"

namespace gbv {
GBV_STORE_LAUNCHERS(bf16, StoreBrickCorners<GBV_VOXEL_BF16>)
}  // namespace gbv
