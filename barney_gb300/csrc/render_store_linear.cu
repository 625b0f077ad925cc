// render_store_linear.cu -- the render kernels of the StoreLinearF32 voxel store
// (one translation unit per store so the builds run in parallel).
#include "render_wavefront.cuh"

namespace gbv {
GBV_STORE_LAUNCHERS(linear, StoreLinearF32)
}  // namespace gbv
