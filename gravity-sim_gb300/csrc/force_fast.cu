// force_fast.cu -- the traversal kernels in FAST math (hardware rsqrt), every launch
// shape; see force_kernels.cuh.
#include "force_kernels.cuh"

namespace gsim {
cudaError_t force_launch_fast(const ForceLaunch& f) { return force_launch_impl<false>(f); }
cudaError_t batch_force_launch_fast(const BatchForceLaunch& b, int* grid_out) {
    return batch_force_launch_impl<false>(b, grid_out);
}
bool force_shape_supported(uint32_t warps, uint32_t short_lists) {
    return short_lists ? warps == 2 : (warps == 1 || warps == 2 || warps == 4);
}
}  // namespace gsim
