// force_exact.cu -- the traversal kernels in REFERENCE math (correctly rounded 1/sqrt),
// every launch shape; see force_kernels.cuh.
#include "force_kernels.cuh"

namespace gsim {
cudaError_t force_launch_exact(const ForceLaunch& f) { return force_launch_impl<true>(f); }
cudaError_t batch_force_launch_exact(const BatchForceLaunch& b, int* grid_out) {
    return batch_force_launch_impl<true>(b, grid_out);
}
}  // namespace gsim
