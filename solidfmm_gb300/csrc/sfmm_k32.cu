// Fused translation kernels, float arithmetic.
#include "sfmm_kernel_impl.cuh"

namespace sfmm {
cudaError_t launch_translate_32(const KParams &p, const LaunchShape &s, int grid, cudaStream_t st)
{
    return launch_typed<float>(p, s, grid, st);
}
int occupancy_32(const LaunchShape &s) { return occupancy_typed<float>(s); }
}  // namespace sfmm
