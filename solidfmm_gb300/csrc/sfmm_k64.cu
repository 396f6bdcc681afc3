// Fused translation kernels, double arithmetic.
#include "sfmm_kernel_impl.cuh"

namespace sfmm {
cudaError_t launch_translate_64(const KParams &p, const LaunchShape &s, int grid, cudaStream_t st)
{
    return launch_typed<double>(p, s, grid, st);
}
int occupancy_64(const LaunchShape &s) { return occupancy_typed<double>(s); }
}  // namespace sfmm
