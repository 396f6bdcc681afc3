// Fused translation kernels, ff arithmetic with block fixed-point swaps.
#include "sfmm_kernel_impl.cuh"

namespace sfmm {
cudaError_t launch_translate_ffq(const KParams &p, const LaunchShape &s, int grid, cudaStream_t st)
{
    return launch_typed<ff, true>(p, s, grid, st);
}
int occupancy_ffq(const LaunchShape &s) { return occupancy_typed<ff, true>(s); }
}  // namespace sfmm
