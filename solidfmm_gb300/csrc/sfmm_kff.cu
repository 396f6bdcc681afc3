// Fused translation kernels, ff arithmetic.
#include "sfmm_kernel_impl.cuh"

namespace sfmm {
cudaError_t launch_translate_ff(const KParams &p, const LaunchShape &s, int grid, cudaStream_t st)
{
    return launch_typed<ff>(p, s, grid, st);
}
int occupancy_ff(const LaunchShape &s) { return occupancy_typed<ff>(s); }
}  // namespace sfmm
