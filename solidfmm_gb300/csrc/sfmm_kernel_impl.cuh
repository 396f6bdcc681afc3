// Explicit instantiation of the fused translation kernel for one arithmetic
// type; included by sfmm_k64.cu, sfmm_k32.cu, sfmm_kff.cu and sfmm_kffq.cu
// (one translation unit each, compiled in parallel).  Instances: group size G
// in {4, 8, 32} and accumulator blocks ACC = ceil(P / G) rounded up to an
// instantiated size; the fixed-point float-float variant (orders <= 28) has
// no one-warp-per-translation instances.
#pragma once

#include "sfmm_launch.hpp"
#include "sfmm_translate.cuh"

namespace sfmm {

// Launch shapes come from best_shape, whose occupancy query (below) has set
// the kernels' shared-memory limit on the current device, so a launch (also
// inside a CUDA graph capture) makes no other runtime call.  Each shape has
// two instances: expansions in device memory, or in host memory read over
// the link (p.in_hbm).
template <class A, int G, int ACC, bool FIX>
static cudaError_t launch_inst(const KParams &p, const LaunchShape &s, int grid, cudaStream_t st)
{
    clear_stale_error();
    if (p.work) {
        if (!p.in_hbm) return cudaErrorInvalidValue;  // work lists are a device-memory form
        k_translate<A, G, ACC, FIX, true, true><<<grid, s.threads, s.smem, st>>>(p);
    } else if (p.in_hbm) {
        k_translate<A, G, ACC, FIX, true><<<grid, s.threads, s.smem, st>>>(p);
    } else {
        k_translate<A, G, ACC, FIX, false><<<grid, s.threads, s.smem, st>>>(p);
    }
    return cudaGetLastError();
}

// resident CTAs per SM of the device-memory instance (the shape's grid
// sizing); the host-memory and work-list instances are set up alongside
template <class A, int G, int ACC, bool FIX>
static int occupancy_inst(const LaunchShape &s)
{
    auto kern = k_translate<A, G, ACC, FIX, true>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448);
    cudaFuncSetAttribute(k_translate<A, G, ACC, FIX, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448);
    cudaFuncSetAttribute(k_translate<A, G, ACC, FIX, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, s.threads, s.smem) != cudaSuccess) return 0;
    return nb;
}

#define SFMM_FOR_SHAPES(X) \
    X(4, 2) X(4, 4) X(4, 6) X(4, 8) X(8, 1) X(8, 2) X(8, 3) X(8, 4) X(32, 2) X(32, 3)

template <class A, bool FIX = false>
static cudaError_t launch_typed(const KParams &p, const LaunchShape &s, int grid, cudaStream_t st)
{
#define X(G_, A_) \
    if constexpr (!(FIX && G_ == 32))                                   \
        if (s.G == G_ && s.acc == A_) return launch_inst<A, G_, A_, FIX>(p, s, grid, st);
    SFMM_FOR_SHAPES(X)
#undef X
    return cudaErrorInvalidValue;
}

template <class A, bool FIX = false>
static int occupancy_typed(const LaunchShape &s)
{
#define X(G_, A_) \
    if constexpr (!(FIX && G_ == 32))              \
        if (s.G == G_ && s.acc == A_) return occupancy_inst<A, G_, A_, FIX>(s);
    SFMM_FOR_SHAPES(X)
#undef X
    return 0;
}

}  // namespace sfmm
