// Explicit instantiation of the fused translation kernel for one arithmetic
// type; included by sfmm_k64.cu, sfmm_k32.cu and sfmm_kff.cu (one translation
// unit each, compiled in parallel).
#pragma once

#include "sfmm_launch.hpp"
#include "sfmm_translate.cuh"

namespace sfmm {

template <class A, int ACC>
static cudaError_t launch_acc(const KParams &p, const LaunchShape &s, int grid, cudaStream_t st)
{
    static bool attr_set = false;
    auto kern = k_translate<A, ACC, false>;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    kern<<<grid, s.threads, s.smem, st>>>(p);
    return cudaGetLastError();
}

template <class A, int ACC>
static int occupancy_acc(const LaunchShape &s)
{
    auto kern = k_translate<A, ACC, false>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 232448);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, s.threads, s.smem) != cudaSuccess) return 1;
    return nb > 0 ? nb : 1;
}

template <class A>
static cudaError_t launch_typed(const KParams &p, const LaunchShape &s, int grid, cudaStream_t st)
{
    switch (s.acc) {
    case 2: return launch_acc<A, 2>(p, s, grid, st);
    case 4: return launch_acc<A, 4>(p, s, grid, st);
    case 6: return launch_acc<A, 6>(p, s, grid, st);
    case 8: return launch_acc<A, 8>(p, s, grid, st);
    default: return cudaErrorInvalidValue;
    }
}

template <class A>
static int occupancy_typed(const LaunchShape &s)
{
    switch (s.acc) {
    case 2: return occupancy_acc<A, 2>(s);
    case 4: return occupancy_acc<A, 4>(s);
    case 6: return occupancy_acc<A, 6>(s);
    case 8: return occupancy_acc<A, 8>(s);
    default: return 1;
    }
}

}  // namespace sfmm
