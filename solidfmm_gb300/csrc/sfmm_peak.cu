// Pipe-peak probes for roofline denominators: FP64 FMA and FP32 FMA
// throughput measured with long dependent-chain-free FMA loops.  The FP64
// and FP32 peaks of GB300 are not published in a form that matches the
// clock under load, so the benchmark measures them in the same run.
#include <cuda_runtime.h>

#include "sfmm.h"
#include "sfmm_launch.hpp"

namespace {

template <class T>
__global__ void k_fma_peak(T *out, int iters, T a, T b)
{
    T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = x0 * a + b;
        x1 = x1 * a + b;
        x2 = x2 * a + b;
        x3 = x3 * a + b;
        x4 = x4 * a + b;
        x5 = x5 * a + b;
        x6 = x6 * a + b;
        x7 = x7 * a + b;
    }
    T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == (T)-1.2345) out[threadIdx.x] = s;  // keep the loop alive
}

__global__ void k_imad_peak(long long *out, int iters, int a, int b)
{
    long long x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
              x7 = x0 + 7;
    int m = a + (int)threadIdx.x;
    for (int i = 0; i < iters; ++i) {
        x0 += (long long)m * b;
        x1 += (long long)m * (b + 1);
        x2 += (long long)m * (b + 2);
        x3 += (long long)m * (b + 3);
        x4 += (long long)m * (b + 4);
        x5 += (long long)m * (b + 5);
        x6 += (long long)m * (b + 6);
        x7 += (long long)m * (b + 7);
        m ^= i;
    }
    long long s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == -12345) out[threadIdx.x] = s;
}

}  // namespace

// Throughput of 32x32->64-bit integer multiply-adds (ops/s, one per MAC).
extern "C" int sfmm_measure_imad_peak(int device, double *ops_per_second)
{
    if (!ops_per_second) return SFMM_INVALID_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return SFMM_CUDA_ERROR;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    void *out = nullptr;
    if (cudaMalloc(&out, 1024 * 8) != cudaSuccess) return SFMM_CUDA_ERROR;
    const int threads = 256, blocks = sms * 8, iters = 16384;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    sfmm::clear_stale_error();
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        k_imad_peak<<<blocks, threads>>>((long long *)out, iters, 3, 5);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return SFMM_CUDA_ERROR;
    *ops_per_second = 8.0 * iters * (double)threads * blocks / (best * 1e-3);
    return SFMM_OK;
}

extern "C" int sfmm_measure_fma_peak(int fp64, int device, double *flops_per_second)
{
    if (!flops_per_second) return SFMM_INVALID_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return SFMM_CUDA_ERROR;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    void *out = nullptr;
    if (cudaMalloc(&out, 1024 * 8) != cudaSuccess) return SFMM_CUDA_ERROR;
    const int threads = 256, blocks = sms * 8;
    const int iters = fp64 ? 4096 : 65536;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    sfmm::clear_stale_error();
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        if (fp64) k_fma_peak<double><<<blocks, threads>>>((double *)out, iters, 0.999999, 1e-7);
        else k_fma_peak<float><<<blocks, threads>>>((float *)out, iters, 0.999999f, 1e-7f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return SFMM_CUDA_ERROR;
    *flops_per_second = 2.0 * 8.0 * iters * (double)threads * blocks / (best * 1e-3);
    return SFMM_OK;
}
