// P2M / P2L expansion building and order bucketing.
//
// P2M/P2L: out[j] += sum_k q_jk * R(x_jk - c_j) (or S), the reference's
// fmadd(q, harmonics::R/S(P, x - c), E) (solid.cpp:70-104) with the R and S
// recurrences of harmonics.cpp:32-80 and :177-224, evaluated column by column
// (fixed m, increasing n) so that each coefficient is accumulated as soon as
// it is produced.  One thread per expansion, FP64 arithmetic.
//
// Bucketing: a counting sort of translation indices by the key
// (p_in, p_out), so that warps see uniform orders.
#include <algorithm>
#include <cstdint>
#include <map>
#include <mutex>

#include "sfmm.h"
#include "sfmm_launch.hpp"

namespace sfmm {

// Expansion j takes particles [j nq, (j+1) nq), or [offset[j], offset[j+1])
// when an offset array is given (ragged leaves).
template <class Out>
__global__ void k_p2x(int kind, int P, long long nexp, long long nq, const uint32_t *__restrict__ offset,
                      const double *__restrict__ q, const double *__restrict__ pos,
                      const double *__restrict__ centre, Out *out, long long stride)
{
    long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= nexp) return;
    Out *o = out + j * stride;
    const double cx = centre[3 * j], cy = centre[3 * j + 1], cz = centre[3 * j + 2];
    const long long k0 = offset ? (long long)offset[j] : j * nq;
    const long long k1 = offset ? (long long)offset[j + 1] : (j + 1) * nq;
    for (long long k = k0; k < k1; ++k) {
        const double w = q[k];
        const double *pp = pos + 3 * k;
        const double x = pp[0] - cx, y = pp[1] - cy, z = pp[2] - cz;
        const double r2 = x * x + y * y + z * z;
        if (kind == 0) {
            // regular harmonics R
            double dr = 1.0, di = 0.0;  // R(m,m)
            for (int m = 0; m < P; ++m) {
                if (m > 0) {
                    double f = (m == 1) ? 0.5 : 1.0 / (2.0 * m);
                    double nr = (dr * x - di * y) * f;
                    double ni = (dr * y + di * x) * f;
                    dr = nr;
                    di = ni;
                }
                // column m: R(m,m), R(m+1,m) = z R(m,m), then the three-term recurrence
                double ar = dr, ai = di;            // R(n-1,m)
                double br = 0.0, bi = 0.0;          // R(n-2,m)
                o[m * (m + 1) + m] += (Out)(w * ar);
                o[(m + 1) * (m + 1) + m] += (Out)(w * ai);
                for (int n = m + 1; n < P; ++n) {
                    double cr, ci;
                    if (n == m + 1) {
                        cr = z * ar;
                        ci = z * ai;
                    } else {
                        double f = 1.0 / ((double)(n + m) * (double)(n - m));
                        cr = (ar * z * (2 * n - 1) - r2 * br) * f;
                        ci = (ai * z * (2 * n - 1) - r2 * bi) * f;
                    }
                    o[n * (n + 1) + m] += (Out)(w * cr);
                    o[(n + 1) * (n + 1) + m] += (Out)(w * ci);
                    br = ar;
                    bi = ai;
                    ar = cr;
                    ai = ci;
                }
            }
        } else {
            // singular harmonics S
            const double r2inv = 1.0 / r2;
            double dr = sqrt(r2inv), di = 0.0;  // S(m,m)
            for (int m = 0; m < P; ++m) {
                if (m > 0) {
                    double f = (2.0 * m - 1.0) * r2inv;
                    double nr = (dr * x - di * y) * f;
                    double ni = (dr * y + di * x) * f;
                    dr = nr;
                    di = ni;
                }
                double ar = dr, ai = di, br = 0.0, bi = 0.0;
                o[m * (m + 1) + m] += (Out)(w * ar);
                o[(m + 1) * (m + 1) + m] += (Out)(w * ai);
                for (int n = m + 1; n < P; ++n) {
                    double cr, ci;
                    if (n == m + 1) {
                        double f = (2.0 * m + 1.0) * z * r2inv;
                        cr = f * ar;
                        ci = f * ai;
                    } else {
                        double c2 = (double)(n + m - 1) * (double)(n - m - 1);
                        cr = (ar * z * (2 * n - 1) - c2 * br) * r2inv;
                        ci = (ai * z * (2 * n - 1) - c2 * bi) * r2inv;
                    }
                    o[n * (n + 1) + m] += (Out)(w * cr);
                    o[(n + 1) * (n + 1) + m] += (Out)(w * ci);
                    br = ar;
                    bi = ai;
                    ar = cr;
                    ai = ci;
                }
            }
        }
    }
}

cudaError_t launch_p2x(bool f64, int kind, int P, long long nexp, long long nq, const uint32_t *offset,
                       const double *q, const double *pos, const double *centre, void *out, long long stride,
                       cudaStream_t st)
{
    if (nexp == 0) return cudaSuccess;
    int tb = 128;
    long long grid = (nexp + tb - 1) / tb;
    clear_stale_error();
    if (f64)
        k_p2x<double><<<(unsigned)grid, tb, 0, st>>>(kind, P, nexp, nq, offset, q, pos, centre, (double *)out,
                                                      stride);
    else
        k_p2x<float><<<(unsigned)grid, tb, 0, st>>>(kind, P, nexp, nq, offset, q, pos, centre, (float *)out,
                                                     stride);
    return cudaGetLastError();
}

// ---- evaluation (L2P / M2P) ----
//
// phi(x) = dot(E, R(x - c)) for a local expansion (kind 0) or
// dot(E, S(x - c)) for a multipole expansion (kind 1), the reference's
// solid dot product (solid.cpp:41-66): sum over n, m >= 0 of re*re + im*im,
// weighted 2 for m > 0.  The harmonics are produced column by column as in
// P2M/P2L and consumed at once, so a thread keeps no expansion-sized state.
// The gradient of a local expansion uses (d/dx - i d/dy) R_n^m = R_{n-1}^{m-1},
// (d/dx + i d/dy) R_n^m = -R_{n-1}^{m+1} and d/dz R_n^m = R_{n-1}^m: each
// R_k^v produced pairs with the degree-(k+1) coefficients v-1, v, v+1.
template <class In>
__global__ void k_eval(int kind, int P, long long npts, const double *__restrict__ pos,
                       const uint32_t *__restrict__ box, const In *__restrict__ E, long long stride,
                       const double *__restrict__ centre, double *pot, double *grad)
{
    const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= npts) return;
    const long long b = box ? (long long)box[j] : j;
    const In *e = E + b * stride;
    const double x = pos[3 * j] - centre[3 * b], y = pos[3 * j + 1] - centre[3 * b + 1],
                 z = pos[3 * j + 2] - centre[3 * b + 2];
    const double r2 = x * x + y * y + z * z;
    auto re = [&](int n, int m) { return (double)e[n * (n + 1) + m]; };
    auto im = [&](int n, int m) { return (double)e[(n + 1) * (n + 1) + m]; };
    double phi = 0, gx = 0, gy = 0, gz = 0;
    const bool want_grad = grad != nullptr && kind == 0;
    if (kind == 0) {
        double dr = 1.0, di = 0.0;  // R(m,m)
        for (int m = 0; m < P; ++m) {
            if (m > 0) {
                const double f = 1.0 / (2.0 * m);
                const double nr = (dr * x - di * y) * f, ni = (dr * y + di * x) * f;
                dr = nr;
                di = ni;
            }
            const double w = m ? 2.0 : 1.0;
            double ar = dr, ai = di, br = 0.0, bi = 0.0;
            for (int n = m; n < P; ++n) {
                double cr = ar, ci = ai;  // R(n,m)
                if (n == m + 1) {
                    cr = z * ar;
                    ci = z * ai;
                } else if (n > m + 1) {
                    const double f = 1.0 / ((double)(n + m) * (double)(n - m));
                    cr = (ar * z * (2 * n - 1) - r2 * br) * f;
                    ci = (ai * z * (2 * n - 1) - r2 * bi) * f;
                }
                phi += w * (re(n, m) * cr + im(n, m) * ci);
                if (want_grad && n + 1 < P) {
                    const int k1 = n + 1;
                    gz += w * (re(k1, m) * cr + im(k1, m) * ci);
                    if (m == 0) {
                        gx += cr * re(k1, 1);
                        gy += cr * im(k1, 1);
                    } else {
                        // conj(R) (L^{m+1} - L^{m-1}) and conj(R) (L^{m-1} + L^{m+1})
                        const double xr = re(k1, m + 1) - re(k1, m - 1), xi = im(k1, m + 1) - im(k1, m - 1);
                        const double yr = re(k1, m - 1) + re(k1, m + 1), yi = im(k1, m - 1) + im(k1, m + 1);
                        gx += cr * xr + ci * xi;
                        gy += cr * yi - ci * yr;
                    }
                }
                if (n > m) {
                    br = ar;
                    bi = ai;
                    ar = cr;
                    ai = ci;
                }
            }
        }
    } else {
        const double r2inv = 1.0 / r2;
        double dr = sqrt(r2inv), di = 0.0;  // S(m,m)
        for (int m = 0; m < P; ++m) {
            if (m > 0) {
                const double f = (2.0 * m - 1.0) * r2inv;
                const double nr = (dr * x - di * y) * f, ni = (dr * y + di * x) * f;
                dr = nr;
                di = ni;
            }
            const double w = m ? 2.0 : 1.0;
            double ar = dr, ai = di, br = 0.0, bi = 0.0;
            for (int n = m; n < P; ++n) {
                double cr = ar, ci = ai;
                if (n == m + 1) {
                    const double f = (2.0 * m + 1.0) * z * r2inv;
                    cr = f * ar;
                    ci = f * ai;
                } else if (n > m + 1) {
                    const double c2 = (double)(n + m - 1) * (double)(n - m - 1);
                    cr = (ar * z * (2 * n - 1) - c2 * br) * r2inv;
                    ci = (ai * z * (2 * n - 1) - c2 * bi) * r2inv;
                }
                phi += w * (re(n, m) * cr + im(n, m) * ci);
                if (n > m) {
                    br = ar;
                    bi = ai;
                    ar = cr;
                    ai = ci;
                }
            }
        }
    }
    pot[j] += phi;
    if (want_grad) {
        grad[3 * j] += gx;
        grad[3 * j + 1] += gy;
        grad[3 * j + 2] += gz;
    }
}

cudaError_t launch_eval(bool f64, int kind, int P, long long npts, const double *pos, const uint32_t *box,
                        const void *E, long long stride, const double *centre, double *pot, double *grad,
                        cudaStream_t st)
{
    if (npts == 0) return cudaSuccess;
    const int tb = 128;
    const long long grid = (npts + tb - 1) / tb;
    clear_stale_error();
    if (f64)
        k_eval<double><<<(unsigned)grid, tb, 0, st>>>(kind, P, npts, pos, box, (const double *)E, stride, centre,
                                                       pot, grad);
    else
        k_eval<float><<<(unsigned)grid, tb, 0, st>>>(kind, P, npts, pos, box, (const float *)E, stride, centre,
                                                      pot, grad);
    return cudaGetLastError();
}

// ---- accumulation of per-target results into targets given by address ----
//
// One warp per target: target[c] += slots[j * stride + c] for c < cnt[j].
// The targets are distinct, so plain read-modify-writes suffice; they may be
// host solids that the GPU reads and writes through the host page tables.
template <class T>
__global__ void k_add_slots(long long nt, const unsigned long long *__restrict__ tptr,
                            const uint32_t *__restrict__ cnt, const T *__restrict__ slots, long long stride)
{
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= nt) return;
    T *o = reinterpret_cast<T *>(tptr[w]);
    const T *r = slots + w * stride;
    for (uint32_t c = lane; c < cnt[w]; c += 32) o[c] += r[c];
}

cudaError_t launch_add_slots(bool f64, long long nt, const unsigned long long *tptr, const uint32_t *cnt,
                             const void *slots, long long stride, cudaStream_t st)
{
    if (nt == 0) return cudaSuccess;
    const int tb = 256;
    const long long grid = (nt * 32 + tb - 1) / tb;
    clear_stale_error();
    if (f64)
        k_add_slots<double><<<(unsigned)grid, tb, 0, st>>>(nt, tptr, cnt, (const double *)slots, stride);
    else
        k_add_slots<float><<<(unsigned)grid, tb, 0, st>>>(nt, tptr, cnt, (const float *)slots, stride);
    return cudaGetLastError();
}

// ---- bucketing by (p_in, p_out) ----

__global__ void k_bucket_count(long long n, const uint32_t *pin, const uint32_t *pout, uint32_t *cnt, int K)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        uint32_t key = min(pin[i], (uint32_t)(K - 1)) * (uint32_t)K + min(pout[i], (uint32_t)(K - 1));
        atomicAdd(&cnt[key], 1u);
    }
}

// single CTA exclusive scan over nkeys counters, any number: thread t
// handles a chunk of ceil(nkeys / 1024) consecutive keys.  Callers: the
// context bucketing (K = P + 1 <= 87) and the allocation-free entry point
// (K = max_order + 1 <= 87, 7 569 keys)
__global__ void k_bucket_scan(uint32_t *cnt, int nkeys)
{
    __shared__ uint32_t part[1024];
    const int t = threadIdx.x;
    const int per = (nkeys + blockDim.x - 1) / blockDim.x;
    uint32_t s = 0;
    for (int k = t * per; k < min(nkeys, (t + 1) * per); ++k) s += cnt[k];
    part[t] = s;
    __syncthreads();
    if (t == 0) {
        uint32_t run = 0;
        for (int k = 0; k < (int)blockDim.x; ++k) {
            uint32_t v = part[k];
            part[k] = run;
            run += v;
        }
    }
    __syncthreads();
    uint32_t run = part[t];
    for (int k = t * per; k < min(nkeys, (t + 1) * per); ++k) {
        uint32_t v = cnt[k];
        cnt[k] = run;
        run += v;
    }
}

__global__ void k_bucket_scatter(long long n, const uint32_t *pin, const uint32_t *pout, uint32_t *off, int K,
                                 uint32_t *order)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        uint32_t key = min(pin[i], (uint32_t)(K - 1)) * (uint32_t)K + min(pout[i], (uint32_t)(K - 1));
        uint32_t pos = atomicAdd(&off[key], 1u);
        order[pos] = (uint32_t)i;
    }
}

size_t bucket_work_words(int P) { return (size_t)(P + 1) * (P + 1); }

cudaError_t launch_bucket(long long n, const uint32_t *pin, const uint32_t *pout, uint32_t *order, uint32_t *work,
                          int P, cudaStream_t st)
{
    const int K = P + 1;
    const int nkeys = K * K;
    clear_stale_error();
    cudaError_t e = cudaMemsetAsync(work, 0, sizeof(uint32_t) * nkeys, st);
    if (e != cudaSuccess) return e;
    if (n == 0) return cudaSuccess;
    int grid = (int)std::min<long long>((n + 255) / 256, 4096);
    k_bucket_count<<<grid, 256, 0, st>>>(n, pin, pout, work, K);
    k_bucket_scan<<<1, 1024, 0, st>>>(work, nkeys);
    k_bucket_scatter<<<grid, 256, 0, st>>>(n, pin, pout, work, K, order);
    return cudaGetLastError();
}

}  // namespace sfmm

// ---- bucketing without allocation ----
//
// The counters of the bucketing sort live in a fixed device array instead of
// context memory, for callers that must not allocate device memory at all:
// codes that hand the whole device to their own memory pool, run under a
// hard per-process memory cap, or issue work from paths where a cudaMalloc
// would stall or fail.  The array is sized for orders up to 86 (the largest
// order a solidfmm operator accepts), 87 x 87 counters = 30 KiB; every GPU
// that loads the library keeps it until the process exits.

namespace {

constexpr int kStaticBucketMaxOrder = 86;
constexpr int kStaticBucketKeys = (kStaticBucketMaxOrder + 1) * (kStaticBucketMaxOrder + 1);

__device__ __align__(256) uint32_t g_bucket_counters[kStaticBucketKeys];

// Device address of g_bucket_counters.  A __device__ array belongs to one CUDA
// context (one per device with the runtime's primary contexts, but a caller
// of the driver API may make another current, and cudaDeviceReset replaces
// the primary one), so the address is looked up again on every call made
// outside a stream capture and cached per current context for calls made
// during a capture, when no lookup may load the module.
std::mutex g_bucket_mtx;
std::map<void *, uint32_t *> g_bucket_addr;

using CtxGetCurrent = int (*)(void **);

// the current CUcontext through the driver entry point (the library does not
// link libcuda, so that it loads on machines without a GPU driver)
void *current_context()
{
    static CtxGetCurrent fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<CtxGetCurrent>(f);
    }();
    void *ctx = nullptr;
    if (!fn || fn(&ctx) != 0) return nullptr;
    return ctx;
}

}  // namespace

extern "C" int sfmm_bucket_by_order_noalloc(size_t n, const uint32_t *p_in, const uint32_t *p_out, uint32_t *order,
                                            size_t max_order, void *stream)
{
    if (max_order > (size_t)kStaticBucketMaxOrder) return SFMM_ORDER_RANGE;
    if (n > 0xffffffffull) return SFMM_INVALID_ARG;
    if (n == 0) return SFMM_OK;
    if (!p_in || !p_out || !order) return SFMM_INVALID_ARG;
    void *ctx = current_context();
    if (!ctx) {  // no context current yet: initialise the current device's primary context
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaSetDevice(dev) != cudaSuccess) return SFMM_CUDA_ERROR;
        ctx = current_context();
    }
    if (!ctx) return SFMM_CUDA_ERROR;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing((cudaStream_t)stream, &cap) != cudaSuccess) return SFMM_CUDA_ERROR;
    uint32_t *counters = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_bucket_mtx);
        if (cap == cudaStreamCaptureStatusNone) {
            // the host-side symbol is only a stand-in for the array; the
            // kernels need its address in the current context
            if (cudaGetSymbolAddress((void **)&counters, g_bucket_counters) != cudaSuccess) return SFMM_CUDA_ERROR;
            g_bucket_addr[ctx] = counters;
        } else {
            auto it = g_bucket_addr.find(ctx);
            if (it == g_bucket_addr.end()) return SFMM_INVALID_ARG;  // first call inside a capture
            counters = it->second;
        }
    }
    // the counters are cleared on the stream before use (launch_bucket)
    cudaError_t e = sfmm::launch_bucket((long long)n, p_in, p_out, order, counters, (int)max_order,
                                        (cudaStream_t)stream);
    return e == cudaSuccess ? SFMM_OK : SFMM_CUDA_ERROR;
}

