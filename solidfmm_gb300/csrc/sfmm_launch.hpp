// Host-side launch interface between the C ABI and the kernel translation units.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace sfmm {

// Clear a stale, non-sticky error that an earlier failed runtime call on this
// thread left behind (a failed allocation, the library's or the caller's), so
// that the cudaGetLastError after a launch reports that launch alone.
inline void clear_stale_error() { (void)cudaGetLastError(); }

struct KParams;

// FFQ: float-float with block fixed-point swaps and beta rotations;
// TC32 / TC16 / TC16X6: the tensor-core kernel with 3xTF32 / 3xBF16 /
// BF16x6 split products
enum class Arith { F64 = 0, F32 = 1, FF = 2, FFQ = 3, TC32 = 4, TC16 = 5, TC16X6 = 6 };
constexpr int kNumArith = 7;
inline bool is_tc(Arith a) { return a == Arith::TC32 || a == Arith::TC16 || a == Arith::TC16X6; }
// operand format of a tensor-core arithmetic (sfmm_tc.cu)
inline int tc_mode(Arith a) { return a == Arith::TC32 ? 0 : (a == Arith::TC16 ? 1 : 2); }

// Largest order the fused translation kernel supports: 4 threads per
// translation up to 32, one warp per translation up to 96 (the reference's
// FP64 limit is 86).
constexpr int kMaxKernelOrder = 96;
// FP32 and float-float arithmetic keep the orthogonal-basis scale factors
// sqrt((n-m)!(n+m)!) in FP32 range only up to this order.
constexpr int kMaxFloatOrder = 28;

struct LaunchShape {
    int G = 4;         // threads per translation
    int acc = 0;       // accumulator blocks per thread, ceil(P/G) rounded to an instantiated size
    int TS = 0;        // translations per CTA
    int spad = 0;      // buffer elements per translation
    size_t smem = 0;   // dynamic shared memory bytes
    int threads = 0;   // G * TS
    int blocks_per_sm = 0;  // resident CTAs per SM (occupancy of this shape)
};

LaunchShape translate_shape(Arith a, int P, int G, int ts);
int default_group(Arith a, int P);
// the tile with the most resident threads per SM for G threads per
// translation (ties: the larger tile, or the smaller with small_tiles), among
// CTAs of at least min_threads threads when one fits
LaunchShape best_shape(Arith a, int P, int G, bool small_tiles = false, int min_threads = 128);

// Launch the fused translation kernel (defined in sfmm_k{64,32,ff,ffq}.cu).
cudaError_t launch_translate(Arith a, const KParams &p, const LaunchShape &s, int grid, cudaStream_t st);
int translate_blocks_per_sm(Arith a, const LaunchShape &s);

// Tensor-core translation kernel (sfmm_tc.cu): device images of the
// constant matrices for one operand format (mode 0 = 3xTF32, 1 = 3xBF16,
// 2 = BF16x6),
// built from the context's host tables for degrees below min(P, 16).
struct HostTables;
struct TcDevTables;
cudaError_t tc_prepare(TcDevTables **out, int mode, const HostTables &host);
void tc_release(TcDevTables *t);
int tc_max_order();
cudaError_t launch_translate_tc(const KParams &p, const TcDevTables *t, int num_sms, cudaStream_t st);

// P2M / P2L (sfmm_p2x.cu)
// expansion j takes particles [j nq, (j+1) nq), or [offset[j], offset[j+1]) with an offset array
cudaError_t launch_p2x(bool f64, int kind, int P, long long nexp, long long nq, const uint32_t *offset,
                       const double *q, const double *pos, const double *centre, void *out, long long stride,
                       cudaStream_t st);

// L2P / M2P evaluation (sfmm_p2x.cu): float-float over normalised copies of
// the nexp expansions in `scratch` (eval_scratch_bytes of it) for orders up
// to 32, else (scratch null or higher orders) one FP64 thread per point.
size_t eval_scratch_bytes(int P, long long nexp);
cudaError_t launch_eval(bool f64, int kind, int P, long long npts, const double *pos, const uint32_t *box,
                        const void *E, long long stride, long long nexp, const double *centre, double *pot,
                        double *grad, void *scratch, cudaStream_t st);

// target[j] += slots[j] for unique host targets given by address (sfmm_p2x.cu)
cudaError_t launch_add_slots(bool f64, long long nt, const unsigned long long *tptr, const uint32_t *cnt,
                             const void *slots, long long stride, cudaStream_t st);

// bucketing by order pair (sfmm_p2x.cu)
cudaError_t launch_bucket(long long n, const uint32_t *pin, const uint32_t *pout, uint32_t *order,
                          uint32_t *work, int P, cudaStream_t st);
size_t bucket_work_words(int P);

}  // namespace sfmm
