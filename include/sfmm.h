/*
 * sfmm.h -- C ABI of solidfmm-gb300: GB300 (sm_103a) translation operators
 * M2M, M2L and L2L on solid-harmonic expansions.
 *
 * This is the only CUDA-facing surface.  The C++ drop-in headers under
 * include/solidfmm/ (solid, harmonics, handles, translations,
 * multithreaded_translator) are implemented on top of it.
 *
 * Expansion layout (identical to the reference's solid<real>,
 * solidfmm/solid.hpp:59-60): an expansion of order P holds P(P+1) reals; for
 * degree n < P the n+1 real parts re(n,0..n) start at n(n+1) and the n+1
 * imaginary parts im(n,0..n) start at (n+1)^2.  Batches address expansions in
 * a uniform-stride array: expansion j starts at base + j*stride reals.
 *
 * Semantics of every translation call (solidfmm/translations.hpp:94-170):
 *   target += T(source, shift),  shift = new centre - old centre,
 * with per-translation source order P_in and target order P_out, both at most
 * the context's order.  M2M and L2L with a zero shift add the first
 * min(P_in,P_out) degrees directly (solidfmm/translations.cpp:540-547).
 *
 * Errors never cross the ABI as exceptions: every function returns an
 * sfmm_status; sfmm_last_error() describes the last failure on a context.
 */
#ifndef SFMM_H
#define SFMM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SFMM_OK = 0,
    SFMM_INVALID_ARG = 1,   /* std::logic_error in the reference (e.g. P == 0, incompatible buffer) */
    SFMM_ORDER_RANGE = 2,   /* std::out_of_range: an order exceeds the operator order */
    SFMM_OVERFLOW = 3,      /* std::overflow_error: order too large for the floating-point type */
    SFMM_DIM_MISMATCH = 4,  /* std::logic_error: source and target dimensions differ */
    SFMM_OOM = 5,           /* std::bad_alloc */
    SFMM_CUDA_ERROR = 6,    /* CUDA runtime failure (no device, launch failure, ...) */
    SFMM_UNSUPPORTED = 7    /* precision mode not available for this data type */
} sfmm_status;

typedef enum { SFMM_F32 = 0, SFMM_F64 = 1 } sfmm_dtype;
typedef enum { SFMM_M2M = 0, SFMM_M2L = 1, SFMM_L2L = 2 } sfmm_op;

/* Arithmetic of the translation kernels.
 * PLAIN:    the storage type's own arithmetic (FP64 for SFMM_F64, FP32 for
 *           SFMM_F32).
 * SPLIT:    FP64 expansions in, FP64 accumulation out, the translation itself
 *           on the FP32 and integer pipes with relative error <= 1e-7 in the
 *           orthonormal (Schmidt) basis: swaps and polar rotations in block
 *           fixed point (int32 mantissas with one exponent per degree row,
 *           Q1.30 coefficients, exact int64 accumulation), the azimuthal
 *           rotations, r-power scaling and z-translation in float-float.
 *           M2M batches with an order bound above 18 run the SPLIT_FF
 *           arithmetic: there the rotation method's error growth with the
 *           degree would take 30-bit mantissas past 1e-7.
 * SPLIT_FF: the same with float-float (double-FP32, ~2^-44 per operation)
 *           for every stage: relative error ~1e-13 at order 16.
 * TC_TF32:  the tensor-core kernel (tcgen05, one thread per translation,
 *           128 translations per MMA tile): every swap and z-translation is
 *           an MMA against constant matrices held in shared memory, with both
 *           operands split in two TF32 pieces (hi*hi + hi*lo + lo*hi, FP32
 *           accumulation in tensor memory); FP64 geometry, FP32 rotations
 *           and scaling, FP64 accumulation into the targets.  FP32-class
 *           error (~1e-7 orthonormal).  Order bounds up to 16; batches with
 *           a larger order bound run SFMM_SPLIT.
 * TC_BF16:  the same kernel with BF16 pieces (kind::f16): ~16-bit operand
 *           precision, error ~1e-5.
 * TC_BF16X6: the same kernel with three BF16 pieces per operand (the six
 *           products whose piece indices sum to at most 2, smallest first)
 *           and float-float edge scaling: each MMA stage rounds about once
 *           in FP32.
 * The split and tensor-core modes need an SFMM_F64 context and orders <= 28
 * (FP32 exponent range of the orthogonal-basis scale factors).  They, and
 * PLAIN on an SFMM_F32 context, run every translation at the length scale
 * of its own shift (sources and results rescaled by exact powers of two in
 * the FP64 <-> FP32 conversions), so their error does not depend on the
 * geometry's length scale; an SFMM_F32 context can only hold coefficients
 * inside the FP32 range. */
typedef enum {
    SFMM_PLAIN = 0,
    SFMM_SPLIT = 1,
    SFMM_SPLIT_FF = 2,
    SFMM_TC_TF32 = 3,
    SFMM_TC_BF16 = 4,
    SFMM_TC_BF16X6 = 5
} sfmm_precision;

/* flags for the batch calls */
enum {
    SFMM_TARGETS_UNIQUE = 0,   /* no two translations of the batch share a target */
    SFMM_TARGETS_REPEAT = 1,   /* targets may repeat: accumulate with atomics */
    SFMM_TARGETS_ON_DEVICE = 2 /* sfmm_translate_host_packed: dst is device memory (see there) */
};

typedef struct sfmm_context sfmm_context;

/* Operator context of order P (the reference's operator_data<real>(P),
 * solidfmm/operator_data.cpp:151-244): builds the rotation/swap/z-translation
 * tables in FP64 on the host and uploads them to `device`.
 * P == 0 -> SFMM_INVALID_ARG; P > 86 (F64) -> SFMM_OVERFLOW (the reference's
 * limit, operator_data.cpp:37-45,157-164).  F32 contexts go up to P = 28
 * (the reference's float limit is 18 because it keeps factorials in FP32;
 * these kernels keep them in FP64 and in the orthogonal basis, so orders up
 * to 28 stay in range); the C++ drop-in operator_data<float> keeps the
 * reference's limit of 18. */
int sfmm_create(sfmm_context **ctx, int dtype, size_t P, int device);
void sfmm_destroy(sfmm_context *ctx);
size_t sfmm_order(const sfmm_context *ctx);
int sfmm_data_type(const sfmm_context *ctx);
const char *sfmm_last_error(const sfmm_context *ctx);
const char *sfmm_status_string(int status);

/* All kernels of the context are launched on this CUDA stream (cudaStream_t
 * passed as void*; NULL = the legacy default stream). */
int sfmm_set_stream(sfmm_context *ctx, void *stream);

/* Device-resident batch (all pointers are device pointers; replaces the
 * lane queues of solidfmm/translations.cpp:474-630 and the worker loop of
 * solidfmm/multithreaded_translator.cpp:261-330).  Translation i:
 *   dst[dst_index[i]] += T_op(src[src_index[i]], shift[3i..3i+2])
 * with orders p_in[i], p_out[i] <= order_bound (0 = the context order).
 * src_index/dst_index NULL mean i; src_count/dst_count are the numbers of
 * expansions addressable through src/dst.  `order` (may be NULL) is a
 * permutation giving the processing order (see sfmm_bucket_by_order).
 * Shifts are FP64 for both data types.  Asynchronous on the context's stream.
 * Entries with an index or order out of range are skipped and flagged in the
 * context's device status word (sfmm_device_status); they never touch memory
 * out of bounds.  Targets must not alias sources. */
int sfmm_translate_device(sfmm_context *ctx, int op, int precision, size_t n,
                          const void *src, size_t src_stride, size_t src_count, const uint32_t *src_index,
                          void *dst, size_t dst_stride, size_t dst_count, const uint32_t *dst_index,
                          const uint32_t *p_in, const uint32_t *p_out, const double *shift,
                          const uint32_t *order, int flags, size_t order_bound);

/* Synchronise the context's stream and return (and clear) its device status
 * word: 0 = every translation since the last call was well formed, bit 0 =
 * some entry had an out-of-range index or order and was skipped. */
int sfmm_device_status(sfmm_context *ctx, int *flags);

/* Contiguous host batch, the bulk form of the classic call: src/dst are HOST
 * arrays of src_count/dst_count expansions with the given strides (pinned
 * memory gives full copy bandwidth), orders/indices/shifts are host arrays as
 * in sfmm_translate_device.  Copies in, translates, copies the updated
 * targets back and synchronises before returning.  Batches without index
 * arrays are pipelined in chunks over three streams so that host-to-device
 * copies, kernels and device-to-host copies overlap.
 * With SFMM_TARGETS_ON_DEVICE in flags, dst (dst_count expansions at
 * dst_stride) is device memory that keeps the results across calls: the
 * kernel reads the host sources where they lie (they must be
 * device-accessible: pinned, or any host memory on a GPU that walks the host
 * page tables, else SFMM_UNSUPPORTED) and accumulates into the device
 * targets (atomics with SFMM_TARGETS_REPEAT), so the host link carries the
 * sources and the batch metadata only -- 2.2 KB per translation at P=16
 * instead of 6.5 KB.  Synchronises before returning. */
int sfmm_translate_host_packed(sfmm_context *ctx, int op, int precision, size_t n,
                               const void *src, size_t src_stride, size_t src_count, const uint32_t *src_index,
                               void *dst, size_t dst_stride, size_t dst_count, const uint32_t *dst_index,
                               const uint32_t *p_in, const uint32_t *p_out, const double *shift, int flags);

/* Host drop-in batch: the classic solidfmm::m2l/m2m/l2l(op, buf, howmany,
 * M**, L**, x, y, z) call (solidfmm/translations.hpp:103-109).  src[i] and
 * dst[i] point at host expansions (in the solid layout, dim components of
 * P(P+1) reals each); x/y/z are arrays of the context's real type.  Orders
 * are checked first (strong guarantee: on error nothing is modified); the
 * call gathers the expansions to the GPU, runs the batch, and scatter-adds
 * the results into the host targets before returning. */
int sfmm_translate_host(sfmm_context *ctx, int op, int precision, size_t n,
                        const void *const *src, const size_t *p_in,
                        void *const *dst, const size_t *p_out, size_t dim,
                        const void *x, const void *y, const void *z);

/* Minimal bounding sphere on the host (the reference's bounding_sphere,
 * solidfmm/sphere.hpp:38-42): the smallest sphere containing n points
 * (r NULL) or n spheres of radii r[i]; out = {x, y, z, radius}.  n == 0 ->
 * SFMM_INVALID_ARG; a degenerate configuration that floating point cannot
 * resolve -> SFMM_UNSUPPORTED (the reference throws std::runtime_error). */
int sfmm_bounding_sphere(size_t n, const double *x, const double *y, const double *z, const double *r,
                         double *out);

/* Launch shape.  The translation kernels run G threads per translation: 4
 * or 8 for order bounds up to 32, one warp (32) above.  By default a context
 * takes G per (precision, order bound) from a built-in table measured on
 * GB300; sfmm_set_group pins G for one (precision, order bound) pair, and
 * sfmm_tune times every supported G, each with the largest and the smallest
 * tile (translations per CTA) that keep the SM fully occupied, on n synthetic
 * translations of `op` on the context's stream (synchronising it) and keeps
 * the fastest for that (op, precision, order bound).  `group`
 * (may be NULL) receives the kept G, `rate` (may be NULL) its measured
 * translations per second.  order_bound 0 = the context order. */
int sfmm_set_group(sfmm_context *ctx, int precision, size_t order_bound, int group);
int sfmm_tune(sfmm_context *ctx, int op, int precision, size_t order_bound, size_t n, int *group,
              double *rate);

/* Execution plans.  A plan is an ordered list of device batches (stages)
 * that runs many times with the same orders and indices: one FMM pass, a
 * mixed-order workload.  sfmm_plan_finalize reads each stage's orders,
 * sorts its translations by order bound max(p_in, p_out) (then by the
 * pair), splits the sorted stage into segments of one order bound, and
 * records one kernel launch per segment into a CUDA graph; the segments of a
 * stage run on concurrent graph branches, the stages in order (a stage sees
 * the results of the ones before it).  sfmm_plan_run replays the graph on
 * the context's stream (asynchronous).  The stage arrays are device
 * pointers that must stay valid, with unchanged orders and indices, while
 * the plan exists; expansions and shifts may change between runs.  Because
 * the segments of a stage run concurrently, a stage whose targets repeat
 * must pass SFMM_TARGETS_REPEAT.  sfmm_plan_segments reports the segments
 * (order bound and size, all stages in order; returns their number). */
typedef struct sfmm_plan sfmm_plan;
int sfmm_plan_create(sfmm_context *ctx, sfmm_plan **plan);
/* Plan options (before sfmm_plan_finalize; flags may be combined):
 * SFMM_PLAN_FUSED  each stage runs as one persistent launch over all its
 *                  orders: the grid fills the GPU once and its CTAs take
 *                  tiles of the order-sorted stage from a device work list
 *                  (largest orders first) until it is empty, with the launch
 *                  shape of the stage's largest order bound.  Stages in a
 *                  tensor-core precision keep one launch per segment.
 * SFMM_PLAN_TUNE   finalize measures launch shapes and launches with the
 *                  fastest: a fused stage's on a synthetic batch with the
 *                  stage's own order distribution (a sample of up to 65 536
 *                  of its translations; the shape stays with the plan), each
 *                  segment's on the segment itself (its sources, indices,
 *                  orders and shifts, writing into a scratch copy of its
 *                  target array, so the plan's targets stay untouched; with
 *                  sfmm_tune's synthetic batch instead when that copy would
 *                  take more than a quarter of the free device memory), for
 *                  every (operator, precision, order bound) the context has
 *                  not measured yet (the shape stays with the context).
 * Default 0: one launch per segment, built-in shapes. */
enum { SFMM_PLAN_FUSED = 1, SFMM_PLAN_TUNE = 2 };
int sfmm_plan_set_options(sfmm_plan *plan, int options);
int sfmm_plan_add(sfmm_plan *plan, int op, int precision, size_t n,
                  const void *src, size_t src_stride, size_t src_count, const uint32_t *src_index,
                  void *dst, size_t dst_stride, size_t dst_count, const uint32_t *dst_index,
                  const uint32_t *p_in, const uint32_t *p_out, const double *shift, int flags);
int sfmm_plan_finalize(sfmm_plan *plan);
int sfmm_plan_run(sfmm_plan *plan);
size_t sfmm_plan_launches(const sfmm_plan *plan);
size_t sfmm_plan_segments(const sfmm_plan *plan, int *bounds, size_t *counts, size_t cap);
void sfmm_plan_destroy(sfmm_plan *plan);

/* Bucket a device batch by (p_in, p_out): writes a permutation of 0..n-1 into
 * `order` (device, n entries) so that translations of equal order pairs are
 * contiguous.  Orders above the context order are counted with the context
 * order (no error: the translation kernels flag such entries).  n above
 * 2^32 - 1 -> SFMM_INVALID_ARG.  Uses ctx scratch; asynchronous. */
int sfmm_bucket_by_order(sfmm_context *ctx, size_t n, const uint32_t *p_in, const uint32_t *p_out,
                         uint32_t *order);

/* Bucketing without any allocation (no counterpart in the reference; the
 * reference has no GPU and allocates its buffers on the host).  For callers
 * that cannot allocate device memory -- codes that give the whole GPU to their
 * own memory pool, processes under a hard device-memory cap, or hot paths
 * where an allocation would stall -- and so cannot create a context either.
 * Same result as sfmm_bucket_by_order (a permutation of 0..n-1 in `order`
 * grouping equal (p_in, p_out) pairs; order within a group is unspecified)
 * for orders up to max_order <= 86; larger max_order returns
 * SFMM_ORDER_RANGE and does nothing.  p_in/p_out values above max_order are
 * counted as max_order (no error), so a max_order below the batch's largest
 * order merges those pairs into the top buckets.  Runs in the CUDA context
 * current at the call (the current device's primary context if none is) and
 * on `stream` (cudaStream_t as void*, NULL = default stream),
 * asynchronously.  Its counters live in one fixed 30 KiB device array per
 * GPU that every call shares: concurrent calls whose kernels overlap on the
 * GPU race and must be serialised (e.g. on one stream).  The array's device
 * address is looked up on every call outside a stream capture and kept per
 * context; a call inside a capture uses the address kept for its context,
 * so make one call in that context before capturing (else
 * SFMM_INVALID_ARG).  Calls no cudaMalloc/cudaFree. */
int sfmm_bucket_by_order_noalloc(size_t n, const uint32_t *p_in, const uint32_t *p_out, uint32_t *order,
                                 size_t max_order, void *stream);

/* L2P / M2P on the device: for point j with expansion b = box[j] (box NULL:
 * b = j; nexp expansions addressable at `stride` reals, centres FP64),
 *   potential[j] += dot(E[b], R(pos[j] - centre[b]))    (kind 0, local)
 *   potential[j] += dot(E[b], S(pos[j] - centre[b]))    (kind 1, multipole)
 * with dot the reference's solid dot product (solid.cpp:41-66).  For kind 0
 * a non-NULL gradient (3 per point) receives += grad phi(pos[j]) as well.
 * Orders up to 32 with at least one point per four expansions run in
 * float-float on the FP32 pipe over a normalised copy of all nexp
 * expansions, made once per call in context scratch of about
 * nexp * P(P+1) * 8 bytes (allocated or grown on first need; a call inside a
 * stream capture never allocates, and a call without enough scratch runs
 * FP64); error about 1e-14 of the sum of the terms' magnitudes.  Other calls
 * run in FP64.  Calls on one context share the scratch (serialised by a lock,
 * ordered on the context's stream).  Box indices are not range-checked
 * (device data). */
int sfmm_eval_device(sfmm_context *ctx, int kind, size_t npts, const double *pos, const uint32_t *box,
                     const void *E, size_t stride, size_t nexp, const double *centre, double *potential,
                     double *gradient);

/* P2M / P2L on the device (the reference's fmadd(q, harmonics::R/S(P, x-c), E),
 * solid.cpp:70-104 with harmonics.cpp:32-80,177-224): for expansion j,
 *   out[j] += sum_{k<nq} charge[j*nq+k] * R(pos[j*nq+k] - centre[j])   (kind 0)
 *   out[j] += sum_{k<nq} charge[j*nq+k] * S(pos[j*nq+k] - centre[j])   (kind 1)
 * FP64 arithmetic; out has the context's data type and order P. */
int sfmm_p2x_device(sfmm_context *ctx, int kind, size_t nexp, size_t nq, const double *charge,
                    const double *pos, const double *centre, void *out, size_t out_stride);

/* The same with ragged particle sets (leaves of a tree with their particles
 * sorted by leaf): expansion j takes particles k in [offset[j], offset[j+1])
 * (offset: nexp + 1 non-decreasing device values; not range-checked). */
int sfmm_p2x_ragged_device(sfmm_context *ctx, int kind, size_t nexp, const uint32_t *offset,
                           const double *charge, const double *pos, const double *centre, void *out,
                           size_t out_stride);

/* Diagnostics: measured FMA-pipe throughput (flop/s, 2 per FMA) of the
 * device, FP64 (fp64 = 1) or FP32 (fp64 = 0); the roofline denominator of
 * the plain FP64 and split-precision kernels. */
int sfmm_measure_fma_peak(int fp64, int device, double *flops_per_second);
/* Diagnostics: measured throughput of 32x32->64-bit integer multiply-adds
 * (operations/s, one per multiply-add). */
int sfmm_measure_imad_peak(int device, double *ops_per_second);

/* Diagnostics: the FP64 operator tables of order P as dense row-major
 * arrays.  which: 0/1 = W_R/W_I of degree n (d x d, entry (i,j)); 2/3/4 =
 * z-translation matrix H_m of M2M/M2L/L2L for column m = n ((P-m) x (P-m),
 * entry (n'-m, k-m)); 5..8 = edge factors e_in_M, e_in_L, e_out_L, e_out_M
 * (index n(n+1)/2+m).  Writes min(cap, count) values to out (may be NULL)
 * and the full count to *count.  Host only, needs no GPU. */
int sfmm_host_table(size_t P, int which, int n, double *out, size_t cap, size_t *count);

/* Number of kernel launches issued by this context since creation. */
uint64_t sfmm_launch_count(const sfmm_context *ctx);

#ifdef __cplusplus
}
#endif
#endif
