// Context internals shared by the C ABI (sfmm_capi.cpp) and the execution
// plans (sfmm_plan.cpp).  Not part of the public interface.
#pragma once

#include "sfmm.h"

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstdint>
#include <map>
#include <mutex>
#include <set>
#include <tuple>
#include <string>
#include <utility>
#include <vector>

#include "sfmm_hostbatch.hpp"
#include "sfmm_launch.hpp"
#include "sfmm_tables.hpp"

namespace sfmm {

struct DevTables {
    void *W = nullptr, *ein_M = nullptr, *ein_L = nullptr, *eout_L = nullptr, *eout_M = nullptr;
    void *H[3] = {nullptr, nullptr, nullptr};
    void *Wq = nullptr;  // Q1.30 swap matrices (fixed-point variant only)
    void *W8 = nullptr, *Wq8 = nullptr;  // 8-row padded copies (HostTables::W8), contexts above order 32
    bool ready = false;
};

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t b)
    {
        if (b <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, b);
        if (e == cudaSuccess) bytes = b;
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
};

struct HostBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t b)
    {
        if (b <= bytes) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMallocHost(&p, b);
        if (e == cudaSuccess) bytes = b;
        return e;
    }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
};

}  // namespace sfmm

struct sfmm_context {
    int dtype = SFMM_F64;
    int P = 0;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    sfmm::HostTables host;
    sfmm::DevTables tab[sfmm::kNumArith];  // indexed by Arith (the tensor-core modes use tc[])
    sfmm::TcDevTables *tc[3] = {nullptr, nullptr, nullptr};  // tensor-core operand images by format
    std::string err;
    std::atomic<uint64_t> launches{0};
    std::mutex mtx;  // serialises host-path calls (one translator object, one stream)
    std::mutex setup_mtx;  // table uploads and the launch-shape cache (device calls may come from several threads)
    std::mutex eval_mtx;   // the L2P/M2P scratch (d_eval): sized and used by one call at a time
    int *d_status = nullptr;  // device error word of the translation kernels
    // host-path staging (three pipeline slots for the packed host call)
    sfmm::DevBuf d_src[3], d_dst[3], d_meta[3], d_shift[3], d_work;
    sfmm::DevBuf d_eval;  // normalised expansions of the float-float L2P/M2P
    sfmm::HostBuf h_src, h_dst, h_meta, h_shift;
    cudaStream_t pipe[3] = {nullptr, nullptr, nullptr};
    // (op, arith, order bound) -> launch shape: operators tuned apart keep
    // their own shapes at one order
    std::map<std::tuple<int, int, int>, sfmm::LaunchShape> shapes;
    int *d_woff = nullptr, *d_hoff = nullptr;            // table offsets (shared by all arithmetics)
    int *d_woff8 = nullptr;                              // offsets of the 8-row padded swap blocks
    bool pageable_access = false;  // the GPU reads pageable host memory through the host page tables
    sfmm::SlotScratch slot_scratch;  // target table of the classic host call
    std::set<std::tuple<int, int, int>> tuned;  // (op, arith, order bound) shapes measured by sfmm_tune
};

namespace sfmm {

// NVTX range over a scope, shown by profilers on the host timeline (a no-op
// unless a tool is attached)
struct Range {
    explicit Range(const char *name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range &) = delete;
    Range &operator=(const Range &) = delete;
};

// record an error on the context and return the status
int fail(sfmm_context *c, int st, const char *fmt, ...);
int cuda_fail(sfmm_context *c, cudaError_t e, const char *what);
// arithmetic of a precision mode on this context
int arith_of(sfmm_context *c, int precision, Arith *out);
// upload the arithmetic's tables once
int ensure_tables(sfmm_context *c, Arith a);
// the arithmetic a batch of op with this order bound runs in (split M2M above
// order 18 runs float-float; tensor-core modes above order 16 run split)
Arith resolve_arith(Arith a, int op, int Pbound);
// device address of a caller's host array when the kernels can use it
// directly (pinned host memory, or pageable memory on a GPU that uses the host
// page tables), else nullptr
const void *device_view(sfmm_context *c, const void *host);
// tables and launch shape of (arithmetic, order bound) for op, so that a
// launch makes no allocation (plans call this before a graph capture)
int prepare_launch(sfmm_context *c, int op, Arith a, int Pbound, LaunchShape *shape = nullptr);
// replace (or, with nullptr, drop) the cached launch shape of (op, arith, order bound)
void set_shape(sfmm_context *c, std::tuple<int, int, int> key, const LaunchShape *s);
// one validated translation launch on device pointers (translation i of the
// batch is perm[i] when perm is given)
// A work list (work, work_counter, nwork: see KParams) turns the launch into
// one persistent grid that takes its tiles from the list; `shape` (may be
// null) replaces the context's launch shape for this launch.
struct WorkList {
    const uint2 *work = nullptr;
    unsigned *counter = nullptr;
    long long n = 0;
};
int run_batch(sfmm_context *c, cudaStream_t stream, int op, Arith a, int Pbound, long long n, const void *src,
              long long sstride, long long nsrc, const uint32_t *sidx, void *dst, long long dstride, long long ndst,
              const uint32_t *tidx, const uint32_t *pin, const uint32_t *pout, const double *shift,
              const uint32_t *perm, int flags, long long nidx = -1,
              const unsigned long long *src_ptr = nullptr, const unsigned long long *dst_ptr = nullptr,
              bool in_hbm = true, const WorkList *wl = nullptr, const LaunchShape *shape = nullptr);

}  // namespace sfmm
