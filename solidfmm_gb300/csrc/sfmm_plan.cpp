// Execution plans (include/sfmm.h, sfmm_plan_*): ordered stages of device
// batches, each sorted by order and split into segments of one order bound,
// recorded once into a CUDA graph and replayed.
//
// The reference runs such workloads as lane queues that pad every lane of a
// batch to the largest order in it (translations.cpp:474-630) on threads
// that each own a target partition (multithreaded_translator.cpp:261-330).
// Here the sort puts translations of equal order bound side by side, so each
// segment's kernel is launched with the shared-memory footprint and group
// size of its own order, and the segments of a stage run concurrently on
// forked graph branches so that small segments share the GPU.
#include "sfmm.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <new>
#include <vector>

#include "sfmm_context.hpp"
#include "sfmm_launch.hpp"

using namespace sfmm;

namespace {

constexpr int kBranches = 4;  // concurrent graph branches per stage

struct Segment {
    int bound;
    size_t off, cnt;
};

struct Stage {
    int op, precision;
    Arith a;
    size_t n;
    const void *src;
    size_t sstride, scount;
    const uint32_t *sidx;
    void *dst;
    size_t dstride, dcount;
    const uint32_t *tidx;
    const uint32_t *pin, *pout;
    const double *shift;
    int flags;
    size_t perm_off = 0;
    std::vector<Segment> segs;
};

}  // namespace

struct sfmm_plan {
    sfmm_context *ctx = nullptr;
    std::vector<Stage> stages;
    uint32_t *d_perm = nullptr;
    cudaStream_t cap = nullptr;
    cudaStream_t side[kBranches] = {};
    std::vector<cudaEvent_t> events;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    size_t launches = 0;
    bool finalized = false;
};

namespace {

void release(sfmm_plan *p)
{
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    for (cudaEvent_t e : p->events) cudaEventDestroy(e);
    for (cudaStream_t s : p->side)
        if (s) cudaStreamDestroy(s);
    if (p->cap) cudaStreamDestroy(p->cap);
    if (p->d_perm) cudaFree(p->d_perm);
}

cudaEvent_t new_event(sfmm_plan *p)
{
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
    p->events.push_back(e);
    return e;
}

// Records every stage's launches on the capture stream (and forked side
// streams); returns a status, leaving the capture open for the caller to end.
int record(sfmm_plan *p)
{
    sfmm_context *c = p->ctx;
    for (const Stage &s : p->stages) {
        if (s.segs.empty()) continue;
        const uint32_t *perm = p->d_perm + s.perm_off;
        if (s.segs.size() == 1) {
            const Segment &g = s.segs[0];
            int st = run_batch(c, p->cap, s.op, s.a, g.bound, (long long)g.cnt, s.src, (long long)s.sstride,
                               (long long)s.scount, s.sidx, s.dst, (long long)s.dstride, (long long)s.dcount, s.tidx,
                               s.pin, s.pout, s.shift, perm + g.off, s.flags, (long long)s.n);
            if (st) return st;
            p->launches++;
            continue;
        }
        cudaEvent_t fork = new_event(p);
        if (!fork || cudaEventRecord(fork, p->cap) != cudaSuccess)
            return fail(c, SFMM_CUDA_ERROR, "plan capture: fork event");
        const int nb = (int)std::min<size_t>(kBranches, s.segs.size());
        for (int b = 0; b < nb; ++b)
            if (cudaStreamWaitEvent(p->side[b], fork, 0) != cudaSuccess)
                return fail(c, SFMM_CUDA_ERROR, "plan capture: fork");
        // largest segments first, dealt round-robin to the branches
        std::vector<size_t> order(s.segs.size());
        for (size_t k = 0; k < order.size(); ++k) order[k] = k;
        std::sort(order.begin(), order.end(), [&](size_t x, size_t y) {
            return (size_t)s.segs[x].bound * s.segs[x].bound * s.segs[x].cnt >
                   (size_t)s.segs[y].bound * s.segs[y].bound * s.segs[y].cnt;
        });
        for (size_t k = 0; k < order.size(); ++k) {
            const Segment &g = s.segs[order[k]];
            int st = run_batch(c, p->side[k % nb], s.op, s.a, g.bound, (long long)g.cnt, s.src,
                               (long long)s.sstride, (long long)s.scount, s.sidx, s.dst, (long long)s.dstride,
                               (long long)s.dcount, s.tidx, s.pin, s.pout, s.shift, perm + g.off, s.flags,
                               (long long)s.n);
            if (st) return st;
            p->launches++;
        }
        for (int b = 0; b < nb; ++b) {
            cudaEvent_t join = new_event(p);
            if (!join || cudaEventRecord(join, p->side[b]) != cudaSuccess ||
                cudaStreamWaitEvent(p->cap, join, 0) != cudaSuccess)
                return fail(c, SFMM_CUDA_ERROR, "plan capture: join");
        }
    }
    return SFMM_OK;
}

}  // namespace

extern "C" {

int sfmm_plan_create(sfmm_context *c, sfmm_plan **out)
{
    if (!c || !out) return SFMM_INVALID_ARG;
    *out = nullptr;
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, SFMM_CUDA_ERROR, "cannot select device %d", c->device);
    sfmm_plan *p = new (std::nothrow) sfmm_plan;
    if (!p) return fail(c, SFMM_OOM, "plan");
    p->ctx = c;
    bool ok = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking) == cudaSuccess;
    for (int b = 0; b < kBranches && ok; ++b)
        ok = cudaStreamCreateWithFlags(&p->side[b], cudaStreamNonBlocking) == cudaSuccess;
    if (!ok) {
        release(p);
        delete p;
        return fail(c, SFMM_CUDA_ERROR, "plan streams");
    }
    *out = p;
    return SFMM_OK;
}

int sfmm_plan_add(sfmm_plan *p, int op, int precision, size_t n, const void *src, size_t src_stride,
                  size_t src_count, const uint32_t *src_index, void *dst, size_t dst_stride, size_t dst_count,
                  const uint32_t *dst_index, const uint32_t *p_in, const uint32_t *p_out, const double *shift,
                  int flags)
{
    if (!p) return SFMM_INVALID_ARG;
    sfmm_context *c = p->ctx;
    if (p->finalized) return fail(c, SFMM_INVALID_ARG, "plan already finalized");
    if (op < SFMM_M2M || op > SFMM_L2L) return fail(c, SFMM_INVALID_ARG, "unknown operator %d", op);
    Arith a;
    int st = arith_of(c, precision, &a);
    if (st) return st;
    if (n > 0xffffffffull) return fail(c, SFMM_INVALID_ARG, "stage larger than 2^32 translations");
    if (n && (!src || !dst || !p_in || !p_out || !shift)) return fail(c, SFMM_INVALID_ARG, "null device pointer in stage");
    Stage s{};
    s.op = op;
    s.precision = precision;
    s.a = a;
    s.n = n;
    s.src = src;
    s.sstride = src_stride;
    s.scount = src_count;
    s.sidx = src_index;
    s.dst = dst;
    s.dstride = dst_stride;
    s.dcount = dst_count;
    s.tidx = dst_index;
    s.pin = p_in;
    s.pout = p_out;
    s.shift = shift;
    s.flags = flags;
    try {
        p->stages.push_back(s);
    } catch (const std::bad_alloc &) {
        return fail(c, SFMM_OOM, "plan stage");
    }
    return SFMM_OK;
}

int sfmm_plan_finalize(sfmm_plan *p)
{
    if (!p) return SFMM_INVALID_ARG;
    Range range("sfmm plan finalize");
    sfmm_context *c = p->ctx;
    if (p->finalized) return fail(c, SFMM_INVALID_ARG, "plan already finalized");
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, SFMM_CUDA_ERROR, "cannot select device %d", c->device);
    // a failed finalize may be retried (after fixing the stage data): start clean
    p->launches = 0;
    for (Stage &s : p->stages) s.segs.clear();
    if (p->d_perm) {
        cudaFree(p->d_perm);
        p->d_perm = nullptr;
    }
    // 1. sort every stage by (bound, p_in, p_out) on the host
    std::vector<uint32_t> perm;
    try {
        for (Stage &s : p->stages) {
            s.perm_off = perm.size();
            if (!s.n) continue;
            std::vector<uint32_t> pin(s.n), pout(s.n);
            if (cudaMemcpy(pin.data(), s.pin, s.n * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(pout.data(), s.pout, s.n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
                return fail(c, SFMM_CUDA_ERROR, "plan: reading stage orders");
            std::vector<uint64_t> key(s.n);
            int pmax = 0;
            for (size_t i = 0; i < s.n; ++i) {
                if (pin[i] > (uint32_t)c->P || pout[i] > (uint32_t)c->P)
                    return fail(c, SFMM_ORDER_RANGE, "plan: translation %zu has orders (%u,%u) above the operator order %d",
                                i, pin[i], pout[i], c->P);
                const uint64_t b = std::max<uint32_t>(std::max(pin[i], pout[i]), 1u);
                pmax = std::max(pmax, (int)b);
                key[i] = (((b << 8 | pin[i]) << 8 | pout[i]) << 32) | i;
            }
            const size_t need = (size_t)pmax * (pmax + 1);
            if (s.sstride < need || s.dstride < need)
                return fail(c, SFMM_INVALID_ARG, "plan: expansion stride smaller than P(P+1) for order %d", pmax);
            std::sort(key.begin(), key.end());
            size_t k0 = 0;
            for (size_t k = 0; k < s.n; ++k) {
                perm.push_back((uint32_t)key[k]);
                const int b = (int)(key[k] >> 48);
                const bool last = k + 1 == s.n || (int)(key[k + 1] >> 48) != b;
                if (last) {
                    s.segs.push_back(Segment{b, k0, k + 1 - k0});
                    k0 = k + 1;
                }
            }
        }
    } catch (const std::bad_alloc &) {
        return fail(c, SFMM_OOM, "plan sort");
    }
    if (!perm.empty()) {
        if (cudaMalloc(&p->d_perm, perm.size() * 4) != cudaSuccess) return fail(c, SFMM_OOM, "plan permutation");
        if (cudaMemcpy(p->d_perm, perm.data(), perm.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(c, SFMM_CUDA_ERROR, "plan permutation upload");
    }
    // 2. tables and launch shapes before the capture (no allocation inside it)
    for (const Stage &s : p->stages)
        for (const Segment &g : s.segs) {
            int st = prepare_launch(c, s.op, s.a, g.bound);
            if (st) return st;
        }
    // 3. capture
    if (cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return fail(c, SFMM_CUDA_ERROR, "plan: begin capture");
    int st = record(p);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(p->cap, &g);
    if (st) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess || !g) return cuda_fail(c, e, "plan: end capture");
    p->graph = g;
    if ((e = cudaGraphInstantiate(&p->exec, g, 0)) != cudaSuccess) return cuda_fail(c, e, "plan: instantiate");
    p->finalized = true;
    return SFMM_OK;
}

int sfmm_plan_run(sfmm_plan *p)
{
    if (!p) return SFMM_INVALID_ARG;
    Range range("sfmm plan replay");
    sfmm_context *c = p->ctx;
    if (!p->finalized) return fail(c, SFMM_INVALID_ARG, "plan not finalized");
    cudaError_t e = cudaGraphLaunch(p->exec, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "plan: graph launch");
    c->launches += p->launches;
    return SFMM_OK;
}

size_t sfmm_plan_launches(const sfmm_plan *p) { return p ? p->launches : 0; }

size_t sfmm_plan_segments(const sfmm_plan *p, int *bounds, size_t *counts, size_t cap)
{
    if (!p) return 0;
    size_t k = 0;
    for (const Stage &s : p->stages)
        for (const Segment &g : s.segs) {
            if (k < cap) {
                if (bounds) bounds[k] = g.bound;
                if (counts) counts[k] = g.cnt;
            }
            ++k;
        }
    return k;
}

void sfmm_plan_destroy(sfmm_plan *p)
{
    if (!p) return;
    cudaSetDevice(p->ctx->device);
    release(p);
    delete p;
}

}  // extern "C"
