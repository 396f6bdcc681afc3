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
#include <cmath>
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
    // fused mode: one launch at the stage's largest bound over a work list
    bool fused = false;
    int fused_bound = 0;
    size_t work_off = 0, nwork = 0;
    LaunchShape shape;  // fused launch shape (tuned on the stage's own orders, else the context's)
    std::vector<uint32_t> spin, spout;  // tuning sample of the stage's orders, sorted by bound
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
    int options = 0;
    uint2 *d_work = nullptr;        // work lists of the fused stages
    unsigned *d_counters = nullptr; // one tile counter per stage
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
    if (p->d_work) cudaFree(p->d_work);
    if (p->d_counters) cudaFree(p->d_counters);
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
    for (size_t k = 0; k < p->stages.size(); ++k) {
        const Stage &s = p->stages[k];
        if (s.segs.empty()) continue;
        const uint32_t *perm = p->d_perm + s.perm_off;
        if (s.fused) {  // reset the stage's tile counter, one persistent launch
            WorkList wl;
            wl.work = p->d_work + s.work_off;
            wl.counter = p->d_counters + k;
            wl.n = (long long)s.nwork;
            if (cudaMemsetAsync(wl.counter, 0, sizeof(unsigned), p->cap) != cudaSuccess)
                return fail(c, SFMM_CUDA_ERROR, "plan capture: work counter reset");
            int st = run_batch(c, p->cap, s.op, s.a, s.fused_bound, (long long)s.n, s.src, (long long)s.sstride,
                               (long long)s.scount, s.sidx, s.dst, (long long)s.dstride, (long long)s.dcount, s.tidx,
                               s.pin, s.pout, s.shift, perm, s.flags, (long long)s.n, nullptr, nullptr, true, &wl,
                               &s.shape);
            if (st) return st;
            p->launches++;
            continue;
        }
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

// A segment's launch shape measured on the segment itself: its sources,
// index arrays, orders and shifts and its stage's atomic mode, written into a
// scratch copy of the target array (the plan's targets stay untouched).
// Every candidate shape (each group size with its largest and smallest
// full-occupancy tile, among CTAs of four warps or more and among all) runs
// once to warm up and once timed.  *done stays false when the scratch
// targets would take more than a quarter of the free device memory or
// cannot be allocated: the caller then measures on synthetic data.
int tune_segment(sfmm_context *c, const sfmm_plan *p, const Stage &s, const Segment &g, bool *done)
{
    *done = false;
    const Arith a = resolve_arith(s.a, s.op, g.bound);
    const size_t bytes = s.dcount * s.dstride * (c->dtype == SFMM_F64 ? 8 : 4);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        (void)cudaGetLastError();
        return SFMM_OK;
    }
    if (bytes == 0 || bytes > free_b / 4) return SFMM_OK;
    void *dst = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaMalloc(&dst, bytes) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
        (void)cudaGetLastError();
        if (dst) cudaFree(dst);
        if (e0) cudaEventDestroy(e0);
        return SFMM_OK;
    }
    const uint32_t *perm = p->d_perm + s.perm_off + g.off;
    const auto key = std::make_tuple(s.op, (int)a, g.bound);
    LaunchShape cands[12], best;
    int ncand = 0;
    for (int G : {4, 8, 32})
        for (int min_threads : {128, 32})
            for (bool small : {false, true}) {
                const LaunchShape sh = best_shape(a, g.bound, G, small, min_threads);
                bool seen = !sh.acc;
                for (int k = 0; k < ncand && !seen; ++k) seen = cands[k].G == sh.G && cands[k].TS == sh.TS;
                if (!seen) cands[ncand++] = sh;
            }
    float best_ms = 0;
    int st = SFMM_OK;
    cudaError_t e = cudaMemsetAsync(dst, 0, bytes, c->stream);
    for (int ci = 0; ci < ncand && st == SFMM_OK && e == cudaSuccess; ++ci) {
        set_shape(c, key, &cands[ci]);
        for (int rep = 0; rep < 2 && st == SFMM_OK && e == cudaSuccess; ++rep) {
            if (rep == 1) e = cudaEventRecord(e0, c->stream);
            st = run_batch(c, c->stream, s.op, s.a, g.bound, (long long)g.cnt, s.src, (long long)s.sstride,
                           (long long)s.scount, s.sidx, dst, (long long)s.dstride, (long long)s.dcount, s.tidx,
                           s.pin, s.pout, s.shift, perm, s.flags, (long long)s.n);
            if (rep == 1 && e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
        }
        float ms = 0;
        if (st == SFMM_OK && e == cudaSuccess && (e = cudaEventSynchronize(e1)) == cudaSuccess)
            e = cudaEventElapsedTime(&ms, e0, e1);
        if (st == SFMM_OK && e == cudaSuccess && (!best.acc || ms < best_ms)) {
            best = cands[ci];
            best_ms = ms;
        }
    }
    cudaFree(dst);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    set_shape(c, key, best.acc ? &best : nullptr);
    if (st != SFMM_OK) return st;
    if (e != cudaSuccess) return cuda_fail(c, e, "plan: tuning a segment");
    if (best.acc) {
        std::lock_guard<std::mutex> lk(c->setup_mtx);
        c->tuned.insert(std::make_tuple(s.op, (int)a, g.bound));
        *done = true;
    }
    return SFMM_OK;
}

// Tiles of TS translations over order-sorted segments, largest order bound
// first.
void build_work(const std::vector<Segment> &segs, int TS, std::vector<uint2> &work)
{
    std::vector<const Segment *> order;
    for (const Segment &g : segs) order.push_back(&g);
    std::sort(order.begin(), order.end(), [](const Segment *x, const Segment *y) { return x->bound > y->bound; });
    for (const Segment *g : order)
        for (size_t o = 0; o < g->cnt; o += (size_t)TS)
            work.push_back(make_uint2((unsigned)(g->off + o), (unsigned)std::min<size_t>(TS, g->cnt - o)));
}

// The fused stage's launch shape measured on a synthetic batch with the
// stage's own order distribution (its sample of orders, sorted by bound):
// every group size with the largest and the smallest full-occupancy tile,
// each timed as one work-list launch (one warm-up, three timed).
int tune_fused(sfmm_context *c, Stage &s)
{
    const Arith a = resolve_arith(s.a, s.op, s.fused_bound);
    const size_t n = s.spin.size();
    const int Pb = s.fused_bound;
    const size_t S = (size_t)Pb * (Pb + 1);
    std::vector<Segment> segs;
    for (size_t k = 0, k0 = 0; k < n; ++k) {
        const int b = (int)std::max(std::max(s.spin[k], s.spout[k]), 1u);
        const bool last = k + 1 == n || (int)std::max(std::max(s.spin[k + 1], s.spout[k + 1]), 1u) != b;
        if (last) {
            segs.push_back(Segment{b, k0, k + 1 - k0});
            k0 = k + 1;
        }
    }
    std::vector<double> sh(3 * n);
    for (size_t i = 0; i < n; ++i) {  // shifts of length 2.5 in varied directions
        const double t = 0.7 * (double)i, u = 0.3 + 2.4 * (double)(i % 97) / 97.0;
        sh[3 * i] = 2.5 * std::sin(u) * std::cos(t);
        sh[3 * i + 1] = 2.5 * std::sin(u) * std::sin(t);
        sh[3 * i + 2] = 2.5 * std::cos(u);
    }
    const size_t es = c->dtype == SFMM_F64 ? 8 : 4;
    void *src = nullptr, *dst = nullptr, *meta = nullptr, *wk = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&] {
        for (void *q : {src, dst, meta, wk})
            if (q) cudaFree(q);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    const size_t nw_max = n + segs.size() + 1;  // tiles of at least one translation
    cudaError_t e;
    if ((e = cudaMalloc(&src, n * S * es)) != cudaSuccess || (e = cudaMalloc(&dst, n * S * es)) != cudaSuccess ||
        (e = cudaMalloc(&meta, n * (2 * sizeof(uint32_t) + 3 * sizeof(double)) + sizeof(unsigned))) != cudaSuccess ||
        (e = cudaMalloc(&wk, nw_max * sizeof(uint2))) != cudaSuccess) {
        cleanup();
        return fail(c, SFMM_OOM, "plan tuning buffers");
    }
    double *d_sh = static_cast<double *>(meta);
    uint32_t *d_pin = reinterpret_cast<uint32_t *>(d_sh + 3 * n), *d_pout = d_pin + n;
    unsigned *d_cnt = reinterpret_cast<unsigned *>(d_pout + n);
    cudaStream_t st = c->stream;
    if ((e = cudaMemsetAsync(src, 0x3e, n * S * es, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(dst, 0, n * S * es, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_sh, sh.data(), 3 * n * sizeof(double), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_pin, s.spin.data(), n * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_pout, s.spout.data(), n * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess) {
        cleanup();
        return cuda_fail(c, e, "plan tuning setup");
    }
    LaunchShape best;
    float best_ms = 0;
    std::vector<LaunchShape> cands;
    for (int G : {4, 8, 32})
        for (int min_threads : {128, 32})
            for (bool small : {false, true}) {
                const LaunchShape cs = best_shape(a, Pb, G, small, min_threads);
                bool seen = !cs.acc;
                for (const LaunchShape &k : cands) seen = seen || (k.G == cs.G && k.TS == cs.TS);
                if (!seen) cands.push_back(cs);
            }
    int rc = SFMM_OK;
    for (const LaunchShape &cs : cands) {
        std::vector<uint2> work;
        build_work(segs, cs.TS, work);
        WorkList wl;
        wl.work = static_cast<const uint2 *>(wk);
        wl.counter = d_cnt;
        wl.n = (long long)work.size();
        if ((e = cudaMemcpyAsync(wk, work.data(), work.size() * sizeof(uint2), cudaMemcpyHostToDevice, st)) !=
            cudaSuccess) {
            rc = cuda_fail(c, e, "plan tuning work list");
            break;
        }
        float ms = 0;
        for (int rep = 0; rep < 4 && rc == SFMM_OK; ++rep) {
            if (rep == 1 && (e = cudaEventRecord(e0, st)) != cudaSuccess) break;
            if ((e = cudaMemsetAsync(d_cnt, 0, sizeof(unsigned), st)) != cudaSuccess) break;
            rc = run_batch(c, st, s.op, s.a, Pb, (long long)n, src, (long long)S, (long long)n, nullptr, dst,
                           (long long)S, (long long)n, nullptr, d_pin, d_pout, d_sh, nullptr, 0, (long long)n,
                           nullptr, nullptr, true, &wl, &cs);
        }
        if (rc == SFMM_OK && e == cudaSuccess && (e = cudaEventRecord(e1, st)) == cudaSuccess &&
            (e = cudaEventSynchronize(e1)) == cudaSuccess)
            e = cudaEventElapsedTime(&ms, e0, e1);
        if (rc != SFMM_OK) break;
        if (e != cudaSuccess) {
            rc = cuda_fail(c, e, "plan tuning run");
            break;
        }
        if (!best.acc || ms < best_ms) {
            best = cs;
            best_ms = ms;
        }
    }
    cleanup();
    if (rc != SFMM_OK) return rc;
    if (best.acc) s.shape = best;
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
            s.spin.clear();
            s.spout.clear();
            if ((p->options & SFMM_PLAN_FUSED) && (p->options & SFMM_PLAN_TUNE)) {  // tuning sample, in order
                const size_t ns = std::min<size_t>(s.n, 65536);
                for (size_t k = 0; k < ns; ++k) {
                    const uint32_t i = (uint32_t)key[k * s.n / ns];
                    s.spin.push_back(pin[i]);
                    s.spout.push_back(pout[i]);
                }
            }
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
    // 2. fused stages (not in a tensor-core precision): one launch at the
    //    stage's largest bound
    for (Stage &s : p->stages) {
        s.fused = false;
        if (!(p->options & SFMM_PLAN_FUSED) || s.segs.empty() || is_tc(s.a)) continue;
        s.fused = true;
        for (const Segment &g : s.segs) s.fused_bound = std::max(s.fused_bound, g.bound);
    }
    // 3. measured launch shapes (optional), then tables and launch shapes
    //    before the capture (no allocation inside it)
    for (Stage &s : p->stages) {
        s.shape = LaunchShape{};
        if (s.fused && (p->options & SFMM_PLAN_TUNE) && !s.spin.empty()) {
            int st = tune_fused(c, s);
            if (st) return st;
        }
    }
    if (p->options & SFMM_PLAN_TUNE)
        for (const Stage &s : p->stages)
            for (const Segment &g : s.segs) {
                if (s.fused) break;  // measured on its own orders above
                const int bound = s.fused ? s.fused_bound : g.bound;
                if (is_tc(resolve_arith(s.a, s.op, bound))) continue;  // one shape: nothing to choose
                const auto key = std::make_tuple(s.op, (int)resolve_arith(s.a, s.op, bound), bound);
                bool have;
                {
                    std::lock_guard<std::mutex> lk(c->setup_mtx);
                    have = c->tuned.count(key) != 0;
                }
                if (have) continue;
                bool done = false;
                int st = tune_segment(c, p, s, g, &done);
                if (st) return st;
                if (done) continue;
                const size_t cnt = s.fused ? s.n : g.cnt;  // too large a target array: synthetic data
                st = sfmm_tune(c, s.op, s.precision, (size_t)bound,
                               std::min<size_t>(std::max<size_t>(cnt, 4096), 65536), nullptr, nullptr);
                if (st) return st;
            }
    std::vector<uint2> work;
    for (Stage &s : p->stages) {
        if (s.fused) {
            LaunchShape sh;
            int st = prepare_launch(c, s.op, s.a, s.fused_bound, &sh);
            if (st) return st;
            if (!s.shape.acc) s.shape = sh;  // not tuned on the stage: the context's shape
            s.work_off = work.size();
            try {
                build_work(s.segs, s.shape.TS, work);
            } catch (const std::bad_alloc &) {
                return fail(c, SFMM_OOM, "plan work list");
            }
            s.nwork = work.size() - s.work_off;
            continue;
        }
        for (const Segment &g : s.segs) {
            int st = prepare_launch(c, s.op, s.a, g.bound);
            if (st) return st;
        }
    }
    if (p->d_work) {
        cudaFree(p->d_work);
        p->d_work = nullptr;
    }
    if (p->d_counters) {
        cudaFree(p->d_counters);
        p->d_counters = nullptr;
    }
    if (!work.empty()) {
        if (cudaMalloc(&p->d_work, work.size() * sizeof(uint2)) != cudaSuccess ||
            cudaMalloc(&p->d_counters, p->stages.size() * sizeof(unsigned)) != cudaSuccess)
            return fail(c, SFMM_OOM, "plan work list");
        if (cudaMemcpy(p->d_work, work.data(), work.size() * sizeof(uint2), cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(c, SFMM_CUDA_ERROR, "plan work list upload");
    }
    // 4. capture
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

int sfmm_plan_set_options(sfmm_plan *p, int options)
{
    if (!p) return SFMM_INVALID_ARG;
    if (p->finalized) return fail(p->ctx, SFMM_INVALID_ARG, "plan already finalized");
    if (options & ~(SFMM_PLAN_FUSED | SFMM_PLAN_TUNE)) return fail(p->ctx, SFMM_INVALID_ARG, "unknown plan option");
    p->options = options;
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
