// Translation batches in host memory: the packed call (contiguous host
// arrays of expansions, sfmm_translate_host_packed) and the classic call over
// arrays of solid addresses (sfmm_translate_host, behind the drop-in
// m2l/m2m/l2l overloads and multithreaded_translator, translations.hpp:103-170).
// Where the GPU can use the caller's memory (pinned, or pageable on a GPU
// that walks the host page tables, as GB300 over NVLink-C2C) the kernel reads
// and updates the host expansions in place; otherwise the batch is staged
// through pinned and device buffers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <exception>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "sfmm.h"
#include "sfmm_context.hpp"
#include "sfmm_hostbatch.hpp"
#include "sfmm_launch.hpp"

using namespace sfmm;

extern "C" {

int sfmm_translate_host_packed(sfmm_context *c, int op, int precision, size_t n, const void *src,
                               size_t src_stride, size_t src_count, const uint32_t *src_index, void *dst,
                               size_t dst_stride, size_t dst_count, const uint32_t *dst_index, const uint32_t *p_in,
                               const uint32_t *p_out, const double *shift, int flags)
{
    if (!c) return SFMM_INVALID_ARG;
    Range range("sfmm host packed call");
    if (op < SFMM_M2M || op > SFMM_L2L) return fail(c, SFMM_INVALID_ARG, "unknown operator %d", op);
    Arith a;
    int st = arith_of(c, precision, &a);
    if (st) return st;
    if (n == 0) return SFMM_OK;
    if (!src || !dst || !p_in || !p_out || !shift) return fail(c, SFMM_INVALID_ARG, "null host pointer in batch");
    // checked call: validate everything before touching the targets
    uint32_t pmax = 1;
    for (size_t i = 0; i < n; ++i) {
        if (p_in[i] > (uint32_t)c->P || p_out[i] > (uint32_t)c->P)
            return fail(c, SFMM_ORDER_RANGE, "translation %zu: orders (%u,%u) exceed the operator order %d", i,
                        p_in[i], p_out[i], c->P);
        pmax = std::max(pmax, std::max(p_in[i], p_out[i]));
        if (src_index && src_index[i] >= src_count) return fail(c, SFMM_INVALID_ARG, "source index out of range");
        if (dst_index && dst_index[i] >= dst_count) return fail(c, SFMM_INVALID_ARG, "target index out of range");
    }
    if (!src_index && src_count < n) return fail(c, SFMM_INVALID_ARG, "fewer sources than translations");
    if (!dst_index && dst_count < n) return fail(c, SFMM_INVALID_ARG, "fewer targets than translations");
    if (src_stride < (size_t)pmax * (pmax + 1) || dst_stride < (size_t)pmax * (pmax + 1))
        return fail(c, SFMM_INVALID_ARG, "expansion stride smaller than P(P+1)");
    std::lock_guard<std::mutex> lock(c->mtx);
    cudaSetDevice(c->device);
    const size_t es = c->dtype == SFMM_F64 ? 8 : 4;
    cudaError_t e;
    for (int k = 0; k < 3; ++k)
        if (!c->pipe[k] && (e = cudaStreamCreateWithFlags(&c->pipe[k], cudaStreamNonBlocking)) != cudaSuccess)
            return cuda_fail(c, e, "stream create");
    if (flags & SFMM_TARGETS_ON_DEVICE) {
        // device-resident targets: the kernel streams the host sources over
        // the link and accumulates in device memory (no target traffic on it)
        const void *vs = device_view(c, src);
        if (!vs) return fail(c, SFMM_UNSUPPORTED, "device targets need device-accessible host sources");
        const size_t nm = n * (2 + (src_index ? 1 : 0) + (dst_index ? 1 : 0));
        if ((e = c->d_meta[0].ensure(nm * sizeof(uint32_t))) != cudaSuccess ||
            (e = c->d_shift[0].ensure(n * 3 * sizeof(double))) != cudaSuccess)
            return cuda_fail(c, e, "device buffers");
        uint32_t *dm = (uint32_t *)c->d_meta[0].p;
        uint32_t *dsi = src_index ? dm + 2 * n : nullptr;
        uint32_t *dti = dst_index ? dm + (src_index ? 3 : 2) * n : nullptr;
        double *dsh = (double *)c->d_shift[0].p;
        cudaStream_t s = c->pipe[0];
        if ((e = cudaMemcpyAsync(dm, p_in, n * 4, cudaMemcpyHostToDevice, s)) ||
            (e = cudaMemcpyAsync(dm + n, p_out, n * 4, cudaMemcpyHostToDevice, s)) ||
            (e = cudaMemcpyAsync(dsh, shift, n * 3 * sizeof(double), cudaMemcpyHostToDevice, s)) ||
            (dsi && (e = cudaMemcpyAsync(dsi, src_index, n * 4, cudaMemcpyHostToDevice, s))) ||
            (dti && (e = cudaMemcpyAsync(dti, dst_index, n * 4, cudaMemcpyHostToDevice, s))))
            return cuda_fail(c, e, "host-to-device copy");
        // the host-memory instance (no L2 prefetch: the sources are on the host)
        st = run_batch(c, s, op, a, (int)pmax, (long long)n, vs, (long long)src_stride, (long long)src_count, dsi,
                       dst, (long long)dst_stride, (long long)dst_count, dti, dm, dm + n, dsh, nullptr,
                       flags & ~SFMM_TARGETS_ON_DEVICE, -1, nullptr, nullptr, false);
        if (st) return st;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(c, e, "synchronise");
        return SFMM_OK;
    }
    const bool pipelined = !src_index && !dst_index;
    // Zero-copy: when the caller's arrays are device-accessible (pinned host
    // memory, or any host memory where the GPU walks the host page tables, as
    // over GB300's NVLink-C2C), the kernel reads the sources and updates the
    // targets in place over the host link.  The link carries the same bytes
    // as the staged copies, but the kernel's reads and writes overlap on it
    // fully (45 vs 37 M translations/s at P=16).  Batches with repeated
    // targets keep their atomics in device memory (staged path).
    if (pipelined && !(flags & SFMM_TARGETS_REPEAT)) {
        const void *vs = device_view(c, src);
        void *vd = const_cast<void *>(device_view(c, dst));
        if (vs && vd) {
            if ((e = c->d_meta[0].ensure(n * 2 * sizeof(uint32_t))) != cudaSuccess ||
                (e = c->d_shift[0].ensure(n * 3 * sizeof(double))) != cudaSuccess)
                return cuda_fail(c, e, "device buffers");
            uint32_t *dm = (uint32_t *)c->d_meta[0].p;
            double *dsh = (double *)c->d_shift[0].p;
            cudaStream_t s = c->pipe[0];
            if ((e = cudaMemcpyAsync(dm, p_in, n * 4, cudaMemcpyHostToDevice, s)) ||
                (e = cudaMemcpyAsync(dm + n, p_out, n * 4, cudaMemcpyHostToDevice, s)) ||
                (e = cudaMemcpyAsync(dsh, shift, n * 3 * sizeof(double), cudaMemcpyHostToDevice, s)))
                return cuda_fail(c, e, "host-to-device copy");
            // the host-memory instance: no L2 prefetch, no unrolled gather
            // (over the link both compete with the demand reads)
            st = run_batch(c, s, op, a, (int)pmax, (long long)n, vs, (long long)src_stride, (long long)src_count,
                           nullptr, vd, (long long)dst_stride, (long long)dst_count, nullptr, dm, dm + n, dsh, nullptr,
                           flags, -1, nullptr, nullptr, false);
            if (st) return st;
            if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(c, e, "synchronise");
            return SFMM_OK;
        }
    }
    // chunk of translations per pipeline step
    size_t chunk = pipelined ? std::max<size_t>(8192, (n + 23) / 24) : n;
    if (chunk > n) chunk = n;
    size_t nchunks = (n + chunk - 1) / chunk;
    size_t sc = pipelined ? chunk : src_count;  // expansions per slot
    size_t dc = pipelined ? chunk : dst_count;
    int slots = pipelined ? (int)std::min<size_t>(3, nchunks) : 1;
    for (int k = 0; k < slots; ++k) {
        if ((e = c->d_src[k].ensure(sc * src_stride * es)) != cudaSuccess) return cuda_fail(c, e, "device buffers");
        if ((e = c->d_dst[k].ensure(dc * dst_stride * es)) != cudaSuccess) return cuda_fail(c, e, "device buffers");
        if ((e = c->d_meta[k].ensure(chunk * 4 * sizeof(uint32_t))) != cudaSuccess) return cuda_fail(c, e, "device buffers");
        if ((e = c->d_shift[k].ensure(chunk * 3 * sizeof(double))) != cudaSuccess) return cuda_fail(c, e, "device buffers");
    }
    const char *hs = (const char *)src;
    char *hd = (char *)dst;
    for (size_t ci = 0; ci < nchunks; ++ci) {
        int k = (int)(ci % slots);
        cudaStream_t s = c->pipe[k];
        size_t b = ci * chunk, m = std::min(chunk, n - b);
        uint32_t *dm = (uint32_t *)c->d_meta[k].p;
        double *dsh = (double *)c->d_shift[k].p;
        size_t ns = pipelined ? m : src_count, nd = pipelined ? m : dst_count;
        const char *srcp = pipelined ? hs + b * src_stride * es : hs;
        char *dstp = pipelined ? hd + b * dst_stride * es : hd;
        if ((e = cudaMemcpyAsync(c->d_src[k].p, srcp, ns * src_stride * es, cudaMemcpyHostToDevice, s)) ||
            (e = cudaMemcpyAsync(c->d_dst[k].p, dstp, nd * dst_stride * es, cudaMemcpyHostToDevice, s)) ||
            (e = cudaMemcpyAsync(dm, p_in + b, m * 4, cudaMemcpyHostToDevice, s)) ||
            (e = cudaMemcpyAsync(dm + chunk, p_out + b, m * 4, cudaMemcpyHostToDevice, s)) ||
            (e = cudaMemcpyAsync(dsh, shift + 3 * b, m * 3 * sizeof(double), cudaMemcpyHostToDevice, s)))
            return cuda_fail(c, e, "host-to-device copy");
        if (src_index && (e = cudaMemcpyAsync(dm + 2 * chunk, src_index, m * 4, cudaMemcpyHostToDevice, s)))
            return cuda_fail(c, e, "host-to-device copy");
        if (dst_index && (e = cudaMemcpyAsync(dm + 3 * chunk, dst_index, m * 4, cudaMemcpyHostToDevice, s)))
            return cuda_fail(c, e, "host-to-device copy");
        st = run_batch(c, s, op, a, (int)pmax, (long long)m, c->d_src[k].p, (long long)src_stride, (long long)ns,
                       src_index ? dm + 2 * chunk : nullptr, c->d_dst[k].p, (long long)dst_stride, (long long)nd,
                       dst_index ? dm + 3 * chunk : nullptr, dm, dm + chunk, dsh, nullptr, flags);
        if (st) return st;
        if ((e = cudaMemcpyAsync(dstp, c->d_dst[k].p, nd * dst_stride * es, cudaMemcpyDeviceToHost, s)))
            return cuda_fail(c, e, "device-to-host copy");
    }
    for (int k = 0; k < slots; ++k)
        if ((e = cudaStreamSynchronize(c->pipe[k])) != cudaSuccess) return cuda_fail(c, e, "synchronise");
    return SFMM_OK;
}

int sfmm_translate_host(sfmm_context *c, int op, int precision, size_t n, const void *const *src, const size_t *p_in,
                        void *const *dst, const size_t *p_out, size_t dim, const void *x, const void *y,
                        const void *z)
{
    if (!c) return SFMM_INVALID_ARG;
    Range range("sfmm host call");
    if (op < SFMM_M2M || op > SFMM_L2L) return fail(c, SFMM_INVALID_ARG, "unknown operator %d", op);
    Arith a;
    int st = arith_of(c, precision, &a);
    if (st) return st;
    if (n == 0 || dim == 0) return SFMM_OK;
    if (!src || !dst || !p_in || !p_out || !x || !y || !z) return fail(c, SFMM_INVALID_ARG, "null host pointer");
    ClassicInput in;
    in.n = n;
    in.src = src;
    in.p_in = p_in;
    in.dst = dst;
    in.p_out = p_out;
    in.dim = dim;
    in.x = x;
    in.y = y;
    in.z = z;
    in.f64 = c->dtype == SFMM_F64;
    in.P = (size_t)c->P;
    ClassicScan sc;
    try {
        sc = classic_scan(in, host_threads(n * dim));
    } catch (const std::exception &) {
        return fail(c, SFMM_OOM, "host threads");
    }
    if (sc.bad != SIZE_MAX) {
        if (sc.bad_kind == 1)
            return fail(c, SFMM_ORDER_RANGE, "orders exceeding operator data (translation %zu)", sc.bad);
        return fail(c, SFMM_INVALID_ARG, "null solid pointer");
    }
    // One entry per (translation, component) that has work (a zero order adds
    // nothing); targets named more than once share a slot.
    const size_t M = sc.entries;
    if (M == 0) return SFMM_OK;
    if (M >= ((size_t)1 << 31)) return fail(c, SFMM_INVALID_ARG, "more than 2^31 translations in one call");
    const size_t pmax = sc.pmax;
    const size_t es = c->dtype == SFMM_F64 ? 8 : 4;
    const size_t stride = pmax * (pmax + 1);
    std::lock_guard<std::mutex> lock(c->mtx);
    cudaSetDevice(c->device);
    cudaError_t e;
    cudaStream_t s = c->stream;
    // metadata, in pinned staging and on the device alike: source addresses |
    // target addresses | p_in | p_out | target slots | (8-byte aligned) slot
    // addresses [M] | slot sizes [M]; shifts separately
    const size_t toff = (M * 28 + 7) & ~(size_t)7;
    const size_t meta_bytes = toff + M * 12;
    if ((e = c->h_meta.ensure(meta_bytes)) || (e = c->h_shift.ensure(M * 3 * sizeof(double))))
        return cuda_fail(c, e, "pinned staging");
    if ((e = c->d_meta[0].ensure(meta_bytes)) || (e = c->d_shift[0].ensure(M * 3 * sizeof(double))))
        return cuda_fail(c, e, "device buffers");
    char *hm = (char *)c->h_meta.p;
    ClassicEntries ent;
    ent.sptr = (unsigned long long *)hm;
    ent.dptr = ent.sptr + M;
    ent.pin = (uint32_t *)(ent.dptr + M);
    ent.pout = ent.pin + M;
    ent.tidx = ent.pin + 2 * M;
    ent.tptr = (unsigned long long *)(hm + toff);
    ent.tcnt = (uint32_t *)(ent.tptr + M);
    ent.shift = (double *)c->h_shift.p;
    bool repeat = false;
    size_t nt = 0;
    try {
        Range fill_range("sfmm host bookkeeping");
        nt = classic_fill(in, sc, ent, c->slot_scratch, &repeat);
    } catch (const std::bad_alloc &) {
        return fail(c, SFMM_OOM, "host bookkeeping");
    } catch (const std::exception &) {
        return fail(c, SFMM_OOM, "host threads");
    }
    char *mb = (char *)c->d_meta[0].p;
    auto *d_sptr = (unsigned long long *)mb;
    auto *d_dptr = d_sptr + M;
    auto *d_pin = (uint32_t *)(d_dptr + M);
    uint32_t *d_pout = d_pin + M, *d_tidx = d_pin + 2 * M;
    auto *d_tptr = (unsigned long long *)(mb + toff);
    uint32_t *d_tcnt = (uint32_t *)(d_tptr + M);
    const double *d_sh = (const double *)c->d_shift[0].p;
    if ((e = cudaMemcpyAsync(mb, hm, M * 28, cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemcpyAsync((void *)d_sh, ent.shift, M * 3 * sizeof(double), cudaMemcpyHostToDevice, s)))
        return cuda_fail(c, e, "host-to-device copy");
    if (c->pageable_access) {
        // The GPU reads the source solids and updates the target solids where
        // they are, through the host page tables: no staging copies.
        if (!repeat) {
            st = run_batch(c, s, op, a, (int)pmax, (long long)M, nullptr, 0, (long long)M, nullptr, nullptr, 0,
                           (long long)M, nullptr, d_pin, d_pout, d_sh, nullptr, SFMM_TARGETS_UNIQUE, -1, d_sptr,
                           d_dptr, false);
            if (st) return st;
        } else {
            // repeated targets: sums per target in device slots (atomics),
            // then one read-modify-write of each host target
            if ((e = cudaMemcpyAsync(d_tptr, ent.tptr, nt * 8, cudaMemcpyHostToDevice, s)) ||
                (e = cudaMemcpyAsync(d_tcnt, ent.tcnt, nt * 4, cudaMemcpyHostToDevice, s)))
                return cuda_fail(c, e, "host-to-device copy");
            if ((e = c->d_dst[0].ensure(nt * stride * es)) || (e = cudaMemsetAsync(c->d_dst[0].p, 0, nt * stride * es, s)))
                return cuda_fail(c, e, "device buffers");
            st = run_batch(c, s, op, a, (int)pmax, (long long)M, nullptr, 0, (long long)M, nullptr, c->d_dst[0].p,
                           (long long)stride, (long long)nt, d_tidx, d_pin, d_pout, d_sh, nullptr, SFMM_TARGETS_REPEAT,
                           -1, d_sptr, nullptr, false);
            if (st) return st;
            if ((e = launch_add_slots(c->dtype == SFMM_F64, (long long)nt, d_tptr, d_tcnt, c->d_dst[0].p,
                                      (long long)stride, s)) != cudaSuccess)
                return cuda_fail(c, e, "target accumulation kernel");
            c->launches++;
        }
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(c, e, "synchronise");
        return SFMM_OK;
    }
    // Staged path (the GPU cannot use pageable host memory): gather the
    // sources into pinned staging, translate into per-target slots, copy the
    // slots back and add them into the host targets.
    if ((e = c->h_src.ensure(M * stride * es)) || (e = c->h_dst.ensure(nt * stride * es)))
        return cuda_fail(c, e, "pinned staging");
    if ((e = c->d_src[0].ensure(M * stride * es)) || (e = c->d_dst[0].ensure(nt * stride * es)))
        return cuda_fail(c, e, "device buffers");
    char *hs = (char *)c->h_src.p;
    char *hd = (char *)c->h_dst.p;
    const size_t nthr = std::min<size_t>(std::min<size_t>(std::max(1u, std::thread::hardware_concurrency()), 16),
                                         M / 4096 + 1);
    auto parallel = [&](size_t cnt, auto &&fn) {
        if (nthr <= 1) {
            fn(0, cnt);
            return;
        }
        std::vector<std::thread> th;
        for (size_t t = 0; t < nthr; ++t) th.emplace_back(fn, cnt * t / nthr, cnt * (t + 1) / nthr);
        for (auto &t : th) t.join();
    };
    parallel(M, [&](size_t lo, size_t hi) {
        for (size_t k = lo; k < hi; ++k)
            std::memcpy(hs + k * stride * es, (const void *)(uintptr_t)ent.sptr[k],
                        (size_t)ent.pin[k] * (ent.pin[k] + 1) * es);
    });
    if ((e = cudaMemcpyAsync(c->d_src[0].p, hs, M * stride * es, cudaMemcpyHostToDevice, s)) ||
        (e = cudaMemsetAsync(c->d_dst[0].p, 0, nt * stride * es, s)))
        return cuda_fail(c, e, "host-to-device copy");
    st = run_batch(c, s, op, a, (int)pmax, (long long)M, c->d_src[0].p, (long long)stride, (long long)M, nullptr,
                   c->d_dst[0].p, (long long)stride, (long long)nt, d_tidx, d_pin, d_pout, d_sh, nullptr,
                   repeat ? SFMM_TARGETS_REPEAT : SFMM_TARGETS_UNIQUE);
    if (st) return st;
    if ((e = cudaMemcpyAsync(hd, c->d_dst[0].p, nt * stride * es, cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s)))
        return cuda_fail(c, e, "device-to-host copy");
    // scatter-add into the host targets (buf2solid); targets are distinct
    parallel(nt, [&](size_t lo, size_t hi) {
        for (size_t j = lo; j < hi; ++j) {
            if (c->dtype == SFMM_F64) {
                double *o = (double *)(uintptr_t)ent.tptr[j];
                const double *r = (const double *)(hd + j * stride * es);
                for (size_t q = 0; q < ent.tcnt[j]; ++q) o[q] += r[q];
            } else {
                float *o = (float *)(uintptr_t)ent.tptr[j];
                const float *r = (const float *)(hd + j * stride * es);
                for (size_t q = 0; q < ent.tcnt[j]; ++q) o[q] += r[q];
            }
        }
    });
    return SFMM_OK;
}

}  // extern "C"
