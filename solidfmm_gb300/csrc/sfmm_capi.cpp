// C ABI of solidfmm-gb300 (include/sfmm.h): contexts, table upload, launch
// shapes and tuning, device-resident batches, P2M/P2L and evaluation entry
// points; batches in host memory are in sfmm_host.cpp.  No exception crosses
// this boundary.
#include "sfmm.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "sfmm_context.hpp"
#include "sfmm_launch.hpp"
#include "sfmm_params.hpp"
#include "sfmm_tables.hpp"

using namespace sfmm;

namespace sfmm {

int fail(sfmm_context *c, int st, const char *fmt, ...)
{
    if (c) {
        char b[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(b, sizeof b, fmt, ap);
        va_end(ap);
        c->err = b;
    }
    return st;
}

int cuda_fail(sfmm_context *c, cudaError_t e, const char *what)
{
    return fail(c, SFMM_CUDA_ERROR, "%s: %s", what, cudaGetErrorString(e));
}

size_t esize(Arith a) { return a == Arith::F32 ? sizeof(float) : (a == Arith::F64 ? sizeof(double) : 2 * sizeof(float)); }

// convert an FP64 table into the arithmetic's element type
std::vector<unsigned char> convert(const std::vector<double> &v, Arith a)
{
    std::vector<unsigned char> out(v.size() * esize(a));
    for (size_t i = 0; i < v.size(); ++i) {
        if (a == Arith::F64) {
            std::memcpy(&out[i * 8], &v[i], 8);
        } else if (a == Arith::F32) {
            float f = (float)v[i];
            std::memcpy(&out[i * 4], &f, 4);
        } else {
            float hi = (float)v[i];
            float lo = (float)(v[i] - (double)hi);
            std::memcpy(&out[i * 8], &hi, 4);
            std::memcpy(&out[i * 8 + 4], &lo, 4);
        }
    }
    return out;
}

cudaError_t upload(void **dst, const std::vector<double> &v, Arith a)
{
    auto bytes = convert(v, a);
    cudaError_t e = cudaMalloc(dst, bytes.size() ? bytes.size() : 16);
    if (e != cudaSuccess) return e;
    if (bytes.empty()) return cudaSuccess;
    return cudaMemcpy(*dst, bytes.data(), bytes.size(), cudaMemcpyHostToDevice);
}

void free_tables(DevTables &t)
{
    void *ps[] = {t.W, t.ein_M, t.ein_L, t.eout_L, t.eout_M, t.H[0], t.H[1], t.H[2], t.Wq, t.W8, t.Wq8};
    for (void *p : ps)
        if (p) cudaFree(p);
    t = DevTables{};
}

namespace {

void free_offsets(sfmm_context *c)
{
    int **ps[] = {&c->d_woff, &c->d_hoff, &c->d_woff8};
    for (int **p : ps) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
}

// the offset arrays of the tables, all or none (a partial set is freed)
cudaError_t upload_offsets(sfmm_context *c)
{
    const size_t n8 = c->host.woff8.size();
    if (c->d_woff && c->d_hoff && (!n8 || c->d_woff8)) return cudaSuccess;
    free_offsets(c);
    cudaError_t e = cudaMalloc(&c->d_woff, sizeof(int) * c->P);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_hoff, sizeof(int) * c->P);
    if (e == cudaSuccess && n8) e = cudaMalloc(&c->d_woff8, sizeof(int) * n8);
    if (e == cudaSuccess)
        e = cudaMemcpy(c->d_woff, c->host.woff.data(), sizeof(int) * c->P, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(c->d_hoff, c->host.hoff.data(), sizeof(int) * c->P, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n8)
        e = cudaMemcpy(c->d_woff8, c->host.woff8.data(), sizeof(int) * n8, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) free_offsets(c);
    return e;
}

}  // namespace

int ensure_tables(sfmm_context *c, Arith a)
{
    if (is_tc(a)) {
        const int mode = tc_mode(a);
        if (c->tc[mode]) return SFMM_OK;
        cudaError_t e = tc_prepare(&c->tc[mode], mode, c->host);
        if (e != cudaSuccess) return cuda_fail(c, e, "tensor-core table upload");
        return SFMM_OK;
    }
    DevTables &t = c->tab[(int)a];
    if (t.ready) return SFMM_OK;
    cudaError_t e = upload_offsets(c);
    if (e != cudaSuccess) return cuda_fail(c, e, "table upload");
    const bool w8 = !c->host.W8.empty();
    // |w| <= 1 (orthogonal matrices): round(w 2^30) fits int32
    auto upload_q30 = [](void **dst, const std::vector<double> &W) {
        std::vector<int32_t> q(W.size());
        for (size_t i = 0; i < q.size(); ++i) q[i] = (int32_t)std::llround(std::ldexp(W[i], 30));
        cudaError_t err = cudaMalloc(dst, q.size() * sizeof(int32_t) + 16);
        if (err == cudaSuccess) err = cudaMemcpy(*dst, q.data(), q.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
        return err;
    };
    e = upload(&t.W, c->host.W, a);
    if (e == cudaSuccess && w8) e = upload(&t.W8, c->host.W8, a);
    if (e == cudaSuccess) e = upload(&t.ein_M, c->host.e_in_M, a);
    if (e == cudaSuccess) e = upload(&t.ein_L, c->host.e_in_L, a);
    if (e == cudaSuccess) e = upload(&t.eout_L, c->host.e_out_L, a);
    if (e == cudaSuccess) e = upload(&t.eout_M, c->host.e_out_M, a);
    for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = upload(&t.H[k], c->host.H[k], a);
    if (e == cudaSuccess && a == Arith::FFQ) e = upload_q30(&t.Wq, c->host.W);
    if (e == cudaSuccess && a == Arith::FFQ && w8) e = upload_q30(&t.Wq8, c->host.W8);
    if (e != cudaSuccess) {
        free_tables(t);  // a partial set is retried from scratch on the next call
        return cuda_fail(c, e, "table upload");
    }
    t.ready = true;
    return SFMM_OK;
}


int arith_of(sfmm_context *c, int precision, Arith *out)
{
    if (precision == SFMM_PLAIN) {
        *out = c->dtype == SFMM_F64 ? Arith::F64 : Arith::F32;
        return SFMM_OK;
    }
    if (precision == SFMM_SPLIT || precision == SFMM_SPLIT_FF) {
        if (c->dtype != SFMM_F64)
            return fail(c, SFMM_UNSUPPORTED, "split precision needs an FP64 context (FP64 accumulation targets)");
        *out = precision == SFMM_SPLIT ? Arith::FFQ : Arith::FF;
        return SFMM_OK;
    }
    if (precision == SFMM_TC_TF32 || precision == SFMM_TC_BF16 || precision == SFMM_TC_BF16X6) {
        if (c->dtype != SFMM_F64)
            return fail(c, SFMM_UNSUPPORTED, "tensor-core precision needs an FP64 context (FP64 accumulation targets)");
        *out = precision == SFMM_TC_TF32 ? Arith::TC32 : (precision == SFMM_TC_BF16 ? Arith::TC16 : Arith::TC16X6);
        return SFMM_OK;
    }
    return fail(c, SFMM_INVALID_ARG, "unknown precision mode %d", precision);
}

// Split precision keeps its 1e-7 contract (orthonormal basis) with the
// fixed-point rotations for M2L and L2L up to order 28 and M2M up to order
// 18.  Past that the rotation method's own error growth with the degree
// (about 1.35x per degree for M2M, in every arithmetic) pushes 30-bit
// mantissas above 1e-7, and the batch runs in float-float instead.
constexpr int kFixedM2MOrder = 18;
// The tensor-core kernel holds a tile's expansions in tensor memory up to
// order 16; batches with a larger order bound run the split kernel.
Arith resolve_arith(Arith a, int op, int Pbound)
{
    if (is_tc(a) && Pbound > tc_max_order()) a = Arith::FFQ;
    if (a == Arith::FFQ && op == SFMM_M2M && Pbound > kFixedM2MOrder) return Arith::FF;
    return a;
}

int prepare_launch(sfmm_context *c, int op, Arith a, int Pbound, LaunchShape *shape)
{
    a = resolve_arith(a, op, Pbound);
    if (Pbound < 1) Pbound = 1;
    std::lock_guard<std::mutex> lk(c->setup_mtx);
    int st = ensure_tables(c, a);
    if (st) return st;
    if (is_tc(a)) {  // one 128-thread CTA per SM, one translation per thread
        if (shape) {
            *shape = LaunchShape{};
            shape->G = 1;
            shape->acc = 1;
            shape->TS = 128;
            shape->threads = 128;
            shape->blocks_per_sm = 1;
        }
        return SFMM_OK;
    }
    const auto key = std::make_tuple(op, (int)a, Pbound);
    auto it = c->shapes.find(key);
    if (it == c->shapes.end()) it = c->shapes.emplace(key, best_shape(a, Pbound, default_group(a, Pbound))).first;
    if (shape) *shape = it->second;
    if (it->second.acc == 0)
        return fail(c, SFMM_UNSUPPORTED, "order %d exceeds the GPU kernels' limit %d", Pbound, kMaxKernelOrder);
    if (a != Arith::F64 && Pbound > kMaxFloatOrder)
        return fail(c, SFMM_UNSUPPORTED, "order %d exceeds %d, the limit of FP32-range arithmetic", Pbound, kMaxFloatOrder);
    return SFMM_OK;
}

void set_shape(sfmm_context *c, std::tuple<int, int, int> key, const LaunchShape *s)
{
    std::lock_guard<std::mutex> lk(c->setup_mtx);
    if (s) c->shapes[key] = *s;
    else c->shapes.erase(key);
}

const void *device_view(sfmm_context *c, const void *host)
{
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type == cudaMemoryTypeHost && at.devicePointer && at.device == c->device) return at.devicePointer;
    if (at.type == cudaMemoryTypeUnregistered && c->pageable_access) return host;
    return nullptr;
}

// The launch itself: validated arguments, device pointers.
int run_batch(sfmm_context *c, cudaStream_t stream, int op, Arith a, int Pbound, long long n, const void *src,
              long long sstride, long long nsrc, const uint32_t *sidx, void *dst, long long dstride, long long ndst,
              const uint32_t *tidx, const uint32_t *pin, const uint32_t *pout, const double *shift,
              const uint32_t *perm, int flags, long long nidx, const unsigned long long *src_ptr,
              const unsigned long long *dst_ptr, bool in_hbm, const WorkList *wl, const LaunchShape *shape)
{
    if (n == 0) return SFMM_OK;
    static const char *const kName[3] = {"sfmm m2m launch", "sfmm m2l launch", "sfmm l2l launch"};
    Range range(kName[(op >= SFMM_M2M && op <= SFMM_L2L) ? op - SFMM_M2M : 1]);
    a = resolve_arith(a, op, Pbound);
    if (Pbound < 1) Pbound = 1;
    LaunchShape s;
    int st = prepare_launch(c, op, a, Pbound, &s);
    if (st) return st;
    if (shape && !is_tc(a)) s = *shape;
    KParams p{};
    p.op = op;
    p.P = Pbound;
    p.Ptab = c->P;
    p.n = n;
    p.src = src;
    p.sstride = sstride;
    p.nsrc = nsrc;
    p.sidx = sidx;
    p.dst = dst;
    p.dstride = dstride;
    p.ndst = ndst;
    p.tidx = tidx;
    p.status = c->d_status;
    p.pin = pin;
    p.pout = pout;
    p.shift = shift;
    p.perm = perm;
    p.nidx = nidx < 0 ? n : nidx;
    p.src_ptr = src_ptr;
    p.dst_ptr = dst_ptr;
    p.atomic = (flags & SFMM_TARGETS_REPEAT) ? 1 : 0;
    p.in_hbm = in_hbm ? 1 : 0;
    if (wl) {
        if (is_tc(a)) return fail(c, SFMM_UNSUPPORTED, "work lists run the split and plain kernels");
        p.work = wl->work;
        p.work_counter = wl->counter;
        p.nwork = wl->n;
    }
    if (is_tc(a)) {
        cudaError_t e = launch_translate_tc(p, c->tc[tc_mode(a)], c->num_sms, stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "tensor-core translation kernel launch");
        c->launches++;
        return SFMM_OK;
    }
    const DevTables &t = c->tab[(int)a];
    // swap blocks padded for this launch's group size (4 or 8 threads per
    // translation step 8 rows, one warp 32)
    const bool w8 = s.G != 32 && c->d_woff8;
    p.W = w8 ? t.W8 : t.W;
    p.Wq = static_cast<const int *>(w8 ? t.Wq8 : t.Wq);
    p.woff = w8 ? c->d_woff8 : c->d_woff;
    p.hoff = c->d_hoff;
    p.rowpad = c->host.pad;
    p.ein = (op == SFMM_L2L) ? t.ein_L : t.ein_M;
    p.eout = (op == SFMM_M2M) ? t.eout_M : t.eout_L;
    p.H = t.H[op];
    p.spad = s.spad;
    p.TS = s.TS;
    long long tiles = wl ? wl->n : (n + s.TS - 1) / s.TS;
    long long grid = (long long)c->num_sms * s.blocks_per_sm;
    if (grid > tiles) grid = tiles;
    if (grid < 1) return fail(c, SFMM_CUDA_ERROR, "no launch shape runs order %d (G %d, %d translations per CTA)",
                              Pbound, s.G, s.TS);
    if (a != Arith::F64 && s.spad > kDegreeTableSize)
        return fail(c, SFMM_UNSUPPORTED, "buffer of %d slots above the FP32-range kernels' degree table", s.spad);
    if (wl) {  // the tile descriptor's two words after the meta arrays
        s.smem += 8;
        if (s.smem > 232448) return fail(c, SFMM_UNSUPPORTED, "work-list launch above the shared-memory limit");
    }
    cudaError_t e = launch_translate(a, p, s, (int)grid, stream);
    if (e != cudaSuccess)
        return fail(c, SFMM_CUDA_ERROR, "translation kernel launch (order %d, G %d, %d per CTA, %zu B shared, grid %lld): %s",
                    Pbound, s.G, s.TS, s.smem, grid, cudaGetErrorString(e));
    c->launches++;
    return SFMM_OK;
}

}  // namespace sfmm

namespace sfmm {

LaunchShape translate_shape(Arith a, int P, int G, int ts)
{
    LaunchShape s;
    const int per_warp = 32 / G;  // translations per warp
    if (P < 1 || P > kMaxKernelOrder || ts < per_warp || ts % per_warp || G * ts > 256) return s;
    if ((G == 32) != (P > 32)) return s;  // one warp per translation exactly for orders above 32
    int acc = (P + G - 1) / G;
    if (G == 4) acc = acc <= 2 ? 2 : (acc <= 4 ? 4 : (acc <= 6 ? 6 : 8));
    if (G == 32) acc = acc <= 2 ? 2 : 3;
    s.G = G;
    s.acc = acc;
    int scap = P * (P + 1) + 4;  // room for the swap loops' zero-coefficient reads past the last row
    // Translation stride in shared memory.  The swap and z loops read one or
    // two slots per translation, broadcast to its group; the per-element
    // stages touch G consecutive slots per translation.  With 8 translations
    // per warp (G = 4) bases 4 banks apart keep the broadcasts conflict-free;
    // with 4 per warp (G = 8) bases 8 banks apart keep both patterns at the
    // minimum number of wavefronts.
    const int mod = esize(a) == 8 ? 16 : 32;
    const int want = esize(a) == 8 ? (G == 8 ? 4 : 2) : (G == 8 ? 8 : 4);
    s.spad = scap + ((want - scap) % mod + mod) % mod;
    s.TS = ts;
    s.threads = G * ts;
    s.smem = (size_t)ts * s.spad * esize(a) + 5 * sizeof(uint32_t) * ts;
    if (s.smem > 232448) return LaunchShape{};
    return s;
}

// Threads per translation by default: one warp above order 32; below, 4 or
// 8 from a sweep on GB300 (M2L, uniform orders 2..32, both group sizes): 8
// threads pay off once the per-translation buffers limit the SM to a few
// warps and the group's own arithmetic is cheap enough to leave latency
// exposed (FP64 from order 24, FP32 from 17, both split modes from 14).
int default_group(Arith a, int P)
{
    if (P > 32) return 32;
    switch (a) {
    case Arith::F64: return P >= 24 ? 8 : 4;
    case Arith::F32: return P >= 17 ? 8 : 4;
    case Arith::FF: return P >= 14 ? 8 : 4;
    case Arith::FFQ: return P >= 14 ? 8 : 4;
    }
    return 4;
}

// The tile size that keeps the most threads resident per SM (shared memory
// and registers permitting) for G threads per translation; ties go to the
// larger tile (fewer CTAs), or to the smaller one with small_tiles (shorter
// waits at the tile barriers).
LaunchShape best_shape(Arith a, int P, int G, bool small_tiles, int min_threads)
{
    // By default CTAs of at least four warps: one-warp tiles can hold a few
    // more threads per SM at high orders, but ran up to 40% slower on GB300
    // (split M2L P=22: 1 976 CTAs of 32 threads, instruction-fetch stalls and
    // a lower L1 hit rate for the tables); smaller CTAs when no larger tile
    // fits, or when sfmm_tune measures them faster (split P=27: +6%).
    for (int floor_threads : {min_threads, 32}) {
        LaunchShape best;
        long best_threads = 0;
        for (int ts = 256 / G; ts >= 32 / G; ts -= 32 / G) {
            if (G * ts < floor_threads) break;
            LaunchShape s = translate_shape(a, P, G, ts);
            if (!s.acc) continue;
            s.blocks_per_sm = translate_blocks_per_sm(a, s);
            long th = (long)s.blocks_per_sm * s.threads;
            if (th > 0 && (th > best_threads || (small_tiles && th == best_threads))) {
                best_threads = th;
                best = s;
            }
        }
        if (best.acc) return best;
    }
    return LaunchShape{};
}

cudaError_t launch_translate_64(const KParams &, const LaunchShape &, int, cudaStream_t);
cudaError_t launch_translate_32(const KParams &, const LaunchShape &, int, cudaStream_t);
cudaError_t launch_translate_ff(const KParams &, const LaunchShape &, int, cudaStream_t);
cudaError_t launch_translate_ffq(const KParams &, const LaunchShape &, int, cudaStream_t);
int occupancy_64(const LaunchShape &);
int occupancy_32(const LaunchShape &);
int occupancy_ff(const LaunchShape &);
int occupancy_ffq(const LaunchShape &);

cudaError_t launch_translate(Arith a, const KParams &p, const LaunchShape &s, int grid, cudaStream_t st)
{
    switch (a) {
    case Arith::F64: return launch_translate_64(p, s, grid, st);
    case Arith::F32: return launch_translate_32(p, s, grid, st);
    case Arith::FFQ: return launch_translate_ffq(p, s, grid, st);
    default: return launch_translate_ff(p, s, grid, st);
    }
}

int translate_blocks_per_sm(Arith a, const LaunchShape &s)
{
    switch (a) {
    case Arith::F64: return occupancy_64(s);
    case Arith::F32: return occupancy_32(s);
    case Arith::FFQ: return occupancy_ffq(s);
    default: return occupancy_ff(s);
    }
}

}  // namespace sfmm

extern "C" {

const char *sfmm_status_string(int s)
{
    switch (s) {
    case SFMM_OK: return "ok";
    case SFMM_INVALID_ARG: return "invalid argument";
    case SFMM_ORDER_RANGE: return "order out of range";
    case SFMM_OVERFLOW: return "order too large for the floating-point type";
    case SFMM_DIM_MISMATCH: return "dimension mismatch";
    case SFMM_OOM: return "out of memory";
    case SFMM_CUDA_ERROR: return "CUDA error";
    case SFMM_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
    }
}

int sfmm_create(sfmm_context **out, int dtype, size_t P, int device)
{
    if (!out) return SFMM_INVALID_ARG;
    *out = nullptr;
    if (dtype != SFMM_F32 && dtype != SFMM_F64) return SFMM_INVALID_ARG;
    if (P == 0) return SFMM_INVALID_ARG;
    if ((dtype == SFMM_F32 && P > (size_t)kMaxFloatOrder) || (dtype == SFMM_F64 && P > 86)) return SFMM_OVERFLOW;
    sfmm_context *c = new (std::nothrow) sfmm_context;
    if (!c) return SFMM_OOM;
    c->dtype = dtype;
    c->P = (int)P;
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device) == cudaSuccess)
            c->pageable_access = v != 0;
    }
    if (e != cudaSuccess) {
        delete c;
        return SFMM_CUDA_ERROR;
    }
    try {
        c->host = build_tables((int)P);
    } catch (const std::bad_alloc &) {
        delete c;
        return SFMM_OOM;
    }
    if (cudaMalloc(&c->d_status, sizeof(int)) != cudaSuccess || cudaMemset(c->d_status, 0, sizeof(int)) != cudaSuccess) {
        if (c->d_status) cudaFree(c->d_status);
        delete c;
        return SFMM_CUDA_ERROR;
    }
    *out = c;
    return SFMM_OK;
}

void sfmm_destroy(sfmm_context *c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    for (auto &t : c->tab) free_tables(t);
    for (auto &t : c->tc) tc_release(t);
    for (int k = 0; k < 3; ++k) {
        c->d_src[k].release();
        c->d_dst[k].release();
        c->d_meta[k].release();
        c->d_shift[k].release();
        if (c->pipe[k]) cudaStreamDestroy(c->pipe[k]);
    }
    c->d_work.release();
    c->d_eval.release();
    if (c->d_status) cudaFree(c->d_status);
    free_offsets(c);
    c->h_src.release();
    c->h_dst.release();
    c->h_meta.release();
    c->h_shift.release();
    delete c;
}

size_t sfmm_order(const sfmm_context *c) { return c ? (size_t)c->P : 0; }
int sfmm_data_type(const sfmm_context *c) { return c ? c->dtype : -1; }
const char *sfmm_last_error(const sfmm_context *c) { return c ? c->err.c_str() : "null context"; }
uint64_t sfmm_launch_count(const sfmm_context *c) { return c ? c->launches.load() : 0; }

int sfmm_host_table(size_t P, int which, int n, double *out, size_t cap, size_t *count)
{
    if (P == 0 || P > 86 || !count) return SFMM_INVALID_ARG;
    HostTables t;
    try {
        t = build_tables((int)P);
    } catch (const std::bad_alloc &) {
        return SFMM_OOM;
    }
    std::vector<double> v;
    if (which == 0 || which == 1) {  // dense W_R / W_I of degree n, row-major (i, j)
        if (n < 0 || n >= (int)P) return SFMM_INVALID_ARG;
        const int d = n + 1;
        for (int i = 0; i < d; ++i)
            for (int j = 0; j < d; ++j) v.push_back(w_entry(t, n, which, i, j));
    } else if (which >= 2 && which <= 4) {  // dense H_m (n', k) of op which-2, row-major, m = n
        const int m = n, L = (int)P - m;
        if (m < 0 || m >= (int)P) return SFMM_INVALID_ARG;
        const int HR = hrows(L, t.pad);
        for (int a = 0; a < L; ++a)
            for (int k = 0; k < L; ++k) v.push_back(t.H[which - 2][t.hoff[m] + (size_t)k * HR + a]);
    } else if (which >= 5 && which <= 8) {  // edge factors
        const std::vector<double> *e[] = {&t.e_in_M, &t.e_in_L, &t.e_out_L, &t.e_out_M};
        v = *e[which - 5];
    } else {
        return SFMM_INVALID_ARG;
    }
    *count = v.size();
    if (out) std::memcpy(out, v.data(), sizeof(double) * std::min(cap, v.size()));
    return SFMM_OK;
}

int sfmm_set_stream(sfmm_context *c, void *stream)
{
    if (!c) return SFMM_INVALID_ARG;
    c->stream = (cudaStream_t)stream;
    return SFMM_OK;
}

int sfmm_set_group(sfmm_context *c, int precision, size_t order_bound, int group)
{
    if (!c) return SFMM_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mtx);
    Arith a;
    int st = arith_of(c, precision, &a);
    if (st) return st;
    if (order_bound > (size_t)c->P) return fail(c, SFMM_ORDER_RANGE, "order bound %zu exceeds the context order %d", order_bound, c->P);
    const int Pb = order_bound ? (int)order_bound : c->P;
    if (is_tc(resolve_arith(a, SFMM_M2L, Pb)))
        return fail(c, SFMM_UNSUPPORTED, "the tensor-core kernel runs one thread per translation");
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, SFMM_CUDA_ERROR, "cannot select device %d", c->device);
    LaunchShape s[3];
    for (int op = SFMM_M2M; op <= SFMM_L2L; ++op) {  // every operator at this order
        s[op - SFMM_M2M] = best_shape(resolve_arith(a, op, Pb), Pb, group);
        if (!s[op - SFMM_M2M].acc)
            return fail(c, SFMM_INVALID_ARG, "no kernel runs %d threads per translation at order %d", group, Pb);
    }
    std::lock_guard<std::mutex> lk2(c->setup_mtx);
    for (int op = SFMM_M2M; op <= SFMM_L2L; ++op)
        c->shapes[std::make_tuple(op, (int)resolve_arith(a, op, Pb), Pb)] = s[op - SFMM_M2M];
    return SFMM_OK;
}

int sfmm_tune(sfmm_context *c, int op, int precision, size_t order_bound, size_t n, int *group, double *rate)
{
    if (!c) return SFMM_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mtx);
    if (op < SFMM_M2M || op > SFMM_L2L) return fail(c, SFMM_INVALID_ARG, "unknown operation %d", op);
    Arith a;
    int st = arith_of(c, precision, &a);
    if (st) return st;
    if (order_bound > (size_t)c->P) return fail(c, SFMM_ORDER_RANGE, "order bound %zu exceeds the context order %d", order_bound, c->P);
    if (n == 0 || n > (size_t)1 << 24) return fail(c, SFMM_INVALID_ARG, "tuning sample of %zu translations", n);
    const int Pb = order_bound ? (int)order_bound : c->P;
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, SFMM_CUDA_ERROR, "cannot select device %d", c->device);
    const size_t S = (size_t)Pb * (Pb + 1), es = c->dtype == SFMM_F64 ? 8 : 4;
    // synthetic batch: constant coefficients, orders Pb, shifts of length
    // 2.5 in varied directions (the kernels' cost does not depend on values)
    std::vector<uint32_t> ord(n, (uint32_t)Pb);
    std::vector<double> sh(3 * n);
    for (size_t i = 0; i < n; ++i) {
        const double t = 0.7 * (double)i, u = 0.3 + 2.4 * (double)(i % 97) / 97.0;
        sh[3 * i] = 2.5 * std::sin(u) * std::cos(t);
        sh[3 * i + 1] = 2.5 * std::sin(u) * std::sin(t);
        sh[3 * i + 2] = 2.5 * std::cos(u);
    }
    void *src = nullptr, *dst = nullptr, *meta = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&] {
        if (src) cudaFree(src);
        if (dst) cudaFree(dst);
        if (meta) cudaFree(meta);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    cudaError_t e;
    if ((e = cudaMalloc(&src, n * S * es)) != cudaSuccess || (e = cudaMalloc(&dst, n * S * es)) != cudaSuccess ||
        (e = cudaMalloc(&meta, n * (2 * sizeof(uint32_t) + 3 * sizeof(double)))) != cudaSuccess) {
        cleanup();
        return e == cudaErrorMemoryAllocation ? fail(c, SFMM_OOM, "tuning buffers") : cuda_fail(c, e, "tuning buffers");
    }
    double *d_shift = static_cast<double *>(meta);
    uint32_t *d_ord = reinterpret_cast<uint32_t *>(d_shift + 3 * n);
    cudaStream_t stream = c->stream;
    if ((e = cudaMemsetAsync(src, 0x3e, n * S * es, stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(dst, 0, n * S * es, stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_shift, sh.data(), 3 * n * sizeof(double), cudaMemcpyHostToDevice, stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_ord, ord.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, stream)) != cudaSuccess ||
        (e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess) {
        cleanup();
        return cuda_fail(c, e, "tuning setup");
    }
    a = resolve_arith(a, op, Pb);
    if (is_tc(a)) {  // one launch shape: time it
        float ms = 0;
        for (int rep = 0; rep < 2 && st == SFMM_OK; ++rep) {
            if (rep == 1 && (e = cudaEventRecord(e0, stream)) != cudaSuccess) break;
            for (int k = 0; k < (rep ? 3 : 1) && st == SFMM_OK; ++k)
                st = run_batch(c, stream, op, a, Pb, (long long)n, src, (long long)S, (long long)n, nullptr, dst,
                               (long long)S, (long long)n, nullptr, d_ord, d_ord, d_shift, nullptr, 0);
            if (rep == 1 && (e = cudaEventRecord(e1, stream)) != cudaSuccess) break;
        }
        if (st == SFMM_OK && e == cudaSuccess && (e = cudaEventSynchronize(e1)) == cudaSuccess)
            e = cudaEventElapsedTime(&ms, e0, e1);
        cleanup();
        if (st != SFMM_OK) return st;
        if (e != cudaSuccess) return cuda_fail(c, e, "tuning run");
        if (group) *group = 1;
        if (rate) *rate = ms > 0 ? 3.0 * (double)n / (ms * 1e-3) : 0.0;
        return SFMM_OK;
    }
    const auto key = std::make_tuple(op, (int)a, Pb);
    LaunchShape best;
    double best_rate = 0;
    // candidates: every group size that runs at this order, each with the
    // largest and the smallest full-occupancy tile, among CTAs of four warps
    // or more and among all tiles (distinct shapes only)
    LaunchShape cands[12];
    int ncand = 0;
    for (int G : {4, 8, 32})
        for (int min_threads : {128, 32})
            for (bool small : {false, true}) {
                const LaunchShape s = best_shape(a, Pb, G, small, min_threads);
                bool seen = !s.acc;
                for (int k = 0; k < ncand && !seen; ++k) seen = cands[k].G == s.G && cands[k].TS == s.TS;
                if (!seen) cands[ncand++] = s;
            }
    for (int ci = 0; ci < ncand; ++ci) {
        const LaunchShape s = cands[ci];
        set_shape(c, key, &s);
        float ms = 0;
        for (int rep = 0; rep < 2 && st == SFMM_OK; ++rep) {  // warm-up, then timed
            if (rep == 1 && (e = cudaEventRecord(e0, stream)) != cudaSuccess) break;
            for (int k = 0; k < (rep ? 3 : 1) && st == SFMM_OK; ++k)
                st = run_batch(c, stream, op, a, Pb, (long long)n, src, (long long)S, (long long)n, nullptr, dst,
                               (long long)S, (long long)n, nullptr, d_ord, d_ord, d_shift, nullptr, 0);
            if (rep == 1 && (e = cudaEventRecord(e1, stream)) != cudaSuccess) break;
        }
        if (st == SFMM_OK && e == cudaSuccess && (e = cudaEventSynchronize(e1)) == cudaSuccess)
            e = cudaEventElapsedTime(&ms, e0, e1);
        if (st != SFMM_OK || e != cudaSuccess) {
            set_shape(c, key, nullptr);
            cleanup();
            return st != SFMM_OK ? st : cuda_fail(c, e, "tuning run");
        }
        const double r = ms > 0 ? 3.0 * (double)n / (ms * 1e-3) : 0.0;
        if (r > best_rate) {
            best_rate = r;
            best = s;
        }
    }
    cleanup();
    if (!best.acc) {
        set_shape(c, key, nullptr);
        return fail(c, SFMM_UNSUPPORTED, "no kernel for order %d", Pb);
    }
    set_shape(c, key, &best);
    {
        std::lock_guard<std::mutex> lk2(c->setup_mtx);
        c->tuned.insert(std::make_tuple(op, (int)a, Pb));
    }
    if (group) *group = best.G;
    if (rate) *rate = best_rate;
    return SFMM_OK;
}

int sfmm_translate_device(sfmm_context *c, int op, int precision, size_t n, const void *src, size_t src_stride,
                          size_t src_count, const uint32_t *src_index, void *dst, size_t dst_stride,
                          size_t dst_count, const uint32_t *dst_index, const uint32_t *p_in, const uint32_t *p_out,
                          const double *shift, const uint32_t *order, int flags, size_t order_bound)
{
    if (!c) return SFMM_INVALID_ARG;
    if (op < SFMM_M2M || op > SFMM_L2L) return fail(c, SFMM_INVALID_ARG, "unknown operator %d", op);
    Arith a;
    int st = arith_of(c, precision, &a);
    if (st) return st;
    if (n == 0) return SFMM_OK;
    if (n > 0xffffffffull) return fail(c, SFMM_INVALID_ARG, "batch larger than 2^32 translations");
    if (!src || !dst || !p_in || !p_out || !shift)
        return fail(c, SFMM_INVALID_ARG, "null device pointer in batch");
    size_t bound = order_bound ? order_bound : (size_t)c->P;
    if (bound > (size_t)c->P) return fail(c, SFMM_ORDER_RANGE, "order bound %zu exceeds operator order %d", bound, c->P);
    if (src_stride < bound * (bound + 1) || dst_stride < bound * (bound + 1))
        return fail(c, SFMM_INVALID_ARG, "expansion stride smaller than P(P+1) for the order bound");
    cudaSetDevice(c->device);
    return run_batch(c, c->stream, op, a, (int)bound, (long long)n, src, (long long)src_stride,
                     (long long)src_count, src_index, dst, (long long)dst_stride, (long long)dst_count, dst_index,
                     p_in, p_out, shift, order, flags);
}

int sfmm_device_status(sfmm_context *c, int *flags)
{
    if (!c || !flags) return SFMM_INVALID_ARG;
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "stream synchronise");
    int v = 0;
    e = cudaMemcpy(&v, c->d_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, sizeof(int));
    if (e != cudaSuccess) return cuda_fail(c, e, "status read");
    *flags = v;
    return SFMM_OK;
}

int sfmm_bucket_by_order(sfmm_context *c, size_t n, const uint32_t *p_in, const uint32_t *p_out, uint32_t *order)
{
    if (!c) return SFMM_INVALID_ARG;
    Range range("sfmm bucket");
    if (n == 0) return SFMM_OK;
    if (!p_in || !p_out || !order) return fail(c, SFMM_INVALID_ARG, "null device pointer");
    if (n > 0xffffffffull) return fail(c, SFMM_INVALID_ARG, "batch larger than 2^32 - 1 translations");
    cudaSetDevice(c->device);
    cudaError_t e = c->d_work.ensure(bucket_work_words(c->P) * sizeof(uint32_t));
    if (e != cudaSuccess) return cuda_fail(c, e, "bucket workspace");
    e = launch_bucket((long long)n, p_in, p_out, order, (uint32_t *)c->d_work.p, c->P, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "bucket kernels");
    c->launches += 3;
    return SFMM_OK;
}

int sfmm_p2x_device(sfmm_context *c, int kind, size_t nexp, size_t nq, const double *charge, const double *pos,
                    const double *centre, void *out, size_t out_stride)
{
    if (!c) return SFMM_INVALID_ARG;
    Range range("sfmm p2m/p2l");
    if (kind != 0 && kind != 1) return fail(c, SFMM_INVALID_ARG, "kind must be 0 (P2M) or 1 (P2L)");
    if (nexp == 0) return SFMM_OK;
    if (!charge || !pos || !centre || !out) return fail(c, SFMM_INVALID_ARG, "null device pointer");
    if (out_stride < (size_t)c->P * (c->P + 1)) return fail(c, SFMM_INVALID_ARG, "stride smaller than P(P+1)");
    cudaSetDevice(c->device);
    cudaError_t e = launch_p2x(c->dtype == SFMM_F64, kind, c->P, (long long)nexp, (long long)nq, nullptr, charge,
                               pos, centre, out, (long long)out_stride, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "P2M/P2L kernel");
    c->launches++;
    return SFMM_OK;
}

int sfmm_p2x_ragged_device(sfmm_context *c, int kind, size_t nexp, const uint32_t *offset, const double *charge,
                           const double *pos, const double *centre, void *out, size_t out_stride)
{
    if (!c) return SFMM_INVALID_ARG;
    Range range("sfmm p2m/p2l");
    if (kind != 0 && kind != 1) return fail(c, SFMM_INVALID_ARG, "kind must be 0 (P2M) or 1 (P2L)");
    if (nexp == 0) return SFMM_OK;
    if (!offset || !charge || !pos || !centre || !out) return fail(c, SFMM_INVALID_ARG, "null device pointer");
    if (out_stride < (size_t)c->P * (c->P + 1)) return fail(c, SFMM_INVALID_ARG, "stride smaller than P(P+1)");
    cudaSetDevice(c->device);
    cudaError_t e = launch_p2x(c->dtype == SFMM_F64, kind, c->P, (long long)nexp, 0, offset, charge, pos, centre,
                               out, (long long)out_stride, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "P2M/P2L kernel");
    c->launches++;
    return SFMM_OK;
}

int sfmm_eval_device(sfmm_context *c, int kind, size_t npts, const double *pos, const uint32_t *box,
                     const void *E, size_t stride, size_t nexp, const double *centre, double *potential,
                     double *gradient)
{
    if (!c) return SFMM_INVALID_ARG;
    Range range("sfmm l2p/m2p");
    if (kind != 0 && kind != 1) return fail(c, SFMM_INVALID_ARG, "kind must be 0 (L2P) or 1 (M2P)");
    if (npts == 0) return SFMM_OK;
    if (!pos || !E || !centre || !potential) return fail(c, SFMM_INVALID_ARG, "null device pointer");
    if (stride < (size_t)c->P * (c->P + 1)) return fail(c, SFMM_INVALID_ARG, "stride smaller than P(P+1)");
    if (gradient && kind != 0) return fail(c, SFMM_UNSUPPORTED, "gradients are evaluated for local expansions");
    if (!box && nexp < npts) return fail(c, SFMM_INVALID_ARG, "fewer expansions than points without a box index");
    cudaSetDevice(c->device);
    // float-float normalises all nexp expansions into scratch first: worth it
    // from one point per four expansions on.  The scratch is allocated (or
    // grown) outside stream capture only; a call without enough of it (in a
    // capture, or when the allocation fails) runs the FP64 kernel.
    std::lock_guard<std::mutex> lk(c->eval_mtx);  // calls share the scratch, in stream order
    void *scratch = nullptr;
    const size_t need = 4 * npts >= nexp ? eval_scratch_bytes(c->P, (long long)nexp) : 0;
    if (need) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(c->stream, &cs);
        if (cs == cudaStreamCaptureStatusNone && c->d_eval.ensure(need) != cudaSuccess) clear_stale_error();
        if (c->d_eval.bytes >= need) scratch = c->d_eval.p;
    }
    cudaError_t e = launch_eval(c->dtype == SFMM_F64, kind, c->P, (long long)npts, pos, box, E, (long long)stride,
                                (long long)nexp, centre, potential, gradient, scratch, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "L2P/M2P kernel");
    c->launches++;
    return SFMM_OK;
}

}  // extern "C"
