/*
 * extern "C" wrapper around the reference solidfmm library, compiled together
 * with the reference sources into oracle/_ref/libsolidfmm_ref.so.
 *
 * TEST INFRASTRUCTURE ONLY.  Tests, the golden-fixture generator and the
 * CPU-baseline leg of bench.py call it through ctypes as a checker; nothing
 * in the product links or loads it.
 *
 * Expansions are passed in a uniform-stride flat layout: expansion j starts
 * at base + j*stride reals and holds a solid of order P[j] in the
 * reference's layout (solidfmm/solid.hpp:59-60, re(n,m) at n(n+1)+m,
 * im(n,m) at (n+1)^2+m).  Translation i maps source src_idx[i] onto target
 * tgt_idx[i] with shift xyz[3i..3i+2].
 *
 * mode 0: classic single-thread overload with pointer arrays
 *         (solidfmm/translations.hpp:103-109)
 * mode 1: single-thread translation_info overload (translations.hpp:111-116)
 * mode 2: multithreaded_translator checked call (translations.hpp:76-78)
 * mode 3: multithreaded_translator unchecked call (translations.hpp:80-82)
 */
#include <solidfmm/solid.hpp>
#include <solidfmm/handles.hpp>
#include <solidfmm/harmonics.hpp>
#include <solidfmm/translations.hpp>
#include <solidfmm/swap_matrix.hpp>
#include <solidfmm/sphere.hpp>

#include <chrono>
#include <cstdint>
#include <cstring>
#include <exception>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <cstdio>
#include <thread>
#include <vector>

using namespace solidfmm;

namespace {

template <typename real>
multithreaded_translator<real> &translator(size_t P)
{
    static std::map<size_t, std::unique_ptr<multithreaded_translator<real>>> cache;
    static std::mutex mtx;
    std::lock_guard<std::mutex> g(mtx);
    auto it = cache.find(P);
    if (it == cache.end())
        it = cache.emplace(P, std::make_unique<multithreaded_translator<real>>(P)).first;
    return *it->second;
}

char g_err[512];

template <typename real>
int translate(int op, size_t Pop, size_t n, size_t nsrc, const real *src, const uint32_t *Psrc,
              size_t sstride, size_t ntgt, real *dst, const uint32_t *Ptgt, size_t tstride,
              const uint32_t *sidx, const uint32_t *tidx, const real *xyz, size_t dim, int mode,
              double *seconds)
{
    try {
        std::vector<solid<real>> S, T;
        S.reserve(nsrc);
        T.reserve(ntgt);
        for (size_t j = 0; j < nsrc; ++j) {
            S.emplace_back(Psrc[j], dim);
            size_t cnt = size_t(Psrc[j]) * (Psrc[j] + 1) * dim;
            if (cnt) std::memcpy(S.back().memptr(), src + j * sstride, cnt * sizeof(real));
        }
        for (size_t j = 0; j < ntgt; ++j) {
            T.emplace_back(Ptgt[j], dim);
            size_t cnt = size_t(Ptgt[j]) * (Ptgt[j] + 1) * dim;
            if (cnt) std::memcpy(T.back().memptr(), dst + j * tstride, cnt * sizeof(real));
        }
        std::vector<translation_info<real>> items(n);
        std::vector<const solid<real> *> Mp(n);
        std::vector<solid<real> *> Lp(n);
        std::vector<real> xs(n), ys(n), zs(n);
        for (size_t i = 0; i < n; ++i) {
            items[i] = translation_info<real>{&S[sidx[i]], &T[tidx[i]], xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
            Mp[i] = &S[sidx[i]];
            Lp[i] = &T[tidx[i]];
            xs[i] = xyz[3 * i];
            ys[i] = xyz[3 * i + 1];
            zs[i] = xyz[3 * i + 2];
        }
        auto t0 = std::chrono::steady_clock::now();
        if (mode == 0 || mode == 1) {
            operator_handle<real> oph(Pop);
            buffer_handle<real> buf(oph);
            t0 = std::chrono::steady_clock::now();
            if (mode == 0) {
                if (op == 0) m2m(oph, buf, n, Mp.data(), Lp.data(), xs.data(), ys.data(), zs.data());
                if (op == 1) m2l(oph, buf, n, Mp.data(), Lp.data(), xs.data(), ys.data(), zs.data());
                if (op == 2) l2l(oph, buf, n, Mp.data(), Lp.data(), xs.data(), ys.data(), zs.data());
            } else {
                if (op == 0) m2m(oph, buf, items.data(), items.data() + n);
                if (op == 1) m2l(oph, buf, items.data(), items.data() + n);
                if (op == 2) l2l(oph, buf, items.data(), items.data() + n);
            }
        } else {
            multithreaded_translator<real> &tr = translator<real>(Pop);
            t0 = std::chrono::steady_clock::now();
            if (mode == 2) {
                if (op == 0) tr.m2m(items.data(), items.data() + n);
                if (op == 1) tr.m2l(items.data(), items.data() + n);
                if (op == 2) tr.l2l(items.data(), items.data() + n);
            } else {
                if (op == 0) tr.m2m_unchecked(items.data(), items.data() + n);
                if (op == 1) tr.m2l_unchecked(items.data(), items.data() + n);
                if (op == 2) tr.l2l_unchecked(items.data(), items.data() + n);
            }
        }
        auto t1 = std::chrono::steady_clock::now();
        if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
        for (size_t j = 0; j < ntgt; ++j) {
            size_t cnt = size_t(Ptgt[j]) * (Ptgt[j] + 1) * dim;
            if (cnt) std::memcpy(dst + j * tstride, T[j].memptr(), cnt * sizeof(real));
        }
        return 0;
    } catch (const std::out_of_range &e) {
        std::snprintf(g_err, sizeof g_err, "%s", e.what());
        return 2;
    } catch (const std::overflow_error &e) {
        std::snprintf(g_err, sizeof g_err, "%s", e.what());
        return 3;
    } catch (const std::logic_error &e) {
        std::snprintf(g_err, sizeof g_err, "%s", e.what());
        return 1;
    } catch (const std::exception &e) {
        std::snprintf(g_err, sizeof g_err, "%s", e.what());
        return 9;
    }
}

template <typename real>
void harm(int which, size_t P, real x, real y, real z, real *out)
{
    solid<real> s;
    if (which == 0) s = harmonics::R<real>(P, x, y, z);
    if (which == 1) s = harmonics::S<real>(P, x, y, z);
    if (which == 2) s = harmonics::dR<real>(P, x, y, z);
    if (which == 3) s = harmonics::dS<real>(P, x, y, z);
    size_t cnt = s.order() * (s.order() + 1) * s.dimension();
    if (cnt) std::memcpy(out, s.memptr(), cnt * sizeof(real));
}

template <typename real>
void dotp(size_t PA, size_t dimA, const real *A, size_t PB, size_t dimB, const real *B, real *res)
{
    solid<real> a(PA, dimA), b(PB, dimB);
    std::memcpy(a.memptr(), A, PA * (PA + 1) * dimA * sizeof(real));
    std::memcpy(b.memptr(), B, PB * (PB + 1) * dimB * sizeof(real));
    dot(a, b, res);
}

// A batch of n translations of one operator between separately allocated
// solids of order P, set up once and translated many times through
// multithreaded_translator<double>::*_unchecked, the pattern of the
// reference's tests/benchmark_multithreaded_translator.cpp:64-88.
struct MtBatch {
    int op = 1;
    size_t P = 0;
    std::vector<solid<double>> M, L;
    std::vector<translation_info<double>> items;
};

} // namespace

extern "C" {

// Sources hold a fixed pseudo-random pattern of magnitude 1e-3 (the cost of
// the translation does not depend on the values); targets start at zero.
// Returns nullptr on failure (message in ref_last_error()).
void *ref_mt_batch_create_d(int op, size_t P, size_t n, const double *xyz)
{
    try {
        auto b = std::make_unique<MtBatch>();
        b->op = op;
        b->P = P;
        solid<double> blank(P);
        b->M.assign(n, blank);
        b->L.assign(n, blank);
        b->items.resize(n);
        const size_t S = P * (P + 1);
        uint64_t st = 0x9e3779b97f4a7c15ull;
        for (size_t i = 0; i < n; ++i) {
            double *m = b->M[i].memptr();
            for (size_t c = 0; c < S; ++c) {
                st = st * 6364136223846793005ull + 1442695040888963407ull;
                m[c] = 1e-3 * ((double)(st >> 11) * 0x1.0p-53 - 0.5);
            }
            b->items[i] = translation_info<double>{&b->M[i], &b->L[i], xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
        }
        translator<double>(P).m2l(b->items.data(), b->items.data() + std::min<size_t>(n, 1024));  // warm up
        return b.release();
    } catch (const std::exception &e) {
        std::snprintf(g_err, sizeof g_err, "%s", e.what());
        return nullptr;
    }
}

// one unchecked pass over the whole batch; *seconds = its wall time
int ref_mt_batch_run_d(void *h, double *seconds)
{
    auto *b = static_cast<MtBatch *>(h);
    if (!b) return 1;
    multithreaded_translator<double> &tr = translator<double>(b->P);
    auto *first = b->items.data(), *last = b->items.data() + b->items.size();
    auto t0 = std::chrono::steady_clock::now();
    if (b->op == 0) tr.m2m_unchecked(first, last);
    if (b->op == 1) tr.m2l_unchecked(first, last);
    if (b->op == 2) tr.l2l_unchecked(first, last);
    auto t1 = std::chrono::steady_clock::now();
    if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
    return 0;
}

void ref_mt_batch_destroy_d(void *h) { delete static_cast<MtBatch *>(h); }

const char *ref_last_error() { return g_err; }

int ref_translate_d(int op, size_t Pop, size_t n, size_t nsrc, const double *src, const uint32_t *Psrc,
                    size_t sstride, size_t ntgt, double *dst, const uint32_t *Ptgt, size_t tstride,
                    const uint32_t *sidx, const uint32_t *tidx, const double *xyz, size_t dim, int mode,
                    double *seconds)
{
    return translate<double>(op, Pop, n, nsrc, src, Psrc, sstride, ntgt, dst, Ptgt, tstride, sidx, tidx, xyz,
                             dim, mode, seconds);
}

int ref_translate_f(int op, size_t Pop, size_t n, size_t nsrc, const float *src, const uint32_t *Psrc,
                    size_t sstride, size_t ntgt, float *dst, const uint32_t *Ptgt, size_t tstride,
                    const uint32_t *sidx, const uint32_t *tidx, const float *xyz, size_t dim, int mode,
                    double *seconds)
{
    return translate<float>(op, Pop, n, nsrc, src, Psrc, sstride, ntgt, dst, Ptgt, tstride, sidx, tidx, xyz,
                            dim, mode, seconds);
}

void ref_harmonic_d(int which, size_t P, double x, double y, double z, double *out)
{
    harm<double>(which, P, x, y, z, out);
}
void ref_harmonic_f(int which, size_t P, float x, float y, float z, float *out)
{
    harm<float>(which, P, x, y, z, out);
}
void ref_dot_d(size_t PA, size_t dA, const double *A, size_t PB, size_t dB, const double *B, double *r)
{
    dotp<double>(PA, dA, A, PB, dB, B, r);
}

double ref_swap_B(int n, int m, int l)
{
    static std::unique_ptr<swap_matrix<double>> B;
    if (!B || B->order() <= n) B = std::make_unique<swap_matrix<double>>(n + 1);
    return (*B)(n, m, l);
}

unsigned ref_hw_threads()
{
    return std::thread::hardware_concurrency();
}

// the reference's bounding_sphere over points (r == NULL) or spheres; 0 = ok,
// 1 = std::logic_error, 2 = other exception
int ref_bounding_sphere_d(size_t n, const double *x, const double *y, const double *z, const double *r,
                          double *out)
{
    try {
        sphere<double> s;
        if (!r) {
            s = bounding_sphere(n, x, y, z);
        } else {
            std::vector<sphere<double>> v(n);
            for (size_t i = 0; i < n; ++i) v[i] = sphere<double>{x[i], y[i], z[i], r[i]};
            s = bounding_sphere(v.data(), v.data() + n);
        }
        out[0] = s.x;
        out[1] = s.y;
        out[2] = s.z;
        out[3] = s.r;
        return 0;
    } catch (const std::logic_error &e) {
        std::snprintf(g_err, sizeof g_err, "%s", e.what());
        return 1;
    } catch (const std::exception &e) {
        std::snprintf(g_err, sizeof g_err, "%s", e.what());
        return 2;
    }
}
}
