// Translation operators of the drop-in API on top of the C ABI.
//
// Every overload of the reference (solidfmm/translations.cpp:634-1001 and
// multithreaded_translator.cpp:660-744) reduces to one host batch: the
// per-component (source, target, shift) triples of the call are handed to
// sfmm_translate_host, which gathers them to the GPU, runs one fused kernel
// and scatter-adds the results into the host targets before returning.
// Checked variants validate first and throw the reference's exception types
// without modifying any target.
#include <solidfmm/operator_data.hpp>
#include <solidfmm/solid.hpp>
#include <solidfmm/threadlocal_buffer.hpp>
#include <solidfmm/translations.hpp>

#include <cstdint>
#include <cstdio>
#include <exception>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "sfmm.h"
#include "sfmm_hostbatch.hpp"

namespace solidfmm
{

namespace
{

thread_local bool g_split = false;

template <typename real> struct kind;
template <> struct kind<float> {
    static constexpr const char *name = "float";
};
template <> struct kind<double> {
    static constexpr const char *name = "double";
};

// One batch of component translations in the C ABI's host form.  Each host
// thread keeps its batch between calls (scratch()), so a call of the same
// size as the last one neither allocates nor clears its arrays.
template <typename real>
struct batch {
    std::vector<const void *> src;
    std::vector<void *> dst;
    std::vector<size_t> pin, pout;
    std::vector<real> x, y, z;

    void resize(size_t m)
    {
        src.resize(m);
        dst.resize(m);
        pin.resize(m);
        pout.resize(m);
        x.resize(m);
        y.resize(m);
        z.resize(m);
    }
    // the components of one (source, target) pair at positions k, k+1, ...
    void put(size_t k, const solid<real> &s, solid<real> &t, real xx, real yy, real zz)
    {
        const size_t Si = s.order() * (s.order() + 1), So = t.order() * (t.order() + 1);
        for (size_t d = 0; d < s.dimension(); ++d, ++k) {
            src[k] = s.memptr() + d * Si;
            dst[k] = t.memptr() + d * So;
            pin[k] = s.order();
            pout[k] = t.order();
            x[k] = xx;
            y[k] = yy;
            z[k] = zz;
        }
    }
    int run(sfmm_context *ctx, int op) const
    {
        const int prec = (g_split && sizeof(real) == sizeof(double)) ? SFMM_SPLIT : SFMM_PLAIN;
        return sfmm_translate_host(ctx, op, prec, src.size(), src.data(), pin.data(), dst.data(), pout.data(), 1,
                                   x.data(), y.data(), z.data());
    }
    static batch &scratch()
    {
        static thread_local batch b;
        return b;
    }
};

// One translation of a call: source, target, shift.
template <typename real>
struct pair_ref {
    const solid<real> *s;
    solid<real> *t;
    real x, y, z;
};

const char *op_name(int op) { return op == SFMM_M2M ? "m2m" : (op == SFMM_M2L ? "m2l" : "l2l"); }

void raise(sfmm_context *ctx, int rc, int op, const char *type)
{
    std::string msg = std::string{"solidfmm::"} + op_name(op) + "<" + type + ">(): " + sfmm_last_error(ctx);
    if (rc == SFMM_ORDER_RANGE) throw std::out_of_range{msg};
    if (rc == SFMM_INVALID_ARG || rc == SFMM_DIM_MISMATCH) throw std::logic_error{msg};
    if (rc == SFMM_OOM) throw std::bad_alloc{};
    throw std::runtime_error{msg};
}

[[noreturn]] void die(sfmm_context *ctx, int op, const char *type)
{
    std::fprintf(stderr, "solidfmm::%s_unchecked<%s>(): %s\n", op_name(op), type, sfmm_last_error(ctx));
    std::terminate();
}

template <typename real>
void check_buffer(const operator_data<real> &op, const threadlocal_buffer<real> &buf, int opk)
{
    if (!buf.compatible(op))
        throw std::logic_error{std::string{"solidfmm::"} + op_name(opk) + "<" + kind<real>::name +
                               ">(): operator data and buffer incompatible"};
}

// Check (when asked) and gather the n translations pair(i) of a call into a
// batch, on the host cores in parallel: each share of the translations counts
// its components, then writes its own range.  An invalid pair throws the
// exception a sequential loop would throw first (dimension checked before
// orders, lowest index first).
template <typename real, class Pair>
void gather(int opk, const operator_data<real> &op, size_t n, Pair &&pair, bool checked, batch<real> &b)
{
    const size_t nthr = sfmm::host_threads(n);
    std::vector<size_t> cnt(nthr, 0), bad(nthr, SIZE_MAX);
    std::vector<int> why(nthr, 0);
    sfmm::fork_join(nthr, [&](size_t t) {
        size_t c = 0;
        for (size_t i = sfmm::share_lo(n, t, nthr); i < sfmm::share_lo(n, t + 1, nthr); ++i) {
            const pair_ref<real> r = pair(i);
            if (checked) {
                if (r.s->dimension() != r.t->dimension()) {
                    bad[t] = i;
                    why[t] = 1;
                    break;
                }
                if (r.s->order() > op.order() || r.t->order() > op.order()) {
                    bad[t] = i;
                    why[t] = 2;
                    break;
                }
            }
            c += r.s->dimension();
        }
        cnt[t] = c;
    });
    for (size_t t = 0; t < nthr; ++t) {
        if (bad[t] == SIZE_MAX) continue;
        const std::string where = std::string{"solidfmm::"} + op_name(opk) + "<" + kind<real>::name + ">(): ";
        if (why[t] == 1) throw std::logic_error{where + "dimension mismatch."};
        throw std::out_of_range{where + "orders exceeding operator data."};
    }
    std::vector<size_t> off(nthr + 1, 0);
    for (size_t t = 0; t < nthr; ++t) off[t + 1] = off[t] + cnt[t];
    b.resize(off[nthr]);
    sfmm::fork_join(nthr, [&](size_t t) {
        size_t k = off[t];
        for (size_t i = sfmm::share_lo(n, t, nthr); i < sfmm::share_lo(n, t + 1, nthr); ++i) {
            const pair_ref<real> r = pair(i);
            b.put(k, *r.s, *r.t, r.x, r.y, r.z);
            k += r.s->dimension();
        }
    });
}

template <typename real>
void classic(int opk, const operator_data<real> &op, threadlocal_buffer<real> &buf, size_t howmany,
             const solid<real> *const *const M, solid<real> *const *const L, const real *x, const real *y,
             const real *z)
{
    check_buffer(op, buf, opk);
    batch<real> &b = batch<real>::scratch();
    gather(opk, op, howmany, [&](size_t i) { return pair_ref<real>{M[i], L[i], x[i], y[i], z[i]}; }, true, b);
    int rc = b.run(op.context(), opk);
    if (rc) raise(op.context(), rc, opk, kind<real>::name);
}

template <typename real>
void items(int opk, const operator_data<real> &op, const translation_info<real> *begin,
           const translation_info<real> *end, bool checked)
{
    batch<real> &b = batch<real>::scratch();
    gather(opk, op, size_t(end - begin),
           [&](size_t i) { return pair_ref<real>{begin[i].source, begin[i].target, begin[i].x, begin[i].y, begin[i].z}; },
           checked, b);
    int rc = b.run(op.context(), opk);
    if (rc) {
        if (checked) raise(op.context(), rc, opk, kind<real>::name);
        die(op.context(), opk, kind<real>::name);
    }
}

}  // namespace

void set_split_precision(bool enable) noexcept { g_split = enable; }
bool split_precision() noexcept { return g_split; }

#define SFMM_DEFINE_OPS(NAME, OPK)                                                                                   \
    void NAME(const operator_data<float> &op, threadlocal_buffer<float> &buf, size_t howmany,                       \
              const solid<float> *const *const A, solid<float> *const *const B, const float *x, const float *y,     \
              const float *z)                                                                                        \
    {                                                                                                                \
        classic<float>(OPK, op, buf, howmany, A, B, x, y, z);                                                        \
    }                                                                                                                \
    void NAME(const operator_data<double> &op, threadlocal_buffer<double> &buf, size_t howmany,                     \
              const solid<double> *const *const A, solid<double> *const *const B, const double *x,                   \
              const double *y, const double *z)                                                                      \
    {                                                                                                                \
        classic<double>(OPK, op, buf, howmany, A, B, x, y, z);                                                       \
    }                                                                                                                \
    void NAME(const operator_data<float> &op, threadlocal_buffer<float> &buf, const translation_info<float> *begin, \
              const translation_info<float> *end)                                                                    \
    {                                                                                                                \
        check_buffer(op, buf, OPK);                                                                                  \
        items<float>(OPK, op, begin, end, true);                                                                     \
    }                                                                                                                \
    void NAME(const operator_data<double> &op, threadlocal_buffer<double> &buf,                                     \
              const translation_info<double> *begin, const translation_info<double> *end)                            \
    {                                                                                                                \
        check_buffer(op, buf, OPK);                                                                                  \
        items<double>(OPK, op, begin, end, true);                                                                    \
    }                                                                                                                \
    void NAME##_unchecked(const operator_data<float> &op, threadlocal_buffer<float> &,                              \
                          const translation_info<float> *begin, const translation_info<float> *end) noexcept        \
    {                                                                                                                \
        items<float>(OPK, op, begin, end, false);                                                                    \
    }                                                                                                                \
    void NAME##_unchecked(const operator_data<double> &op, threadlocal_buffer<double> &,                            \
                          const translation_info<double> *begin, const translation_info<double> *end) noexcept      \
    {                                                                                                                \
        items<double>(OPK, op, begin, end, false);                                                                   \
    }

SFMM_DEFINE_OPS(m2m, SFMM_M2M)
SFMM_DEFINE_OPS(m2l, SFMM_M2L)
SFMM_DEFINE_OPS(l2l, SFMM_L2L)
#undef SFMM_DEFINE_OPS

//////////////////////////////////
// multithreaded_translator     //
//////////////////////////////////

template <typename real>
class multithreaded_translator<real>::impl
{
public:
    explicit impl(size_t P) : op(P) {}
    operator_data<real> op;
};

template <typename real>
multithreaded_translator<real>::multithreaded_translator(size_t P) : p{new impl(P)}
{
}

template <typename real>
multithreaded_translator<real>::multithreaded_translator(size_t P, hwloc_topology *topology, cpuset_t *begin,
                                                         cpuset_t *end)
    : p{nullptr}
{
    if (topology == nullptr)
        throw std::runtime_error{"solidfmm::multithreaded_translator: NULL hwloc_topology_t passed to constructor."};
    if (begin == end) throw std::logic_error{"solidfmm::multithreaded_translator: empty set of cpusets."};
    p = new impl(P);
}

template <typename real>
multithreaded_translator<real>::multithreaded_translator(multithreaded_translator &&rhs) noexcept : p{rhs.p}
{
    rhs.p = nullptr;
}

template <typename real>
multithreaded_translator<real> &multithreaded_translator<real>::operator=(multithreaded_translator &&rhs) noexcept
{
    impl *t = p;
    p = rhs.p;
    rhs.p = t;
    return *this;
}

template <typename real>
multithreaded_translator<real>::~multithreaded_translator()
{
    delete p;
}

template <typename real>
void multithreaded_translator<real>::schedule_equally_among_threads() noexcept
{
}

template <typename real>
void multithreaded_translator<real>::schedule_by_measuring_throughput()
{
}

template <typename real>
void multithreaded_translator<real>::m2m(const item *begin, const item *end) const
{
    items<real>(SFMM_M2M, p->op, begin, end, true);
}
template <typename real>
void multithreaded_translator<real>::m2l(const item *begin, const item *end) const
{
    items<real>(SFMM_M2L, p->op, begin, end, true);
}
template <typename real>
void multithreaded_translator<real>::l2l(const item *begin, const item *end) const
{
    items<real>(SFMM_L2L, p->op, begin, end, true);
}
template <typename real>
void multithreaded_translator<real>::m2m_unchecked(const item *begin, const item *end) const noexcept
{
    items<real>(SFMM_M2M, p->op, begin, end, false);
}
template <typename real>
void multithreaded_translator<real>::m2l_unchecked(const item *begin, const item *end) const noexcept
{
    items<real>(SFMM_M2L, p->op, begin, end, false);
}
template <typename real>
void multithreaded_translator<real>::l2l_unchecked(const item *begin, const item *end) const noexcept
{
    items<real>(SFMM_L2L, p->op, begin, end, false);
}

template class multithreaded_translator<float>;
template class multithreaded_translator<double>;

}  // namespace solidfmm
