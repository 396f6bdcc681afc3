// Drop-in check of the C++ API: a program written against solidfmm's public
// headers (solid, harmonics, handles, translations) that translates
// expansions on the GPU and checks the physics against the exact potential
// 1/|x - y| and its gradient, plus the reference's error behaviour.
// Exit status 0 = all checks passed.
#include <solidfmm/handles.hpp>
#include <solidfmm/harmonics.hpp>
#include <solidfmm/operator_data.hpp>
#include <solidfmm/solid.hpp>
#include <solidfmm/threadlocal_buffer.hpp>
#include <solidfmm/translations.hpp>

#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <vector>

using namespace solidfmm;
using harmonics::dR;
using harmonics::R;
using harmonics::S;

static int failures = 0;

static void check(bool ok, const char *what, double v = 0, double lim = 0)
{
    std::printf("%-60s %s  (%.3e vs %.3e)\n", what, ok ? "ok" : "FAIL", v, lim);
    if (!ok) ++failures;
}

// M2L through the classic overload: 32 identical translations into one target
template <typename real>
double m2l_error(size_t P, double *grad_err)
{
    const real xs = 1.1, ys = 0.2, zs = 0.9;  // source
    const real xa = 1, ya = 0, za = 1;        // multipole centre
    const real xb = 0.3, yb = 0.1, zb = 2;    // local centre
    const real x = 0.1, y = 0.2, z = 2.5;     // evaluation point
    const real r = std::sqrt((x - xs) * (x - xs) + (y - ys) * (y - ys) + (z - zs) * (z - zs));
    solid<real> M = R<real>(P, xs - xa, ys - ya, zs - za);
    solid<real> L(P);
    operator_handle<real> op(P);
    buffer_handle<real> buf(op);
    std::vector<const solid<real> *> Mp(32, &M);
    std::vector<solid<real> *> Lp(32, &L);
    std::vector<real> dx(32, xb - xa), dy(32, yb - ya), dz(32, zb - za);
    m2l(op, buf, 32, Mp.data(), Lp.data(), dx.data(), dy.data(), dz.data());
    real phi;
    dot(L, R<real>(P, x - xb, y - yb, z - zb), &phi);
    phi /= 32;
    real g[3];
    dot(L, dR<real>(P, x - xb, y - yb, z - zb), g);
    const real ex[3] = {-(x - xs) / (r * r * r), -(y - ys) / (r * r * r), -(z - zs) / (r * r * r)};
    double gn = 0, ge = 0;
    for (int k = 0; k < 3; ++k) {
        ge += std::pow(g[k] / 32 - ex[k], 2);
        gn += ex[k] * ex[k];
    }
    *grad_err = std::sqrt(ge / gn);
    return r * std::fabs(phi - 1 / r);
}

// M2M then evaluation far away, through multithreaded_translator items
template <typename real>
double m2m_error(size_t P)
{
    const real xs = 0.2, ys = -0.1, zs = 0.15, xa = 0, ya = 0, za = 0, xb = 0.5, yb = 0.5, zb = 0.5;
    const real x = 4, y = -3, z = 2.5;
    solid<real> M = R<real>(P, xs - xa, ys - ya, zs - za);
    solid<real> M2(P);
    multithreaded_translator<real> tr(P);
    translation_info<real> it{&M, &M2, xb - xa, yb - ya, zb - za};
    tr.m2m(&it, &it + 1);
    real phi;
    dot(M2, S<real>(P, x - xb, y - yb, z - zb), &phi);
    const real r = std::sqrt((x - xs) * (x - xs) + (y - ys) * (y - ys) + (z - zs) * (z - zs));
    return r * std::fabs(phi - 1 / r);
}

// L2L: local expansion of a far source, shifted to a nearby centre
template <typename real>
double l2l_error(size_t P)
{
    const real xs = 3, ys = 2, zs = -2.5, xa = 0, ya = 0, za = 0, xb = 0.25, yb = -0.25, zb = 0.25;
    const real x = 0.35, y = -0.1, z = 0.3;
    solid<real> La = S<real>(P, xs - xa, ys - ya, zs - za);
    solid<real> Lb(P);
    operator_data<real> op(P);
    threadlocal_buffer<real> buf(op);
    translation_info<real> it{&La, &Lb, xb - xa, yb - ya, zb - za};
    l2l(op, buf, &it, &it + 1);
    real phi;
    dot(Lb, R<real>(P, x - xb, y - yb, z - zb), &phi);
    const real r = std::sqrt((x - xs) * (x - xs) + (y - ys) * (y - ys) + (z - zs) * (z - zs));
    return r * std::fabs(phi - 1 / r);
}

int main()
{
    char msg[128];
    double g;
    const double m2l_lim[][2] = {{4, 2e-2}, {10, 2e-4}, {16, 1e-6}, {30, 1e-9}, {40, 1e-10}};
    for (auto &c : m2l_lim) {
        double e = m2l_error<double>((size_t)c[0], &g);
        std::snprintf(msg, sizeof msg, "double M2L P=%d potential", (int)c[0]);
        check(e < c[1], msg, e, c[1]);
        std::snprintf(msg, sizeof msg, "double M2L P=%d gradient", (int)c[0]);
        check(g < 50 * c[1], msg, g, 50 * c[1]);
    }
    {
        double e = m2l_error<float>(10, &g);
        check(e < 1e-3, "float M2L P=10 potential", e, 1e-3);
    }
    for (size_t P : {6, 12, 20}) {
        double e = m2m_error<double>(P);
        std::snprintf(msg, sizeof msg, "double M2M P=%zu potential", P);
        check(e < std::pow(0.25, (double)P) * 10, msg, e, std::pow(0.25, (double)P) * 10);
        e = l2l_error<double>(P);
        std::snprintf(msg, sizeof msg, "double L2L P=%zu potential", P);
        check(e < std::pow(0.2, (double)P) * 10, msg, e, std::pow(0.2, (double)P) * 10);
    }
    // split precision moves the potential error by far less than its 1e-7
    // contract on the expansions
    {
        double gp, gs;
        double ep = m2l_error<double>(16, &gp);
        set_split_precision(true);
        double es = m2l_error<double>(16, &gs);
        set_split_precision(false);
        check(std::fabs(ep - es) < 1e-8, "split vs plain M2L P=16", std::fabs(ep - es), 1e-8);
    }
    // error behaviour of the reference (checked variants throw before touching anything)
    bool threw = false;
    try {
        operator_handle<double> bad(0);
    } catch (const std::logic_error &) {
        threw = true;
    }
    check(threw, "operator_handle(0) throws logic_error");
    threw = false;
    try {
        operator_handle<float> bad(19);
    } catch (const std::overflow_error &) {
        threw = true;
    }
    check(threw, "operator_handle<float>(19) throws overflow_error");
    {
        operator_handle<double> op(8);
        buffer_handle<double> buf(op);
        solid<double> M = R<double>(10, 0.1, 0.2, 0.3), L(8);
        L.re(0, 0) = 42;
        const solid<double> *Mp = &M;
        solid<double> *Lp = &L;
        double x = 3, y = 0, z = 0;
        threw = false;
        try {
            m2l(op, buf, 1, &Mp, &Lp, &x, &y, &z);
        } catch (const std::out_of_range &) {
            threw = true;
        }
        check(threw && L.re(0, 0) == 42, "order above operator order: out_of_range, target untouched");
        solid<double> M2(8, 2);
        Mp = &M2;
        threw = false;
        try {
            m2l(op, buf, 1, &Mp, &Lp, &x, &y, &z);
        } catch (const std::logic_error &) {
            threw = true;
        }
        check(threw, "dimension mismatch throws logic_error");
        buffer_handle<double> empty;
        solid<double> M3(8);
        Mp = &M3;
        threw = false;
        try {
            m2l(op, empty, 1, &Mp, &Lp, &x, &y, &z);
        } catch (const std::logic_error &) {
            threw = true;
        }
        check(threw, "incompatible buffer throws logic_error");
    }
    // dimension > 1: components translate independently
    {
        const size_t P = 10;
        solid<double> M(P, 2), L(P, 2), L0(P), L1(P);
        solid<double> a = R<double>(P, 0.1, -0.2, 0.3), b = R<double>(P, -0.3, 0.1, 0.2);
        for (size_t k = 0; k < P * (P + 1); ++k) {
            M.memptr()[k] = a.memptr()[k];
            M.memptr()[P * (P + 1) + k] = b.memptr()[k];
        }
        operator_handle<double> op(P);
        buffer_handle<double> buf(op);
        translation_info<double> it[3] = {{&M, &L, 2, 1, -2}, {&a, &L0, 2, 1, -2}, {&b, &L1, 2, 1, -2}};
        m2l(op, buf, it, it + 3);
        double d = 0;
        for (size_t k = 0; k < P * (P + 1); ++k)
            d = std::fmax(d, std::fabs(L.memptr()[k] - L0.memptr()[k]) +
                                 std::fabs(L.memptr()[P * (P + 1) + k] - L1.memptr()[k]));
        check(d < 1e-12 * std::fabs(L0.re(0, 0)), "dim=2 components translate independently", d, 0);
    }
    std::printf("%d failure(s)\n", failures);
    return failures ? 1 : 0;
}
