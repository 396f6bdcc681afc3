// Solid harmonics R, S and their gradients for the drop-in API.
//
// The recurrences are Dehnen's (doc/solidfmm.tex:1076-1093; the reference
// evaluates them in solidfmm/harmonics.cpp:32-224): diagonal, sub-diagonal,
// then a three-term recurrence in n for every m.  One template evaluates
// them over a number type that is either a plain real or a real carrying its
// three partial derivatives, so the gradients dR, dS (harmonics.cpp:82-174,
// 227-349) come from the same recurrence by forward differentiation.
#include <solidfmm/harmonics.hpp>
#include <solidfmm/solid.hpp>

#include <cmath>

namespace solidfmm
{
namespace harmonics
{
namespace
{

// value and gradient (d/dx, d/dy, d/dz)
template <typename real>
struct grad3 {
    real v, g[3];
    grad3(real v_ = 0, real gx = 0, real gy = 0, real gz = 0) : v(v_), g{gx, gy, gz} {}
};
template <typename real>
grad3<real> operator+(const grad3<real> &a, const grad3<real> &b)
{
    return {a.v + b.v, a.g[0] + b.g[0], a.g[1] + b.g[1], a.g[2] + b.g[2]};
}
template <typename real>
grad3<real> operator-(const grad3<real> &a, const grad3<real> &b)
{
    return {a.v - b.v, a.g[0] - b.g[0], a.g[1] - b.g[1], a.g[2] - b.g[2]};
}
template <typename real>
grad3<real> operator*(const grad3<real> &a, const grad3<real> &b)
{
    return {a.v * b.v, a.g[0] * b.v + a.v * b.g[0], a.g[1] * b.v + a.v * b.g[1], a.g[2] * b.v + a.v * b.g[2]};
}
template <typename real>
grad3<real> operator*(real s, const grad3<real> &a)
{
    return {s * a.v, s * a.g[0], s * a.g[1], s * a.g[2]};
}

template <typename real>
real value(real a) { return a; }
template <typename real>
real value(const grad3<real> &a) { return a.v; }

template <typename num, typename real>
num scal(real s) { return num(s); }

// Evaluates R (singular = false) or S (singular = true) for all n < P,
// 0 <= m <= n, calling put(n, m, re, im) for every coefficient.
template <typename num, typename real, typename Put>
void recurrence(size_t P, bool singular, const num &x, const num &y, const num &z, Put put)
{
    if (P == 0) return;
    const num r2 = x * x + y * y + z * z;
    num inv2;
    num d_re, d_im;  // diagonal coefficient (m, m)
    if (singular) {
        const real r2v = value<real>(r2);
        const real inv = real(1) / r2v;
        // d(1/r2) = -(1/r2)^2 d(r2); d(1/r) = -(1/2) (1/r)^3 d(r2)
        inv2 = r2;
        inv2.v = inv;
        for (int k = 0; k < 3; ++k) inv2.g[k] = -inv * inv * r2.g[k];
        const real s = std::sqrt(inv);
        d_re = r2;
        d_re.v = s;
        for (int k = 0; k < 3; ++k) d_re.g[k] = real(-0.5) * s * inv * r2.g[k];
    } else {
        d_re = num(real(1));
    }
    d_im = num(real(0));
    for (size_t m = 0; m < P; ++m) {
        if (m > 0) {
            // R: (x+iy)/(2m) R(m-1,m-1);  S: (2m-1)(x+iy)/r^2 S(m-1,m-1)
            num nr = d_re * x - d_im * y;
            num ni = d_re * y + d_im * x;
            if (singular) {
                nr = real(2 * m - 1) * (nr * inv2);
                ni = real(2 * m - 1) * (ni * inv2);
            } else {
                nr = (real(1) / real(2 * m)) * nr;
                ni = (real(1) / real(2 * m)) * ni;
            }
            d_re = nr;
            d_im = ni;
        }
        put(m, m, d_re, d_im);
        num ar = d_re, ai = d_im, br = num(real(0)), bi = num(real(0));
        for (size_t n = m + 1; n < P; ++n) {
            num cr, ci;
            if (singular) {
                if (n == m + 1) {
                    cr = real(2 * m + 1) * (z * inv2 * ar);
                    ci = real(2 * m + 1) * (z * inv2 * ai);
                } else {
                    const real c2 = real(n + m - 1) * real(n - m - 1);
                    cr = (real(2 * n - 1) * (z * ar) - c2 * br) * inv2;
                    ci = (real(2 * n - 1) * (z * ai) - c2 * bi) * inv2;
                }
            } else {
                if (n == m + 1) {
                    cr = z * ar;
                    ci = z * ai;
                } else {
                    const real f = real(1) / (real(n + m) * real(n - m));
                    cr = f * (real(2 * n - 1) * (z * ar) - r2 * br);
                    ci = f * (real(2 * n - 1) * (z * ai) - r2 * bi);
                }
            }
            put(n, m, cr, ci);
            br = ar;
            bi = ai;
            ar = cr;
            ai = ci;
        }
    }
}

template <typename real>
solid<real> eval(size_t P, real x, real y, real z, bool singular)
{
    if (P == 0) return solid<real>{};
    solid<real> out(P);
    recurrence<grad3<real>, real>(P, singular, grad3<real>(x), grad3<real>(y), grad3<real>(z),
                                  [&](size_t n, size_t m, const grad3<real> &re, const grad3<real> &im) {
                                      out.re(n, m) = re.v;
                                      out.im(n, m) = im.v;
                                  });
    return out;
}

template <typename real>
solid<real> eval_grad(size_t P, real x, real y, real z, bool singular)
{
    solid<real> out(P, 3);
    if (P == 0) return out;
    recurrence<grad3<real>, real>(P, singular, grad3<real>(x, 1, 0, 0), grad3<real>(y, 0, 1, 0),
                                  grad3<real>(z, 0, 0, 1),
                                  [&](size_t n, size_t m, const grad3<real> &re, const grad3<real> &im) {
                                      for (size_t d = 0; d < 3; ++d) {
                                          out.re(n, m, d) = re.g[d];
                                          out.im(n, m, d) = im.g[d];
                                      }
                                  });
    return out;
}

}  // namespace

template <> solid<float> R(size_t P, float x, float y, float z) { return eval<float>(P, x, y, z, false); }
template <> solid<float> S(size_t P, float x, float y, float z) { return eval<float>(P, x, y, z, true); }
template <> solid<float> dR(size_t P, float x, float y, float z) { return eval_grad<float>(P, x, y, z, false); }
template <> solid<float> dS(size_t P, float x, float y, float z) { return eval_grad<float>(P, x, y, z, true); }
template <> solid<double> R(size_t P, double x, double y, double z) { return eval<double>(P, x, y, z, false); }
template <> solid<double> S(size_t P, double x, double y, double z) { return eval<double>(P, x, y, z, true); }
template <> solid<double> dR(size_t P, double x, double y, double z) { return eval_grad<double>(P, x, y, z, false); }
template <> solid<double> dS(size_t P, double x, double y, double z) { return eval_grad<double>(P, x, y, z, true); }

}  // namespace harmonics
}  // namespace solidfmm
