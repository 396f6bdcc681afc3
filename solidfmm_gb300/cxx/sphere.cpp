// Minimal bounding spheres (the reference's solidfmm/sphere.hpp:29-42,
// sphere.cpp:547-647): the smallest sphere containing a set of points or of
// spheres, on the host.
//
// Method: Welzl's move-to-front recursion over a support set of at most four
// balls.  For a support set S (balls internally tangent to the result) the
// candidate is the smallest ball B = (c, R) with |c - c_j| + r_j = R for
// every j and c in the affine hull of the support centres.  Writing
// c = c_0 + Q lambda (Q = [c_1 - c_0, ...]), subtracting the tangency
// equation of ball 0 from the others leaves the linear system
//     2 Q^T Q lambda = u + R v,  u_j = |d_j|^2 + r_0^2 - r_j^2,
//                               v_j = 2 (r_j - r_0),
// so lambda = alpha + R beta, and ball 0's own equation
// |Q(alpha + R beta)| = R - r_0 becomes a quadratic in R whose smallest root
// R >= max r_j is the radius.  For points (r = 0) this is the circumsphere
// of the support points in their affine hull.  The result is verified
// against every input; a failed verification (degenerate support sets in
// floating point) retries in another order and finally throws
// std::runtime_error, as the reference does when its basis computation fails.
// Arithmetic in FP64 for both element types.
#include <solidfmm/sphere.hpp>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <utility>
#include <vector>

#include "sfmm.h"

namespace solidfmm
{

template struct sphere<float>;
template struct sphere<double>;

namespace
{

struct Ball {
    double c[3];
    double r;
};

double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// k x k system (k <= 3) by Gaussian elimination with partial pivoting; two
// right-hand sides.  false if the matrix is singular relative to its size.
bool solve2(int k, double A[3][3], double *x, double *y)
{
    double scale = 0;
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) scale = std::max(scale, std::fabs(A[i][j]));
    if (!(scale > 0)) return false;
    int perm[3] = {0, 1, 2};
    for (int col = 0; col < k; ++col) {
        int piv = col;
        for (int i = col + 1; i < k; ++i)
            if (std::fabs(A[i][col]) > std::fabs(A[piv][col])) piv = i;
        if (std::fabs(A[piv][col]) <= 1e-13 * scale) return false;
        std::swap(A[piv], A[col]);
        std::swap(x[piv], x[col]);
        std::swap(y[piv], y[col]);
        std::swap(perm[piv], perm[col]);
        for (int i = col + 1; i < k; ++i) {
            const double f = A[i][col] / A[col][col];
            for (int j = col; j < k; ++j) A[i][j] -= f * A[col][j];
            x[i] -= f * x[col];
            y[i] -= f * y[col];
        }
    }
    for (int i = k - 1; i >= 0; --i) {
        for (int j = i + 1; j < k; ++j) {
            x[i] -= A[i][j] * x[j];
            y[i] -= A[i][j] * y[j];
        }
        x[i] /= A[i][i];
        y[i] /= A[i][i];
    }
    return true;
}

// The smallest ball internally tangent to the m support balls with its centre
// in the affine hull of theirs; m = 0 gives the empty ball (radius -1).
bool tangent_ball(const Ball *S, int m, Ball &out)
{
    if (m == 0) {
        out = Ball{{0, 0, 0}, -1.0};
        return true;
    }
    if (m == 1) {
        out = S[0];
        return true;
    }
    const int k = m - 1;
    double d[3][3], A[3][3], u[3], v[3];
    for (int j = 0; j < k; ++j)
        for (int a = 0; a < 3; ++a) d[j][a] = S[j + 1].c[a] - S[0].c[a];
    const double r0 = S[0].r;
    double rmax = r0;
    for (int i = 0; i < k; ++i) {
        for (int j = 0; j < k; ++j) A[i][j] = 2 * dot3(d[i], d[j]);
        const double rj = S[i + 1].r;
        u[i] = dot3(d[i], d[i]) + r0 * r0 - rj * rj;
        v[i] = 2 * (rj - r0);
        rmax = std::max(rmax, rj);
    }
    if (!solve2(k, A, u, v)) return false;  // u <- alpha, v <- beta
    double P[3] = {0, 0, 0}, Qb[3] = {0, 0, 0};
    for (int j = 0; j < k; ++j)
        for (int a = 0; a < 3; ++a) {
            P[a] += u[j] * d[j][a];
            Qb[a] += v[j] * d[j][a];
        }
    // a R^2 + 2 b R + c = 0
    const double qa = dot3(Qb, Qb) - 1, qb = dot3(P, Qb) + r0, qc = dot3(P, P) - r0 * r0;
    double roots[2];
    int nr = 0;
    if (std::fabs(qa) <= 1e-14) {
        if (qb == 0) return false;
        roots[nr++] = -qc / (2 * qb);
    } else {
        double disc = qb * qb - qa * qc;
        if (disc < 0) {
            if (disc < -1e-12 * (qb * qb + std::fabs(qa * qc))) return false;
            disc = 0;
        }
        const double s = std::sqrt(disc);
        const double q = -(qb + (qb >= 0 ? s : -s));
        if (q != 0) {
            roots[nr++] = q / qa;
            roots[nr++] = qc / q;
        } else {
            roots[nr++] = -qb / qa;
        }
    }
    double R = -1;
    const double slack = 1e-12 * (rmax + std::sqrt(dot3(P, P)) + 1e-300);
    for (int i = 0; i < nr; ++i)
        if (roots[i] >= rmax - slack && (R < 0 || roots[i] < R)) R = roots[i];
    if (R < 0) return false;
    R = std::max(R, rmax);
    for (int a = 0; a < 3; ++a) out.c[a] = S[0].c[a] + P[a] + R * Qb[a];
    out.r = R;
    return true;
}

bool contains(const Ball &B, const Ball &X, double tol)
{
    if (B.r < 0) return false;
    const double e[3] = {X.c[0] - B.c[0], X.c[1] - B.c[1], X.c[2] - B.c[2]};
    return std::sqrt(dot3(e, e)) + X.r <= B.r + tol;
}

// Welzl's recursion with move-to-front over L[0, end) and the support set
// sup[0, ns); false when a support set is degenerate.
bool mtf(std::vector<Ball> &L, size_t end, Ball *sup, int ns, Ball &mb, double tol)
{
    if (!tangent_ball(sup, ns, mb)) return false;
    if (ns == 4) return true;
    for (size_t i = 0; i < end; ++i) {
        if (!contains(mb, L[i], tol)) {
            sup[ns] = L[i];
            if (!mtf(L, i, sup, ns + 1, mb, tol)) return false;
            std::rotate(L.begin(), L.begin() + (long)i, L.begin() + (long)i + 1);
        }
    }
    return true;
}

// 0 = ok, 1 = empty input, 2 = unresolved degenerate configuration
int minimal_ball(std::vector<Ball> L, Ball &out)
{
    if (L.empty()) return 1;
    double scale = 0;
    for (const Ball &b : L) scale = std::max(scale, std::sqrt(dot3(b.c, b.c)) + std::fabs(b.r));
    const double tol = 1e-11 * (scale + 1e-300);
    const std::vector<Ball> orig = L;
    uint64_t seed = 0x9E3779B97F4A7C15ull;
    for (int attempt = 0; attempt < 4; ++attempt) {
        Ball sup[4];
        Ball mb;
        if (mtf(L, L.size(), sup, 0, mb, tol)) {
            bool ok = mb.r >= 0;
            for (const Ball &b : orig)
                if (ok && !contains(mb, b, 4 * tol)) ok = false;
            if (ok) {
                out = mb;
                return 0;
            }
        }
        // another order (deterministic shuffle)
        L = orig;
        for (size_t i = L.size(); i > 1; --i) {
            seed ^= seed << 13;
            seed ^= seed >> 7;
            seed ^= seed << 17;
            std::swap(L[i - 1], L[seed % i]);
        }
    }
    return 2;
}

template <typename real>
sphere<real> points_impl(size_t n, const real *x, const real *y, const real *z)
{
    if (n == 0 || !x || !y || !z) throw std::logic_error("solidfmm::bounding_sphere: empty set of points");
    std::vector<Ball> L(n);
    for (size_t i = 0; i < n; ++i) L[i] = Ball{{(double)x[i], (double)y[i], (double)z[i]}, 0.0};
    Ball b;
    if (minimal_ball(std::move(L), b))
        throw std::runtime_error("solidfmm::bounding_sphere: degenerate configuration of points");
    return sphere<real>{(real)b.c[0], (real)b.c[1], (real)b.c[2], (real)b.r};
}

template <typename real>
sphere<real> spheres_impl(const sphere<real> *begin, const sphere<real> *end)
{
    if (!begin || !end || end <= begin) throw std::logic_error("solidfmm::bounding_sphere: empty set of spheres");
    std::vector<Ball> L;
    L.reserve((size_t)(end - begin));
    for (const sphere<real> *s = begin; s != end; ++s) L.push_back(Ball{{(double)s->x, (double)s->y, (double)s->z}, (double)s->r});
    Ball b;
    if (minimal_ball(std::move(L), b))
        throw std::runtime_error("solidfmm::bounding_sphere: degenerate configuration of spheres");
    return sphere<real>{(real)b.c[0], (real)b.c[1], (real)b.c[2], (real)b.r};
}

}  // namespace

sphere<float> bounding_sphere(size_t n, const float *x, const float *y, const float *z)
{
    return points_impl(n, x, y, z);
}
sphere<double> bounding_sphere(size_t n, const double *x, const double *y, const double *z)
{
    return points_impl(n, x, y, z);
}
sphere<float> bounding_sphere(const sphere<float> *begin, const sphere<float> *end) { return spheres_impl(begin, end); }
sphere<double> bounding_sphere(const sphere<double> *begin, const sphere<double> *end)
{
    return spheres_impl(begin, end);
}

}  // namespace solidfmm

extern "C" int sfmm_bounding_sphere(size_t n, const double *x, const double *y, const double *z, const double *r,
                                    double *out)
{
    using namespace solidfmm;
    if (n == 0 || !x || !y || !z || !out) return SFMM_INVALID_ARG;
    try {
        std::vector<Ball> L(n);
        for (size_t i = 0; i < n; ++i) L[i] = Ball{{x[i], y[i], z[i]}, r ? r[i] : 0.0};
        Ball b;
        const int st = minimal_ball(std::move(L), b);
        if (st) return st == 1 ? SFMM_INVALID_ARG : SFMM_UNSUPPORTED;
        out[0] = b.c[0];
        out[1] = b.c[1];
        out[2] = b.c[2];
        out[3] = b.r;
        return SFMM_OK;
    } catch (...) {
        return SFMM_OOM;
    }
}
