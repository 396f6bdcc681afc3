// P2M / P2L expansion building and order bucketing.
//
// P2M/P2L: out[j] += sum_k q_jk * R(x_jk - c_j) (or S), the reference's
// fmadd(q, harmonics::R/S(P, x - c), E) (solid.cpp:70-104) with the R and S
// recurrences of harmonics.cpp:32-80 and :177-224, evaluated column by column
// (fixed m, increasing n) so that each coefficient is accumulated as soon as
// it is produced.  Orders up to 32: float-float arithmetic on the FP32 pipe,
// lanes owning column pairs (k_p2x_ff); above, one FP64 thread per expansion.
//
// Bucketing: a counting sort of translation indices by the key
// (p_in, p_out), so that warps see uniform orders.
#include <algorithm>
#include <cstdint>
#include <map>
#include <mutex>

#include "sfmm.h"
#include "sfmm_arith.cuh"
#include "sfmm_launch.hpp"

namespace sfmm {

// Expansion j takes particles [j nq, (j+1) nq), or [offset[j], offset[j+1])
// when an offset array is given (ragged leaves).
template <class Out>
__global__ void k_p2x(int kind, int P, long long nexp, long long nq, const uint32_t *__restrict__ offset,
                      const double *__restrict__ q, const double *__restrict__ pos,
                      const double *__restrict__ centre, Out *out, long long stride)
{
    long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= nexp) return;
    Out *o = out + j * stride;
    const double cx = centre[3 * j], cy = centre[3 * j + 1], cz = centre[3 * j + 2];
    const long long k0 = offset ? (long long)offset[j] : j * nq;
    const long long k1 = offset ? (long long)offset[j + 1] : (j + 1) * nq;
    for (long long k = k0; k < k1; ++k) {
        const double w = q[k];
        const double *pp = pos + 3 * k;
        const double x = pp[0] - cx, y = pp[1] - cy, z = pp[2] - cz;
        const double r2 = x * x + y * y + z * z;
        if (kind == 0) {
            // regular harmonics R
            double dr = 1.0, di = 0.0;  // R(m,m)
            for (int m = 0; m < P; ++m) {
                if (m > 0) {
                    double f = (m == 1) ? 0.5 : 1.0 / (2.0 * m);
                    double nr = (dr * x - di * y) * f;
                    double ni = (dr * y + di * x) * f;
                    dr = nr;
                    di = ni;
                }
                // column m: R(m,m), R(m+1,m) = z R(m,m), then the three-term recurrence
                double ar = dr, ai = di;            // R(n-1,m)
                double br = 0.0, bi = 0.0;          // R(n-2,m)
                o[m * (m + 1) + m] += (Out)(w * ar);
                o[(m + 1) * (m + 1) + m] += (Out)(w * ai);
                for (int n = m + 1; n < P; ++n) {
                    double cr, ci;
                    if (n == m + 1) {
                        cr = z * ar;
                        ci = z * ai;
                    } else {
                        double f = 1.0 / ((double)(n + m) * (double)(n - m));
                        cr = (ar * z * (2 * n - 1) - r2 * br) * f;
                        ci = (ai * z * (2 * n - 1) - r2 * bi) * f;
                    }
                    o[n * (n + 1) + m] += (Out)(w * cr);
                    o[(n + 1) * (n + 1) + m] += (Out)(w * ci);
                    br = ar;
                    bi = ai;
                    ar = cr;
                    ai = ci;
                }
            }
        } else {
            // singular harmonics S
            const double r2inv = 1.0 / r2;
            double dr = sqrt(r2inv), di = 0.0;  // S(m,m)
            for (int m = 0; m < P; ++m) {
                if (m > 0) {
                    double f = (2.0 * m - 1.0) * r2inv;
                    double nr = (dr * x - di * y) * f;
                    double ni = (dr * y + di * x) * f;
                    dr = nr;
                    di = ni;
                }
                double ar = dr, ai = di, br = 0.0, bi = 0.0;
                o[m * (m + 1) + m] += (Out)(w * ar);
                o[(m + 1) * (m + 1) + m] += (Out)(w * ai);
                for (int n = m + 1; n < P; ++n) {
                    double cr, ci;
                    if (n == m + 1) {
                        double f = (2.0 * m + 1.0) * z * r2inv;
                        cr = f * ar;
                        ci = f * ai;
                    } else {
                        double c2 = (double)(n + m - 1) * (double)(n - m - 1);
                        cr = (ar * z * (2 * n - 1) - c2 * br) * r2inv;
                        ci = (ai * z * (2 * n - 1) - c2 * bi) * r2inv;
                    }
                    o[n * (n + 1) + m] += (Out)(w * cr);
                    o[(n + 1) * (n + 1) + m] += (Out)(w * ci);
                    br = ar;
                    bi = ai;
                    ar = cr;
                    ai = ci;
                }
            }
        }
    }
}

// ---- float-float P2M / P2L for order bounds up to 32 ----
//
// The same sums on the FP32 pipe.  Coordinates are scaled by a power of two
// rho per expansion (x' = (x - c) / rho, |x'| <= 1 for P2M from the farthest
// charge, |x'| >= 1 for P2L from the nearest) and the columns run on the
// Schmidt-normalised harmonics
//     T_n^m = R_n^m(x') sig(n,m),  U_n^m = S_n^m(x') / sig(n,m),
//     sig(n,m) = sqrt((n+m)! (n-m)!),
// which are bounded by |x'|^n and |x'|^-(n+1), so that no intermediate leaves
// the FP32 range at any order here.  Both obey one recurrence,
//     X_m^m     = d_m v X_{m-1}^{m-1},  d_m = sqrt((2m-1)/(2m)),
//     X_n^m     = a(n,m) zeta X_{n-1}^m - b(n,m) eta X_{n-2}^m,
//     a(n,m)    = (2n-1) / sqrt((n+m)(n-m)),
//     b(n,m)    = sqrt((n+m-1)(n-m-1) / ((n+m)(n-m))),
// with v = x'+iy', zeta = z', eta = |x'|^2 for T (X_0^0 = 1) and
// v = (x'+iy')/|x'|^2, zeta = z'/|x'|^2, eta = 1/|x'|^2 for U (X_0^0 = 1/|x'|):
// harmonics.cpp:32-80 (R) and :177-224 (S) with the normalisation folded into
// the coefficients.  The sums come back to the reference's harmonics once per
// expansion, in FP64: R_n^m(x) = rho^n T / sig, S_n^m(x) = sig U / rho^(n+1).
//
// LP lanes per expansion (LP a power of two, LP <= P <= 2 LP): lane l owns
// columns m1 = l and m2 = P-1-l (one column when they coincide, none when
// m1 > m2), P + 1 harmonics at most per lane.  A chunk of LP charges is
// prepared one per lane (shift, scale, conversion to float-float) and
// broadcast by shuffles; the diagonals v^m come from a prefix product across
// the lanes; the harmonics accumulate in registers and are added to the
// expansion once.
constexpr int kP2xColsMax = 32;

// Tables, evaluated at compile time in FP64: coefficient pairs [s][m] for
// n = m + s as (a.hi, a.lo, b.hi, b.lo), the diagonal constants
// d_1 ... d_m as float-float, and at n(n+1)/2 + m: sig(n, m) and 1/sig(n, m),
// sig as fs 2^se with fs in [1, 2) and fi = 1/fs (float-float), and the
// ratios sig(n+1, m')/sig(n, m) for m' = m, m+1, m-1 (float-float).
constexpr int kP2xNC = kP2xColsMax * (kP2xColsMax + 1) / 2;
struct P2xTables {
    float4 ab[kP2xColsMax][kP2xColsMax];
    float2 diag[kP2xColsMax];
    double sig[kP2xNC];
    double isig[kP2xNC];
    int se[kP2xNC];
    float2 fs[kP2xNC], fi[kP2xNC];
    float2 cz[kP2xNC], cp[kP2xNC], cm[kP2xNC];
};

namespace p2x_tables {
constexpr double csqrt(double x)
{
    if (!(x > 0)) return 0.0;
    double f = 1.0;
    while (x > 4.0) {  // exact rescaling into [1/4, 4]
        x *= 0.25;
        f *= 2.0;
    }
    while (x < 0.25) {
        x *= 4.0;
        f *= 0.5;
    }
    double r = 1.0;
    for (int i = 0; i < 12; ++i) r = 0.5 * (r + x / r);
    return r * f;
}
constexpr float2 split(double v)
{
    const float h = (float)v;
    return float2{h, (float)(v - (double)h)};
}
constexpr double fact(int k)
{
    double f = 1.0;
    for (int i = 2; i <= k; ++i) f *= i;
    return f;
}
constexpr P2xTables make()
{
    P2xTables t{};
    double dm = 1.0;  // product of (2i-1)/(2i), i <= m
    for (int m = 0; m < kP2xColsMax; ++m) {
        if (m > 0) dm *= (double)(2 * m - 1) / (double)(2 * m);
        t.diag[m] = split(csqrt(dm));
        for (int n = m; n < kP2xColsMax; ++n) {
            const int s = n - m;
            if (s >= 1) {
                const double nm = (double)(n + m) * (double)(n - m);
                const float2 a = split((double)(2 * n - 1) / csqrt(nm));
                const float2 b = split(csqrt((double)(n + m - 1) * (double)(n - m - 1) / nm));
                t.ab[s][m] = float4{a.x, a.y, b.x, b.y};
            }
            const int ix = n * (n + 1) / 2 + m;
            const double sg = csqrt(fact(n + m) * fact(n - m));
            t.sig[ix] = sg;
            t.isig[ix] = 1.0 / sg;
            double f = sg;  // sig = f 2^e, f in [1, 2) (exact halvings)
            int e = 0;
            while (f >= 2.0) {
                f *= 0.5;
                ++e;
            }
            t.se[ix] = e;
            t.fs[ix] = split(f);
            t.fi[ix] = split(1.0 / f);
            t.cz[ix] = split(csqrt((double)(n + 1 + m) * (double)(n + 1 - m)));
            t.cp[ix] = split(csqrt((double)(n + m + 1) * (double)(n + m + 2)));
            t.cm[ix] = split(m > 0 ? csqrt((double)(n - m + 1) * (double)(n - m + 2)) : 0.0);
        }
    }
    return t;
}
}  // namespace p2x_tables

__device__ const P2xTables kP2xTab = p2x_tables::make();

struct cpx_ff {
    ff r, i;
};
__device__ __forceinline__ ff ff_shfl(ff a, int src, int width)
{
    return ff{__shfl_sync(0xffffffffu, a.hi, src, width), __shfl_sync(0xffffffffu, a.lo, src, width)};
}
__device__ __forceinline__ cpx_ff cpx_ff_shfl(cpx_ff a, int src, int width)
{
    return cpx_ff{ff_shfl(a.r, src, width), ff_shfl(a.i, src, width)};
}

// a x - b y with one renormalisation (19 FP32 operations)
__device__ __forceinline__ ff ff_fms2(ff a, ff x, ff b, ff y)
{
    const float p = __fmul_rn(a.hi, x.hi);
    float e = __fmaf_rn(a.hi, x.hi, -p);
    e = __fmaf_rn(a.hi, x.lo, e);
    e = __fmaf_rn(a.lo, x.hi, e);
    const float q = __fmul_rn(b.hi, y.hi);
    float f = __fmaf_rn(b.hi, y.hi, -q);
    f = __fmaf_rn(b.hi, y.lo, f);
    f = __fmaf_rn(b.lo, y.hi, f);
    // TwoSum(p, -q)
    const float s = __fsub_rn(p, q);
    const float v = __fsub_rn(s, p);
    const float t = __fsub_rn(__fsub_rn(p, __fsub_rn(s, v)), __fadd_rn(q, v));
    return ff_norm(s, __fadd_rn(t, __fsub_rn(e, f)));
}

__device__ __forceinline__ cpx_ff cpx_ff_mul(cpx_ff a, cpx_ff b)
{
    return cpx_ff{ff_fms2(a.r, b.r, a.i, b.i), ff_fms2(a.r, b.i, ff{-a.i.hi, -a.i.lo}, b.r)};
}

// acc += x, the rounding error of the high words kept in the low word
__device__ __forceinline__ void ffacc_add(ffacc &a, ff x)
{
    const float s = __fadd_rn(a.hi, x.hi);
    const float v = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(x.hi, v));
    a.hi = s;
    a.lo = __fadd_rn(a.lo, __fadd_rn(e, x.lo));
}


// exponent of the largest component of (x, y, z): |x - c| lies in
// [2^e, 2^(e+2)) (sqrt(3) 2^(e+1) < 2^(e+2)); -2^20 for the zero vector
__device__ __forceinline__ int max_exp3(double x, double y, double z)
{
    return max(exp_of(x), max(exp_of(y), exp_of(z)));
}

// A lane's two columns as one run of P + 1 harmonics: column m1 at t < len1
// (t = n - m1), then column m2 at t = len1 + n - m2.  X starts at each
// diagonal (dg1, dg2) and follows the recurrence; the values of the window
// T0 <= t < T0 + NT are added to acc[t - T0].  ab: this block's coefficient
// table.
template <int T0, int NT>
__device__ __forceinline__ void p2x_columns_ff(const float4 *ab, int m1, int len1, int m2, int tot, cpx_ff dg1,
                                               cpx_ff dg2, ff zeta, ff eta, ffacc (&ar)[NT], ffacc (&ai)[NT])
{
    cpx_ff x1 = dg1, x2 = cpx_ff{ff{0.f, 0.f}, ff{0.f, 0.f}};
#pragma unroll
    for (int t = 0; t < T0 + NT; ++t) {
        if (t >= tot) break;
        if (t > 0) {
            const bool second = t >= len1;
            const int m = second ? m2 : m1, s = second ? t - len1 : t;
            const float4 c = ab[(s > 0 ? s : 1) * kP2xColsMax + m];
            const ff A = ff_mul(ff{c.x, c.y}, zeta), B = ff_mul(ff{c.z, c.w}, eta);
            cpx_ff x = cpx_ff{ff_fms2(A, x1.r, B, x2.r), ff_fms2(A, x1.i, B, x2.i)};
            if (s == 0) {  // the second column's diagonal
                x = dg2;
                x1 = cpx_ff{ff{0.f, 0.f}, ff{0.f, 0.f}};
            }
            x2 = x1;
            x1 = x;
        }
        if (t >= T0) {
            ffacc_add(ar[t - T0], x1.r);
            ffacc_add(ai[t - T0], x1.i);
        }
    }
}

template <class Out>
__device__ __forceinline__ void p2x_put(Out *o, int kind, int sh, int n, int m, ffacc re, ffacc im)
{
    const int t = n * (n + 1) / 2 + m;
    const double f = kind == 0 ? ldexp(kP2xTab.isig[t], sh * n) : ldexp(kP2xTab.sig[t], -sh * (n + 1));
    o[n * (n + 1) + m] += (Out)(((double)re.hi + (double)re.lo) * f);
    o[(n + 1) * (n + 1) + m] += (Out)(((double)im.hi + (double)im.lo) * f);
}

// Harmonics T0 .. T0 + NT - 1 of every lane's run (NT = 2 LP + 1 covers all
// of them; orders above 24 take two windows, two launches, to stay within
// the registers).
template <class Out, int LP, int T0, int NT>
__global__ void __launch_bounds__(128) k_p2x_ff(int kind, int P, long long nexp, long long nq,
                                                const uint32_t *__restrict__ offset, const double *__restrict__ q,
                                                const double *__restrict__ pos, const double *__restrict__ centre,
                                                Out *out, long long stride)
{
    __shared__ float4 ab[kP2xColsMax * kP2xColsMax];
    for (int i = threadIdx.x; i < P * kP2xColsMax; i += blockDim.x) ab[i] = (&kP2xTab.ab[0][0])[i];
    __syncthreads();

    const int l = threadIdx.x % LP;
    const long long j = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / LP;
    const bool live = j < nexp;
    const int m1 = l, m2 = P - 1 - l;  // 0 <= m2 < P
    const int len1 = (live && m1 <= m2) ? P - m1 : 0;
    const int tot = len1 + ((live && m1 < m2) ? P - m2 : 0);
    long long kb = 0, cnt = 0;
    double cx = 0, cy = 0, cz = 0;
    if (live) {
        kb = offset ? (long long)offset[j] : j * nq;
        cnt = (offset ? (long long)offset[j + 1] : (j + 1) * nq) - kb;
        cx = centre[3 * j];
        cy = centre[3 * j + 1];
        cz = centre[3 * j + 2];
    }
    // rho = 2^sc: the largest (P2M) or smallest (P2L) distance of the
    // expansion's charges rounded to a power of two, up (P2M) or down (P2L)
    // from the components' exponents, so any double scale works: rho =
    // 2^(e+2) over the largest component's e (P2M: |x'| < 1) or 2^e over the
    // smallest of the charges' largest components (P2L: |x'| >= 1)
    const int kNone = -(1 << 20);
    int ext = kind == 0 ? kNone : (1 << 20);
    for (long long it = l; it < cnt; it += LP) {
        const double *pp = pos + 3 * (kb + it);
        const int e3 = max_exp3(pp[0] - cx, pp[1] - cy, pp[2] - cz);
        if (e3 != kNone) ext = kind == 0 ? max(ext, e3) : min(ext, e3);
    }
    for (int d = LP / 2; d > 0; d >>= 1) {
        const int o = __shfl_xor_sync(0xffffffffu, ext, d, LP);
        ext = kind == 0 ? max(ext, o) : min(ext, o);
    }
    const int sh = ext == kNone || ext == (1 << 20) ? 0 : (kind == 0 ? ext + 2 : ext);  // log2 rho

    ffacc ar[NT], ai[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) ar[t] = ai[t] = ffacc{0.f, 0.f};
    const ff d1 = ff{kP2xTab.diag[m1].x, kP2xTab.diag[m1].y}, d2 = ff{kP2xTab.diag[m2].x, kP2xTab.diag[m2].y};
    const int e = P - LP;  // 0 <= e <= LP

    // chunk loop bound uniform over the warp (the shuffles need every lane)
    const unsigned cntw = __reduce_max_sync(0xffffffffu, (unsigned)cnt);
    for (unsigned c0 = 0; c0 < cntw; c0 += LP) {
        // this lane's charge of the chunk
        ff zeta{0.f, 0.f}, eta{0.f, 0.f}, w{0.f, 0.f};
        cpx_ff v{ff{0.f, 0.f}, ff{0.f, 0.f}};
        if (c0 + l < cnt) {
            const long long k = kb + c0 + l;
            const double *pp = pos + 3 * k;
            const ff x = ff_from_d_scaled(pp[0] - cx, -sh), y = ff_from_d_scaled(pp[1] - cy, -sh),
                     z = ff_from_d_scaled(pp[2] - cz, -sh);
            const ff r2 = ff_add(ff_add(ff_mul(x, x), ff_mul(y, y)), ff_mul(z, z));
            w = ff_from_d_int(q[k]);
            if (kind == 0) {
                zeta = z;
                eta = r2;
                v = cpx_ff{x, y};
            } else {
                const ff ri = ff_rcp(r2);
                zeta = ff_mul(z, ri);
                eta = ri;
                v = cpx_ff{ff_mul(x, ri), ff_mul(y, ri)};
                w = ff_mul(w, ff_sqrt(ri));  // U_0^0 = 1/|x'|
            }
        }
        for (int i = 0; i < LP; ++i) {
            const ff zi = ff_shfl(zeta, i, LP), ei = ff_shfl(eta, i, LP), wi = ff_shfl(w, i, LP);
            const cpx_ff vi = cpx_ff_shfl(v, i, LP);
            // v^l by a prefix product over the lanes; v^m2 = v^(P-LP) v^(LP-1-l)
            cpx_ff pw = l == 0 ? cpx_ff{ff{1.f, 0.f}, ff{0.f, 0.f}} : vi;
#pragma unroll
            for (int d = 1; d < LP; d <<= 1) {
                const cpx_ff o = cpx_ff_shfl(pw, l >= d ? l - d : l, LP);
                if (l >= d) pw = cpx_ff_mul(pw, o);
            }
            cpx_ff ue = cpx_ff_shfl(pw, e < LP ? e : LP - 1, LP);
            if (e == LP) ue = cpx_ff_mul(ue, vi);
            const cpx_ff pm2 = cpx_ff_mul(ue, cpx_ff_shfl(pw, LP - 1 - l, LP));
            const ff k1 = ff_mul(d1, wi), k2 = ff_mul(d2, wi);
            p2x_columns_ff<T0, NT>(ab, m1, len1, m2, tot, cpx_ff{ff_mul(pw.r, k1), ff_mul(pw.i, k1)},
                               cpx_ff{ff_mul(pm2.r, k2), ff_mul(pm2.i, k2)}, zi, ei, ar, ai);
        }
    }
    if (tot <= T0) return;
    // back to R_n^m(x) = rho^n T / sig (P2M) or S_n^m(x) = sig U / rho^(n+1) (P2L)
    Out *o = out + j * stride;
#pragma unroll
    for (int u = 0; u < NT; ++u) {
        const int t = T0 + u;
        if (t < tot) {
            if (t < len1) p2x_put(o, kind, sh, m1 + t, m1, ar[u], ai[u]);
            else p2x_put(o, kind, sh, m2 + t - len1, m2, ar[u], ai[u]);
        }
    }
}

cudaError_t launch_p2x(bool f64, int kind, int P, long long nexp, long long nq, const uint32_t *offset,
                       const double *q, const double *pos, const double *centre, void *out, long long stride,
                       cudaStream_t st)
{
    if (nexp == 0) return cudaSuccess;
    if (P <= kP2xColsMax) {  // lanes per expansion: LP <= P <= 2 LP
        const int LP = P <= 2 ? (P == 1 ? 1 : 2) : P <= 4 ? 2 : P <= 8 ? 4 : P <= 16 ? 8 : 16;
        const int tb = 128;
        const long long grid = (nexp * LP + tb - 1) / tb;
        clear_stale_error();
#define SFMM_P2X_FF(T, L, T0, NT)                                                                        \
    k_p2x_ff<T, L, T0, NT><<<(unsigned)grid, tb, 0, st>>>(kind, P, nexp, nq, offset, q, pos, centre, (T *)out, \
                                                          stride)
#define SFMM_P2X_LP(T)                       \
    switch (LP) {                            \
    case 1: SFMM_P2X_FF(T, 1, 0, 3); break;  \
    case 2: SFMM_P2X_FF(T, 2, 0, 5); break;  \
    case 4: SFMM_P2X_FF(T, 4, 0, 9); break;  \
    case 8: SFMM_P2X_FF(T, 8, 0, 17); break; \
    default:                                 \
        if (P <= 24) {                       \
            SFMM_P2X_FF(T, 16, 0, 25);       \
        } else {                             \
            SFMM_P2X_FF(T, 16, 0, 17);       \
            SFMM_P2X_FF(T, 16, 17, 16);      \
        }                                    \
    }
        if (f64) SFMM_P2X_LP(double) else SFMM_P2X_LP(float)
#undef SFMM_P2X_LP
#undef SFMM_P2X_FF
        return cudaGetLastError();
    }
    int tb = 128;
    long long grid = (nexp + tb - 1) / tb;
    clear_stale_error();
    if (f64)
        k_p2x<double><<<(unsigned)grid, tb, 0, st>>>(kind, P, nexp, nq, offset, q, pos, centre, (double *)out,
                                                      stride);
    else
        k_p2x<float><<<(unsigned)grid, tb, 0, st>>>(kind, P, nexp, nq, offset, q, pos, centre, (float *)out,
                                                     stride);
    return cudaGetLastError();
}

// ---- evaluation (L2P / M2P) ----
//
// phi(x) = dot(E, R(x - c)) for a local expansion (kind 0) or
// dot(E, S(x - c)) for a multipole expansion (kind 1), the reference's
// solid dot product (solid.cpp:41-66): sum over n, m >= 0 of re*re + im*im,
// weighted 2 for m > 0.  The harmonics are produced column by column as in
// P2M/P2L and consumed at once, so a thread keeps no expansion-sized state.
// The gradient of a local expansion uses (d/dx - i d/dy) R_n^m = R_{n-1}^{m-1},
// (d/dx + i d/dy) R_n^m = -R_{n-1}^{m+1} and d/dz R_n^m = R_{n-1}^m: each
// R_k^v produced pairs with the degree-(k+1) coefficients v-1, v, v+1.
template <class In>
__global__ void k_eval(int kind, int P, long long npts, const double *__restrict__ pos,
                       const uint32_t *__restrict__ box, const In *__restrict__ E, long long stride,
                       const double *__restrict__ centre, double *pot, double *grad)
{
    const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= npts) return;
    const long long b = box ? (long long)box[j] : j;
    const In *e = E + b * stride;
    const double x = pos[3 * j] - centre[3 * b], y = pos[3 * j + 1] - centre[3 * b + 1],
                 z = pos[3 * j + 2] - centre[3 * b + 2];
    const double r2 = x * x + y * y + z * z;
    auto re = [&](int n, int m) { return (double)e[n * (n + 1) + m]; };
    auto im = [&](int n, int m) { return (double)e[(n + 1) * (n + 1) + m]; };
    double phi = 0, gx = 0, gy = 0, gz = 0;
    const bool want_grad = grad != nullptr && kind == 0;
    if (kind == 0) {
        double dr = 1.0, di = 0.0;  // R(m,m)
        for (int m = 0; m < P; ++m) {
            if (m > 0) {
                const double f = 1.0 / (2.0 * m);
                const double nr = (dr * x - di * y) * f, ni = (dr * y + di * x) * f;
                dr = nr;
                di = ni;
            }
            const double w = m ? 2.0 : 1.0;
            double ar = dr, ai = di, br = 0.0, bi = 0.0;
            for (int n = m; n < P; ++n) {
                double cr = ar, ci = ai;  // R(n,m)
                if (n == m + 1) {
                    cr = z * ar;
                    ci = z * ai;
                } else if (n > m + 1) {
                    const double f = 1.0 / ((double)(n + m) * (double)(n - m));
                    cr = (ar * z * (2 * n - 1) - r2 * br) * f;
                    ci = (ai * z * (2 * n - 1) - r2 * bi) * f;
                }
                phi += w * (re(n, m) * cr + im(n, m) * ci);
                if (want_grad && n + 1 < P) {
                    const int k1 = n + 1;
                    gz += w * (re(k1, m) * cr + im(k1, m) * ci);
                    if (m == 0) {
                        gx += cr * re(k1, 1);
                        gy += cr * im(k1, 1);
                    } else {
                        // conj(R) (L^{m+1} - L^{m-1}) and conj(R) (L^{m-1} + L^{m+1})
                        const double xr = re(k1, m + 1) - re(k1, m - 1), xi = im(k1, m + 1) - im(k1, m - 1);
                        const double yr = re(k1, m - 1) + re(k1, m + 1), yi = im(k1, m - 1) + im(k1, m + 1);
                        gx += cr * xr + ci * xi;
                        gy += cr * yi - ci * yr;
                    }
                }
                if (n > m) {
                    br = ar;
                    bi = ai;
                    ar = cr;
                    ai = ci;
                }
            }
        }
    } else {
        const double r2inv = 1.0 / r2;
        double dr = sqrt(r2inv), di = 0.0;  // S(m,m)
        for (int m = 0; m < P; ++m) {
            if (m > 0) {
                const double f = (2.0 * m - 1.0) * r2inv;
                const double nr = (dr * x - di * y) * f, ni = (dr * y + di * x) * f;
                dr = nr;
                di = ni;
            }
            const double w = m ? 2.0 : 1.0;
            double ar = dr, ai = di, br = 0.0, bi = 0.0;
            for (int n = m; n < P; ++n) {
                double cr = ar, ci = ai;
                if (n == m + 1) {
                    const double f = (2.0 * m + 1.0) * z * r2inv;
                    cr = f * ar;
                    ci = f * ai;
                } else if (n > m + 1) {
                    const double c2 = (double)(n + m - 1) * (double)(n - m - 1);
                    cr = (ar * z * (2 * n - 1) - c2 * br) * r2inv;
                    ci = (ai * z * (2 * n - 1) - c2 * bi) * r2inv;
                }
                phi += w * (re(n, m) * cr + im(n, m) * ci);
                if (n > m) {
                    br = ar;
                    bi = ai;
                    ar = cr;
                    ai = ci;
                }
            }
        }
    }
    pot[j] += phi;
    if (want_grad) {
        grad[3 * j] += gx;
        grad[3 * j + 1] += gy;
        grad[3 * j + 2] += gz;
    }
}

// ---- float-float L2P / M2P for orders up to 32 ----
//
// The same sums as k_eval on the FP32 pipe, on the Schmidt-normalised
// harmonics of P2M/P2L (k_p2x_ff).  A pre-pass (k_eval_prep, one thread per
// expansion and degree n) writes each coefficient in the matching normalised
// form, e(n,m) = E(n,m) / sig(n,m) for a local expansion or E(n,m) sig(n,m)
// for a multipole, as float-float mantissas at one block exponent per degree
// (e = M 2^s_n, |M| < 4), so that evaluating a point costs an exponent shift
// per coefficient instead of a conversion.  Per point (k_eval_ff):
// x' = (x - c) / rho, rho = 2^sh rounded up from |x - c| for L2P (|x'| <= 1)
// and down for M2P (|x'| >= 1), then
//   E . R(x - c) = sum_{n,m} w_m (e 2^(n sh)) . T_n^m(x')           (L2P)
//   E . S(x - c) = sum_{n,m} w_m (e 2^-((n+1) sh)) . U_n^m(x')      (M2P)
// with w_0 = 1, w_m = 2 (the solid dot product, solid.cpp:41-66).  The
// gradient of a local expansion pairs T_k^v with the degree-(k+1)
// coefficients v, v+1, v-1 as k_eval does with R_k^v, each pairing weighted
// by sig(k+1, v')/sig(k, v), the sum divided by rho.

// x 2^sh as float-float; zero and subnormal x give 0 whatever the shift (the
// block exponent of a degree of tiny coefficients can make sh large enough
// for ff_from_d_scaled's range test to miss them)
__device__ __forceinline__ ff ff_of_scaled(double x, int sh) { return ff_from_d_scaled0(x, sh); }
__device__ __forceinline__ ff ff_of_scaled(float x, int sh) { return ff{ldexp2(x, max(-252, min(252, sh))), 0.f}; }

template <class In>
__global__ void k_eval_prep(int kind, int P, long long nexp, const In *__restrict__ E, long long stride,
                            float4 *__restrict__ Mout, int *__restrict__ sdeg)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= nexp * P) return;
    const long long b = i / P;
    const int n = (int)(i - b * P);
    const In *e = E + b * stride;
    const int t0 = n * (n + 1) / 2;
    int s = -(1 << 20);
    for (int m = 0; m <= n; ++m) {
        const int se = kind ? kP2xTab.se[t0 + m] : -kP2xTab.se[t0 + m];
        s = max(s, max(exp_of(e[n * (n + 1) + m]), exp_of(e[(n + 1) * (n + 1) + m])) + se);
    }
    sdeg[i] = s;  // an all-zero degree keeps -2^20: it never sets a point's scale
    float4 *o = Mout + b * (P * (P + 1) / 2) + t0;
    for (int m = 0; m <= n; ++m) {
        const int se = kind ? kP2xTab.se[t0 + m] : -kP2xTab.se[t0 + m];
        const float2 f2 = kind ? kP2xTab.fs[t0 + m] : kP2xTab.fi[t0 + m];
        const ff f{f2.x, f2.y};
        const ff re = ff_mul(ff_of_scaled(e[n * (n + 1) + m], se - s), f);
        const ff im = ff_mul(ff_of_scaled(e[(n + 1) * (n + 1) + m], se - s), f);
        o[m] = make_float4(re.hi, re.lo, im.hi, im.lo);
    }
}

// coefficient (n, m) of expansion row Mb times 2^ex (|M| < 4: beyond +-252
// the product under- or overflows FP32 in any case)
__device__ __forceinline__ cpx_ff eval_coef(const float4 *Mb, int n, int m, int ex)
{
    ex = max(-252, min(252, ex));
    const float4 v = __ldg(Mb + n * (n + 1) / 2 + m);
    return cpx_ff{ff{ldexp2(v.x, ex), ldexp2(v.y, ex)}, ff{ldexp2(v.z, ex), ldexp2(v.w, ex)}};
}
__device__ __forceinline__ ff ff_tab(const float2 *t, int i)
{
    const float2 v = t[i];
    return ff{v.x, v.y};
}
__device__ __forceinline__ void ffacc_madd(ffacc &a, ff w, ff x) { ffacc_add(a, ff_mul(w, x)); }

__global__ void __launch_bounds__(128) k_eval_ff(int kind, int P, long long npts, const double *__restrict__ pos,
                                                 const uint32_t *__restrict__ box, const float4 *__restrict__ M,
                                                 const int *__restrict__ sdeg, const double *__restrict__ centre,
                                                 double *pot, double *grad)
{
    const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= npts) return;
    const long long b = box ? (long long)box[j] : j;
    const double dx = pos[3 * j] - centre[3 * b], dy = pos[3 * j + 1] - centre[3 * b + 1],
                 dz = pos[3 * j + 2] - centre[3 * b + 2];
    // rho = 2^sh from the largest component's exponent e: 2^(e+2) > |x - c|
    // (L2P), 2^e <= |x - c| (M2P); any double scale
    const int e3 = max_exp3(dx, dy, dz);
    const int sh = e3 == -(1 << 20) ? 0 : (kind == 0 ? e3 + 2 : e3);
    const ff x = ff_from_d_scaled(dx, -sh), y = ff_from_d_scaled(dy, -sh), z = ff_from_d_scaled(dz, -sh);
    const ff r2 = ff_add(ff_add(ff_mul(x, x), ff_mul(y, y)), ff_mul(z, z));
    ff zeta, eta, w0{1.f, 0.f};
    cpx_ff v;
    if (kind == 0) {
        zeta = z;
        eta = r2;
        v = cpx_ff{x, y};
    } else {
        const ff ri = ff_rcp(r2);
        zeta = ff_mul(z, ri);
        eta = ri;
        v = cpx_ff{ff_mul(x, ri), ff_mul(y, ri)};
        w0 = ff_sqrt(ri);  // U_0^0 = 1/|x'|
    }
    const float4 *Mb = M + b * (P * (P + 1) / 2);
    const int *sb = sdeg + b * P;
    const bool want_grad = grad != nullptr && kind == 0;
    // the sums run at the scale 2^-B of the largest degree and return to
    // their own in FP64, so results beyond the FP32 range keep their digits
    int B = -(1 << 29);
    for (int n = 0; n < P; ++n) B = max(B, kind == 0 ? sb[n] + n * sh : sb[n] - (n + 1) * sh);
    if (B < -(1 << 19)) B = 0;  // all coefficients zero
    // v^(2^i), i < 5: every v^m (m < 32) is a product of at most five of
    // them, so its rounding error grows with log m rather than with m
    cpx_ff v2i[5];
    v2i[0] = v;
#pragma unroll
    for (int i = 1; i < 5; ++i) v2i[i] = cpx_ff_mul(v2i[i - 1], v2i[i - 1]);
    // each column sums into fresh accumulators (at most P terms), added to
    // the totals with a renormalising float-float addition
    ff phi{0.f, 0.f}, gx{0.f, 0.f}, gy{0.f, 0.f}, gz{0.f, 0.f};
    for (int m = 0; m < P; ++m) {
        cpx_ff vm{w0, ff{0.f, 0.f}};  // v^m / |x'| (M2P) or v^m (L2P)
#pragma unroll
        for (int i = 0; i < 5; ++i)
            if (m >> i & 1) vm = cpx_ff_mul(vm, v2i[i]);
        const ff dm = ff_tab(kP2xTab.diag, m);
        cpx_ff x1{ff_mul(dm, vm.r), ff_mul(dm, vm.i)}, x2{ff{0.f, 0.f}, ff{0.f, 0.f}};
        ffacc cphi{0.f, 0.f}, cgx{0.f, 0.f}, cgy{0.f, 0.f}, cgz{0.f, 0.f};
        const float wm = m ? 2.f : 1.f;
        for (int n = m; n < P; ++n) {
            if (n > m) {
                const float4 c = kP2xTab.ab[n - m][m];
                const ff A = ff_mul(ff{c.x, c.y}, zeta), B = ff_mul(ff{c.z, c.w}, eta);
                const cpx_ff xn{ff_fms2(A, x1.r, B, x2.r), ff_fms2(A, x1.i, B, x2.i)};
                x2 = x1;
                x1 = xn;
            }
            const int ex = (kind == 0 ? sb[n] + n * sh : sb[n] - (n + 1) * sh) - B;
            const cpx_ff e = eval_coef(Mb, n, m, ex);
            const ff t = ff_fms2(e.r, x1.r, ff{-e.i.hi, -e.i.lo}, x1.i);  // e_re X_re + e_im X_im
            ffacc_add(cphi, ff{t.hi * wm, t.lo * wm});
            if (want_grad && n + 1 < P) {
                const int k1 = n + 1, ix = n * (n + 1) / 2 + m, ex1 = sb[k1] + k1 * sh - B;
                const cpx_ff ez = eval_coef(Mb, k1, m, ex1);
                const ff tz = ff_fms2(ez.r, x1.r, ff{-ez.i.hi, -ez.i.lo}, x1.i);
                ffacc_madd(cgz, ff_tab(kP2xTab.cz, ix), ff{tz.hi * wm, tz.lo * wm});
                const cpx_ff ep = eval_coef(Mb, k1, m + 1, ex1);
                const ff cp = ff_tab(kP2xTab.cp, ix);
                if (m == 0) {  // R_k^0 is real
                    ffacc_madd(cgx, cp, ff_mul(x1.r, ep.r));
                    ffacc_madd(cgy, cp, ff_mul(x1.r, ep.i));
                } else {
                    const cpx_ff em = eval_coef(Mb, k1, m - 1, ex1);
                    const ff cm = ff_tab(kP2xTab.cm, ix);
                    // conj(R) (L^{m+1} - L^{m-1}) and conj(R) (L^{m-1} + L^{m+1}), each L weighted
                    const ff xr = ff_fms2(cp, ep.r, cm, em.r), xi = ff_fms2(cp, ep.i, cm, em.i);
                    const ff yr = ff_fms2(cm, em.r, ff{-cp.hi, -cp.lo}, ep.r);
                    const ff yi = ff_fms2(cm, em.i, ff{-cp.hi, -cp.lo}, ep.i);
                    ffacc_add(cgx, ff_fms2(x1.r, xr, ff{-x1.i.hi, -x1.i.lo}, xi));
                    ffacc_add(cgy, ff_fms2(x1.r, yi, x1.i, yr));
                }
            }
        }
        phi = ff_add(phi, ff{cphi.hi, cphi.lo});
        if (want_grad) {
            gx = ff_add(gx, ff{cgx.hi, cgx.lo});
            gy = ff_add(gy, ff{cgy.hi, cgy.lo});
            gz = ff_add(gz, ff{cgz.hi, cgz.lo});
        }
    }
    pot[j] += ldexp((double)phi.hi + (double)phi.lo, B);
    if (want_grad) {
        const double ir = ldexp(1.0, B - sh);
        grad[3 * j] += ((double)gx.hi + (double)gx.lo) * ir;
        grad[3 * j + 1] += ((double)gy.hi + (double)gy.lo) * ir;
        grad[3 * j + 2] += ((double)gz.hi + (double)gz.lo) * ir;
    }
}

size_t eval_scratch_bytes(int P, long long nexp)
{
    if (P > kP2xColsMax) return 0;
    return (size_t)nexp * ((size_t)P * (P + 1) / 2 * sizeof(float4) + (size_t)P * sizeof(int));
}

cudaError_t launch_eval(bool f64, int kind, int P, long long npts, const double *pos, const uint32_t *box,
                        const void *E, long long stride, long long nexp, const double *centre, double *pot,
                        double *grad, void *scratch, cudaStream_t st)
{
    if (npts == 0) return cudaSuccess;
    const int tb = 128;
    const long long grid = (npts + tb - 1) / tb;
    clear_stale_error();
    if (scratch && P <= kP2xColsMax) {  // float-float: normalise every expansion once, then the points
        float4 *Mn = static_cast<float4 *>(scratch);
        int *sdeg = reinterpret_cast<int *>(Mn + (size_t)nexp * (P * (P + 1) / 2));
        const long long gp = (nexp * P + tb - 1) / tb;
        if (f64)
            k_eval_prep<double><<<(unsigned)gp, tb, 0, st>>>(kind, P, nexp, (const double *)E, stride, Mn, sdeg);
        else
            k_eval_prep<float><<<(unsigned)gp, tb, 0, st>>>(kind, P, nexp, (const float *)E, stride, Mn, sdeg);
        k_eval_ff<<<(unsigned)grid, tb, 0, st>>>(kind, P, npts, pos, box, Mn, sdeg, centre, pot, grad);
        return cudaGetLastError();
    }
    if (f64)
        k_eval<double><<<(unsigned)grid, tb, 0, st>>>(kind, P, npts, pos, box, (const double *)E, stride, centre,
                                                       pot, grad);
    else
        k_eval<float><<<(unsigned)grid, tb, 0, st>>>(kind, P, npts, pos, box, (const float *)E, stride, centre,
                                                      pot, grad);
    return cudaGetLastError();
}

// ---- accumulation of per-target results into targets given by address ----
//
// One warp per target: target[c] += slots[j * stride + c] for c < cnt[j].
// The targets are distinct, so plain read-modify-writes suffice; they may be
// host solids that the GPU reads and writes through the host page tables.
template <class T>
__global__ void k_add_slots(long long nt, const unsigned long long *__restrict__ tptr,
                            const uint32_t *__restrict__ cnt, const T *__restrict__ slots, long long stride)
{
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= nt) return;
    T *o = reinterpret_cast<T *>(tptr[w]);
    const T *r = slots + w * stride;
    for (uint32_t c = lane; c < cnt[w]; c += 32) o[c] += r[c];
}

cudaError_t launch_add_slots(bool f64, long long nt, const unsigned long long *tptr, const uint32_t *cnt,
                             const void *slots, long long stride, cudaStream_t st)
{
    if (nt == 0) return cudaSuccess;
    const int tb = 256;
    const long long grid = (nt * 32 + tb - 1) / tb;
    clear_stale_error();
    if (f64)
        k_add_slots<double><<<(unsigned)grid, tb, 0, st>>>(nt, tptr, cnt, (const double *)slots, stride);
    else
        k_add_slots<float><<<(unsigned)grid, tb, 0, st>>>(nt, tptr, cnt, (const float *)slots, stride);
    return cudaGetLastError();
}

// ---- bucketing by (p_in, p_out) ----

__global__ void k_bucket_count(long long n, const uint32_t *pin, const uint32_t *pout, uint32_t *cnt, int K)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        uint32_t key = min(pin[i], (uint32_t)(K - 1)) * (uint32_t)K + min(pout[i], (uint32_t)(K - 1));
        atomicAdd(&cnt[key], 1u);
    }
}

// single CTA exclusive scan over nkeys counters, any number: thread t
// handles a chunk of ceil(nkeys / 1024) consecutive keys.  Callers: the
// context bucketing (K = P + 1 <= 87) and the allocation-free entry point
// (K = max_order + 1 <= 87, 7 569 keys)
__global__ void k_bucket_scan(uint32_t *cnt, int nkeys)
{
    __shared__ uint32_t part[1024];
    const int t = threadIdx.x;
    const int per = (nkeys + blockDim.x - 1) / blockDim.x;
    uint32_t s = 0;
    for (int k = t * per; k < min(nkeys, (t + 1) * per); ++k) s += cnt[k];
    part[t] = s;
    __syncthreads();
    if (t == 0) {
        uint32_t run = 0;
        for (int k = 0; k < (int)blockDim.x; ++k) {
            uint32_t v = part[k];
            part[k] = run;
            run += v;
        }
    }
    __syncthreads();
    uint32_t run = part[t];
    for (int k = t * per; k < min(nkeys, (t + 1) * per); ++k) {
        uint32_t v = cnt[k];
        cnt[k] = run;
        run += v;
    }
}

__global__ void k_bucket_scatter(long long n, const uint32_t *pin, const uint32_t *pout, uint32_t *off, int K,
                                 uint32_t *order)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        uint32_t key = min(pin[i], (uint32_t)(K - 1)) * (uint32_t)K + min(pout[i], (uint32_t)(K - 1));
        uint32_t pos = atomicAdd(&off[key], 1u);
        order[pos] = (uint32_t)i;
    }
}

size_t bucket_work_words(int P) { return (size_t)(P + 1) * (P + 1); }

cudaError_t launch_bucket(long long n, const uint32_t *pin, const uint32_t *pout, uint32_t *order, uint32_t *work,
                          int P, cudaStream_t st)
{
    const int K = P + 1;
    const int nkeys = K * K;
    clear_stale_error();
    cudaError_t e = cudaMemsetAsync(work, 0, sizeof(uint32_t) * nkeys, st);
    if (e != cudaSuccess) return e;
    if (n == 0) return cudaSuccess;
    int grid = (int)std::min<long long>((n + 255) / 256, 4096);
    k_bucket_count<<<grid, 256, 0, st>>>(n, pin, pout, work, K);
    k_bucket_scan<<<1, 1024, 0, st>>>(work, nkeys);
    k_bucket_scatter<<<grid, 256, 0, st>>>(n, pin, pout, work, K, order);
    return cudaGetLastError();
}

}  // namespace sfmm

// ---- bucketing without allocation ----
//
// The counters of the bucketing sort live in a fixed device array instead of
// context memory, for callers that must not allocate device memory at all:
// codes that hand the whole device to their own memory pool, run under a
// hard per-process memory cap, or issue work from paths where a cudaMalloc
// would stall or fail.  The array is sized for orders up to 86 (the largest
// order a solidfmm operator accepts), 87 x 87 counters = 30 KiB; every GPU
// that loads the library keeps it until the process exits.

namespace {

constexpr int kStaticBucketMaxOrder = 86;
constexpr int kStaticBucketKeys = (kStaticBucketMaxOrder + 1) * (kStaticBucketMaxOrder + 1);

__device__ __align__(256) uint32_t g_bucket_counters[kStaticBucketKeys];

// Device address of g_bucket_counters.  A __device__ array belongs to one CUDA
// context (one per device with the runtime's primary contexts, but a caller
// of the driver API may make another current, and cudaDeviceReset replaces
// the primary one), so the address is looked up again on every call made
// outside a stream capture and cached per current context for calls made
// during a capture, when no lookup may load the module.
std::mutex g_bucket_mtx;
std::map<void *, uint32_t *> g_bucket_addr;

using CtxGetCurrent = int (*)(void **);

// the current CUcontext through the driver entry point (the library does not
// link libcuda, so that it loads on machines without a GPU driver)
void *current_context()
{
    static CtxGetCurrent fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<CtxGetCurrent>(f);
    }();
    void *ctx = nullptr;
    if (!fn || fn(&ctx) != 0) return nullptr;
    return ctx;
}

}  // namespace

extern "C" int sfmm_bucket_by_order_noalloc(size_t n, const uint32_t *p_in, const uint32_t *p_out, uint32_t *order,
                                            size_t max_order, void *stream)
{
    if (max_order > (size_t)kStaticBucketMaxOrder) return SFMM_ORDER_RANGE;
    if (n > 0xffffffffull) return SFMM_INVALID_ARG;
    if (n == 0) return SFMM_OK;
    if (!p_in || !p_out || !order) return SFMM_INVALID_ARG;
    void *ctx = current_context();
    if (!ctx) {  // no context current yet: initialise the current device's primary context
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaSetDevice(dev) != cudaSuccess) return SFMM_CUDA_ERROR;
        ctx = current_context();
    }
    if (!ctx) return SFMM_CUDA_ERROR;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing((cudaStream_t)stream, &cap) != cudaSuccess) return SFMM_CUDA_ERROR;
    uint32_t *counters = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_bucket_mtx);
        if (cap == cudaStreamCaptureStatusNone) {
            // the host-side symbol is only a stand-in for the array; the
            // kernels need its address in the current context
            if (cudaGetSymbolAddress((void **)&counters, g_bucket_counters) != cudaSuccess) return SFMM_CUDA_ERROR;
            g_bucket_addr[ctx] = counters;
        } else {
            auto it = g_bucket_addr.find(ctx);
            if (it == g_bucket_addr.end()) return SFMM_INVALID_ARG;  // first call inside a capture
            counters = it->second;
        }
    }
    // the counters are cleared on the stream before use (launch_bucket)
    cudaError_t e = sfmm::launch_bucket((long long)n, p_in, p_out, order, counters, (int)max_order,
                                        (cudaStream_t)stream);
    return e == cudaSuccess ? SFMM_OK : SFMM_CUDA_ERROR;
}

