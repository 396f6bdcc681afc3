// Fused translation kernel: M2M, M2L and L2L over a batch of translations.
//
// One CTA processes tiles of TS translations; each translation is handled by
// a group of G threads that share its working expansion in a per-CTA
// shared-memory buffer.  Per tile:
//
//   1. cooperative, coalesced gather of the TS source expansions into the
//      buffer (solid2buf, microkernel_generic.cpp:341-359),
//   2. per degree n: forward edge (scale r^{-(n+1)} or r^n, rotate e^{i m alpha},
//      change to the orthogonal swap basis), swap, rotate e^{i m beta}, swap
//      (forward_transform_M/L, translations.cpp:37-85 and 190-240),
//   3. z-translation per column m (zm2l / zm2m, translations.cpp:283-296,
//      366-377, 440-451) as a small dense matrix per m,
//   4. per degree n: swap, rotate e^{-i m beta}, swap, backward edge
//      (backward_transform_L/M, translations.cpp:88-187),
//   5. cooperative, coalesced accumulation into the targets (buf2solid,
//      microkernel_generic.cpp:362-380), with FP64/FP32 atomics when
//      targets may repeat.
//
// Thread q of a group owns rows i = q + G a of every degree-n swap,
// rotation elements m = q + G a, and outputs n' = m + q + G a of every
// z-translation column; each stage keeps its accumulators in registers and
// reads its inputs from the buffer (group members synchronise with
// __syncwarp).  The number of accumulator blocks a stage needs,
// ceil(d / G), is warp-uniform and selects a stage instance compiled for
// exactly that many blocks, so no block is issued only to be predicated off.
// Loop bounds are warp-uniform maxima over the warp's 32/G translations,
// like the reference's lanes padded with zero orders (translations.cpp:504-514);
// inputs past a translation's own order read as zero and outputs past it are
// dropped.
#pragma once

#include <cstdint>
#include <type_traits>

#include "sfmm_arith.cuh"
#include "sfmm_fixed.cuh"
#include "sfmm_params.hpp"

namespace sfmm {

template <class A>
struct src_of {
    using type = double;
};
template <>
struct src_of<float> {
    using type = float;
};


// complex helpers in FP64 for the per-translation geometry
struct cd {
    double c, s;
};
__device__ __forceinline__ cd cmul(cd a, cd b) { return cd{a.c * b.c - a.s * b.s, a.s * b.c + a.c * b.s}; }

__device__ __forceinline__ void prefetch_l2(const void *ptr)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(ptr));
}

template <int N>
struct ic {
    static constexpr int value = N;
};

// Calls f(ic<na>) for na in 1..MAXN (warp-uniform switch).
template <int MAXN, class F>
__device__ __forceinline__ void dispatch(int na, F &&f)
{
    switch (na) {
    case 1: f(ic<1>{}); break;
    case 2: if constexpr (MAXN >= 2) f(ic<2>{}); break;
    case 3: if constexpr (MAXN >= 3) f(ic<3>{}); break;
    case 4: if constexpr (MAXN >= 4) f(ic<4>{}); break;
    case 5: if constexpr (MAXN >= 5) f(ic<5>{}); break;
    case 6: if constexpr (MAXN >= 6) f(ic<6>{}); break;
    case 7: if constexpr (MAXN >= 7) f(ic<7>{}); break;
    case 8: if constexpr (MAXN >= 8) f(ic<8>{}); break;
    default: break;
    }
}

// Rows of a degree's swap-coefficient block in the instance that runs NA
// accumulator blocks of G threads: the tables pad rows to a multiple of 8
// for orders up to 32 (G = 4 or 8) and of 32 above (G = 32), so the row
// count of every degree served by one (G, NA) instance is the same
// compile-time constant.
// The two swap passes of a degree: unrolled for FP64 and FP32 (the second
// pass's loads overlap the first's tail: +1.8% FP64, +3% FP32 at P=20 on
// GB300), rolled for float-float (-5% unrolled)
template <class T>
constexpr int kPassUnroll = std::is_same<T, double>::value || std::is_same<T, float>::value ? 2 : 1;

template <int G, int NA>
__host__ __device__ constexpr int swap_rows()
{
    return G == 32 ? 32 * NA : ((G * NA + 7) & ~7);
}

// Both swap parts of one degree: rows i = q + G a (a < NA) of W_R applied to
// the real parts (columns j = jr, jr+2, ...) and of W_I to the imaginary
// parts (the complementary checkerboard, columns ji = jr^1, ji+2, ...).
// The coefficient block holds only that checkerboard: slot t of row i is
// column jr(i) + 2t (W_R) or ji(i) + 2t (W_I), and each slot stores the R
// rows of W_R followed by the R rows of W_I, so one pointer walks both with
// compile-time offsets.  Rows are zero-padded to R and slots to (d+3)/2, and
// the buffer slots past each expansion are zero, so every load is
// unconditional; operands of the next column pair are fetched before the
// current pair's multiply-adds (software pipelining), and the real and
// imaginary chains are independent (2*NA accumulations per iteration).
template <class AR, int G, int NA>
__device__ __forceinline__ void swap_both(const typename AR::T *__restrict__ W, const typename AR::Stor *xre,
                                          const typename AR::Stor *xim, int d, int n, int q,
                                          typename AR::Acc (&ar)[NA], typename AR::Acc (&ai)[NA])
{
    using T = typename AR::T;
    constexpr int R = swap_rows<G, NA>();
    // unrolling measured on GB300: FP64 runs best rolled (its pipe is the
    // limit; +3% at M2L P=16), FP32 unrolled four times (+7% at P=16 with the
    // passes unrolled too), float-float twice (-10% rolled)
    constexpr int kUnroll = std::is_same<T, double>::value ? 1 : (std::is_same<T, float>::value ? 4 : 2);
    const int jr0 = (q + n) & 1, ji0 = jr0 ^ 1;
    const int cnt = (d + 1) >> 1;  // iterations of the longer part
    const T *w = W + q;
    const typename AR::Stor *xr_p = xre + jr0;
    const typename AR::Stor *xi_p = xim + ji0;
    T xrn = AR::ld(xr_p), xin = AR::ld(xi_p);
    T wrn[NA], win[NA];
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        wrn[a] = AR::ldt(w + G * a);
        win[a] = AR::ldt(w + R + G * a);
    }
#pragma unroll kUnroll
    for (int t = 0; t < cnt; ++t) {
        const T xr = xrn, xi = xin;
        T wr[NA], wi[NA];
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            wr[a] = wrn[a];
            wi[a] = win[a];
        }
        xr_p += 2;
        xi_p += 2;
        w += 2 * R;
        xrn = AR::ld(xr_p);
        xin = AR::ld(xi_p);
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            wrn[a] = AR::ldt(w + G * a);
            win[a] = AR::ldt(w + R + G * a);
        }
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            AR::mac(ar[a], wr[a], xr);
            AR::mac(ai[a], wi[a], xi);
        }
    }
}

// Per-thread geometry of one translation: e^{i m alpha} and e^{i m beta} for
// the rotation elements m = q + G a this thread owns.
template <class AR, int ACC>
struct Trig {
    typename AR::T ca[ACC], sa[ACC], cb[ACC], sb[ACC];
};

// One degree of the forward transform, NA = ceil(d / G) blocks.
template <class AR, int G, int NA, int ACC>
__device__ __forceinline__ void forward_degree(typename AR::Stor *b, int n,
                                               const typename AR::T *__restrict__ WR,
                                               const typename AR::T *__restrict__ ein, typename AR::T f, int q,
                                               const Trig<AR, ACC> &tg)
{
    using T = typename AR::T;
    using Acc = typename AR::Acc;
    using S = typename AR::Stor;
    const int d = n + 1;
    S *bre = b + n * (n + 1);
    S *bim = b + (n + 1) * (n + 1);
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        const int m = q + G * a;
        if (m < d) {
            const T xr = AR::ld(bre + m);
            const T xi = AR::ld(bim + m);
            const T g = AR::mul(f, AR::ldt(ein + m));
            const T gc = AR::mul(g, tg.ca[a]), gs = AR::mul(g, tg.sa[a]);
            AR::st(bre + m, AR::dot2(gc, xr, AR::neg(gs), xi));
            AR::st(bim + m, AR::dot2(gs, xr, gc, xi));
        }
    }
    __syncwarp();
#pragma unroll kPassUnroll<typename AR::T>
    for (int pass = 0; pass < 2; ++pass) {
        Acc ar[NA], ai[NA];
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            ar[a] = AR::acc0();
            ai[a] = AR::acc0();
        }
        swap_both<AR, G, NA>(WR, bre, bim, d, n, q, ar, ai);
        __syncwarp();
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            const int ii = q + G * a;
            if (ii < d) {
                T vr = AR::fin(ar[a]);
                T vi = AR::fin(ai[a]);
                if (pass == 0) {  // rotation by e^{+i m beta} between the two swaps
                    const T wr = AR::dot2(tg.cb[a], vr, AR::neg(tg.sb[a]), vi);
                    const T wi = AR::dot2(tg.sb[a], vr, tg.cb[a], vi);
                    vr = wr;
                    vi = wi;
                }
                AR::st(bre + ii, vr);
                AR::st(bim + ii, vi);
            }
        }
        __syncwarp();
    }
}

// One degree of the backward transform, NA = ceil(d / G) blocks.
template <class AR, int G, int NA, int ACC>
__device__ __forceinline__ void backward_degree(typename AR::Stor *b, int n,
                                                const typename AR::T *__restrict__ WR,
                                                const typename AR::T *__restrict__ eout, typename AR::T f, int q,
                                                const Trig<AR, ACC> &tg)
{
    using T = typename AR::T;
    using Acc = typename AR::Acc;
    using S = typename AR::Stor;
    const int d = n + 1;
    S *bre = b + n * (n + 1);
    S *bim = b + (n + 1) * (n + 1);
#pragma unroll kPassUnroll<typename AR::T>
    for (int pass = 0; pass < 2; ++pass) {
        Acc ar[NA], ai[NA];
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            ar[a] = AR::acc0();
            ai[a] = AR::acc0();
        }
        swap_both<AR, G, NA>(WR, bre, bim, d, n, q, ar, ai);
        __syncwarp();
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            const int ii = q + G * a;
            if (ii < d) {
                T vr = AR::fin(ar[a]);
                T vi = AR::fin(ai[a]);
                if (pass == 0) {  // e^{-i m beta}
                    const T wr = AR::dot2(tg.cb[a], vr, tg.sb[a], vi);
                    const T wi = AR::dot2(tg.cb[a], vi, AR::neg(tg.sb[a]), vr);
                    vr = wr;
                    vi = wi;
                } else {  // e^{-i m alpha}, back to the solid basis, r-power scale
                    const T g = AR::mul(f, AR::ldt(eout + ii));
                    const T gc = AR::mul(g, tg.ca[a]), gs = AR::mul(g, tg.sa[a]);
                    const T wr = AR::dot2(gc, vr, gs, vi);
                    const T wi = AR::dot2(gc, vi, AR::neg(gs), vr);
                    vr = wr;
                    vi = wi;
                }
                AR::st(bre + ii, vr);
                AR::st(bim + ii, vi);
            }
        }
        __syncwarp();
    }
}

// Q1.30 cos / sin of m beta for the rotation elements a thread owns
template <int ACC>
struct FixTrig {
    int c[ACC], s[ACC];
};

__device__ __forceinline__ void st_fixed(float2 *p, int v) { *reinterpret_cast<int *>(p) = v; }

// One degree of the forward transform with the swaps and the beta rotation
// in block fixed point: float-float edge, conversion at the row's block
// exponent, integer swap, renormalise, integer rotation, integer swap,
// renormalise, back to float-float.
template <int G, int NA, int ACC>
__device__ __forceinline__ void forward_degree_fixed(float2 *b, int n, const int *__restrict__ WRq,
                                                     const ff *__restrict__ ein, ff f, int q,
                                                     const Trig<arith<ff>, ACC> &tg, const FixTrig<ACC> &tq)
{
    using AR = arith<ff>;
    const int d = n + 1;
    float2 *bre = b + n * (n + 1);
    float2 *bim = b + (n + 1) * (n + 1);
    ff vr[NA], vi[NA];
    float mx = 0.f;
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        const int m = q + G * a;
        vr[a] = vi[a] = AR::zero();
        if (m < d) {
            const ff xr = AR::ld(bre + m);
            const ff xi = AR::ld(bim + m);
            const ff g = AR::mul(f, AR::ldt(ein + m));
            const ff gc = AR::mul(g, tg.ca[a]), gs = AR::mul(g, tg.sa[a]);
            vr[a] = AR::dot2(gc, xr, AR::neg(gs), xi);
            vi[a] = AR::dot2(gs, xr, gc, xi);
            mx = fmaxf(mx, fmaxf(fabsf(vr[a].hi), fabsf(vi[a].hi)));
        }
    }
    int E = block_exponent(group_max<G>(mx));
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        const int m = q + G * a;
        if (m < d) {
            st_fixed(bre + m, ff_to_fixed(vr[a], E));
            st_fixed(bim + m, ff_to_fixed(vi[a], E));
        }
    }
    __syncwarp();
#pragma unroll 1
    for (int pass = 0; pass < 2; ++pass) {
        long long ar[NA], ai[NA];
#pragma unroll
        for (int a = 0; a < NA; ++a) ar[a] = ai[a] = 0;
        swap_both_fixed<G, NA, swap_rows<G, NA>()>(WRq, bre, bim, d, n, q, ar, ai);
        const int sh = group_renorm_shift<G, NA>(ar, ai);
        E += sh - 30;
        __syncwarp();
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            const int ii = q + G * a;
            if (ii < d) {
                const int xr = round_shift(ar[a], sh), xi = round_shift(ai[a], sh);
                if (pass == 0) {  // rotation by e^{+i m beta} between the two swaps
                    st_fixed(bre + ii, rot_q30(tq.c[a], xr, tq.s[a], xi));
                    st_fixed(bim + ii, rot_q30(tq.c[a], xi, -tq.s[a], xr));
                } else {
                    AR::st(bre + ii, fixed_to_ff(xr, E));
                    AR::st(bim + ii, fixed_to_ff(xi, E));
                }
            }
        }
        __syncwarp();
    }
}

// One degree of the backward transform with fixed-point swaps and beta
// rotation; the alpha rotation and r-power scale stay in float-float.
template <int G, int NA, int ACC>
__device__ __forceinline__ void backward_degree_fixed(float2 *b, int n, const int *__restrict__ WRq,
                                                      const ff *__restrict__ eout, ff f, int q,
                                                      const Trig<arith<ff>, ACC> &tg, const FixTrig<ACC> &tq)
{
    using AR = arith<ff>;
    const int d = n + 1;
    float2 *bre = b + n * (n + 1);
    float2 *bim = b + (n + 1) * (n + 1);
    ff vr[NA], vi[NA];
    float mx = 0.f;
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        const int m = q + G * a;
        vr[a] = vi[a] = AR::zero();
        if (m < d) {
            vr[a] = AR::ld(bre + m);
            vi[a] = AR::ld(bim + m);
            mx = fmaxf(mx, fmaxf(fabsf(vr[a].hi), fabsf(vi[a].hi)));
        }
    }
    int E = block_exponent(group_max<G>(mx));
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        const int m = q + G * a;
        if (m < d) {
            st_fixed(bre + m, ff_to_fixed(vr[a], E));
            st_fixed(bim + m, ff_to_fixed(vi[a], E));
        }
    }
    __syncwarp();
#pragma unroll 1
    for (int pass = 0; pass < 2; ++pass) {
        long long ar[NA], ai[NA];
#pragma unroll
        for (int a = 0; a < NA; ++a) ar[a] = ai[a] = 0;
        swap_both_fixed<G, NA, swap_rows<G, NA>()>(WRq, bre, bim, d, n, q, ar, ai);
        const int sh = group_renorm_shift<G, NA>(ar, ai);
        E += sh - 30;
        __syncwarp();
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            const int ii = q + G * a;
            if (ii < d) {
                const int xr = round_shift(ar[a], sh), xi = round_shift(ai[a], sh);
                if (pass == 0) {  // e^{-i m beta}
                    st_fixed(bre + ii, rot_q30(tq.c[a], xr, -tq.s[a], xi));
                    st_fixed(bim + ii, rot_q30(tq.c[a], xi, tq.s[a], xr));
                } else {  // e^{-i m alpha}, back to the solid basis, r-power scale
                    const ff ur = fixed_to_ff(xr, E), ui = fixed_to_ff(xi, E);
                    const ff g = AR::mul(f, AR::ldt(eout + ii));
                    const ff gc = AR::mul(g, tg.ca[a]), gs = AR::mul(g, tg.sa[a]);
                    AR::st(bre + ii, AR::dot2(gc, ur, gs, ui));
                    AR::st(bim + ii, AR::dot2(gc, ui, AR::neg(gs), ur));
                }
            }
        }
        __syncwarp();
    }
}

// One z-translation column m, outputs n' = m + q + G a (a < NA), kept where
// n' < nout: out(n',m) = sum_{k=kbeg}^{kend-1} H_m[k-m][n'-m] in(k,m), in
// place.  H_m's output rows are zero-padded to a multiple of 8 (HR), so the
// coefficient loads need no bounds check.
template <class AR, int G, int NA>
__device__ __forceinline__ void z_column(typename AR::Stor *b, const typename AR::T *__restrict__ Hm, int HR, int m,
                                         int kbeg, int kend, int nout, int q)
{
    using T = typename AR::T;
    using Acc = typename AR::Acc;
    Acc ar[NA], ai[NA];
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        ar[a] = AR::acc0();
        ai[a] = AR::acc0();
    }
    if (kbeg < kend) {
        // row k of column m: real part at ro = k(k+1) + m, imaginary part at
        // ro + k + 1; both advance by 2(k+1) per row
        const T *h_p = Hm + (long long)(kbeg - m) * HR + q;
        int ro = kbeg * (kbeg + 1) + m, step = 2 * (kbeg + 1);
        T xr = AR::ld(b + ro), xi = AR::ld(b + ro + kbeg + 1);
        T hc[NA];
#pragma unroll
        for (int a = 0; a < NA; ++a) hc[a] = AR::ldt(h_p + G * a);
#pragma unroll 2
        for (int k = kbeg; k < kend - 1; ++k) {  // the operands of row k+1 load before row k's multiply-adds
            ro += step;
            step += 2;
            h_p += HR;
            const T xrn = AR::ld(b + ro), xin = AR::ld(b + ro + k + 2);
            T hn[NA];
#pragma unroll
            for (int a = 0; a < NA; ++a) hn[a] = AR::ldt(h_p + G * a);
#pragma unroll
            for (int a = 0; a < NA; ++a) {
                AR::mac(ar[a], hc[a], xr);
                AR::mac(ai[a], hc[a], xi);
            }
            xr = xrn;
            xi = xin;
#pragma unroll
            for (int a = 0; a < NA; ++a) hc[a] = hn[a];
        }
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            AR::mac(ar[a], hc[a], xr);
            AR::mac(ai[a], hc[a], xi);
        }
    }
    __syncwarp();
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        const int np = m + q + G * a;
        if (np < nout) {
            AR::st(b + np * (np + 1) + m, AR::fin(ar[a]));
            AR::st(b + (np + 1) * (np + 1) + m, AR::fin(ai[a]));
        }
    }
    __syncwarp();
}

// e^{i q gamma} by binary powers of e^{i gamma}, then steps of e^{i G gamma}:
// the rotation factors of the elements m = q + G a a thread owns.
template <int G, int ACC, class C, class Mul, class Out>
__device__ __forceinline__ void rotation_powers(C ea, C eb, C one, int q, Mul cmul_, Out out)
{
    C pa = one, pb = one, ka = ea, kb = eb;
#pragma unroll
    for (int bit = 1; bit < G; bit <<= 1) {
        if (q & bit) {
            pa = cmul_(pa, ka);
            pb = cmul_(pb, kb);
        }
        ka = cmul_(ka, ka);
        kb = cmul_(kb, kb);
    }
#pragma unroll
    for (int a = 0; a < ACC; ++a) {
        out(a, pa, pb);
        if (a + 1 < ACC) {
            pa = cmul_(pa, ka);
            pb = cmul_(pb, kb);
        }
    }
}

struct cff {
    ff c, s;
};

// Degree n of every coefficient index c below kDegreeTableSize (n(n+1) <= c
// < (n+1)(n+2)): the FP32-range kernels scale each coefficient by a power of
// two per degree in the gather and the target update, and one cached byte
// load per coefficient issues fewer instructions than computing the degree.
// Covers the buffers of every order those kernels run (up to 28: at most
// 28 * 29 + 4 slots plus padding), checked on the host against
// kDegreeTableSize.
struct DegreeTable {
    unsigned char d[kDegreeTableSize];
};
constexpr DegreeTable make_degree_table()
{
    DegreeTable t{};
    int n = 0;
    for (int c = 0; c < kDegreeTableSize; ++c) {
        while ((n + 1) * (n + 2) <= c) ++n;
        t.d[c] = (unsigned char)n;
    }
    return t;
}
__device__ const DegreeTable kDegree = make_degree_table();
__device__ __forceinline__ int degree_at(int c) { return (int)__ldg(kDegree.d + c); }

// source coefficient times 2^e in the arithmetic's storage type (exact)
__device__ __forceinline__ ff src_scaled(double x, int e, const ff *) { return ff_from_d_scaled0(x, e); }
__device__ __forceinline__ float src_scaled(float x, int e, const float *) { return f_scaled(x, e); }
// FP64 sources of the FP32 kernel: scaled in FP64 first, so that sources
// beyond the FP32 range come into it
__device__ __forceinline__ float src_scaled(double x, int e, const float *) { return (float)d_scaled(x, e); }

// Per-thread geometry of one translation: |shift|, its inverse and the
// rotation factors.  FP64 for the FP64 and FP32 kernels; float-float for the
// split kernels, which then execute no FP64 instruction here (GB300's FP64
// pipe runs at 1/64 of the FP32 rate).
template <class AR, int G, int ACC, bool FIX>
struct Geometry {
    using T = typename AR::T;
    T r, rinv;           // |shift| and 1/|shift| in the arithmetic
    double rd, rinvd;    // the same in FP64 (FP64 and FP32 kernels)
    Trig<AR, ACC> tg;
    FixTrig<ACC> tq;

    __device__ __forceinline__ Geometry(double x, double y, double z, int q)
    {
        if constexpr (AR::split) {
            using A = arith<ff>;
            const ff fx = ff_from_d_int(x), fy = ff_from_d_int(y), fz = ff_from_d_int(z);
            const ff rxy2 = A::dot2(fx, fx, fy, fy);
            const ff rxy = ff_sqrt(rxy2);
            r = ff_sqrt(A::add(rxy2, A::mul(fz, fz)));
            rinv = ff_rcp(r);
            rd = rinvd = 0.0;
            cff ea{ff{1.f, 0.f}, ff{0.f, 0.f}};
            if (rxy.hi > 0.f) {
                const ff rr = ff_rcp(rxy);
                ea = cff{A::mul(fy, rr), A::mul(fx, rr)};
            }
            const cff eb{A::mul(fz, rinv), A::neg(A::mul(rxy, rinv))};
            auto cm = [](cff a, cff b) {
                return cff{A::dot2(a.c, b.c, A::neg(a.s), b.s), A::dot2(a.s, b.c, a.c, b.s)};
            };
            rotation_powers<G, ACC>(ea, eb, cff{ff{1.f, 0.f}, ff{0.f, 0.f}}, q, cm, [&](int a, cff pa, cff pb) {
                tg.ca[a] = pa.c;
                tg.sa[a] = pa.s;
                tg.cb[a] = pb.c;
                tg.sb[a] = pb.s;
                if constexpr (FIX) {  // Q1.30
                    tq.c[a] = __float2int_rn(pb.c.hi * 1073741824.f) + __float2int_rn(pb.c.lo * 1073741824.f);
                    tq.s[a] = __float2int_rn(pb.s.hi * 1073741824.f) + __float2int_rn(pb.s.lo * 1073741824.f);
                }
            });
        } else {
            const double rxy = hypot(x, y);
            rd = hypot(rxy, z);
            rinvd = 1.0 / rd;
            r = AR::from_d(rd);
            rinv = AR::from_d(rinvd);
            const cd ea = (rxy == 0) ? cd{1.0, 0.0} : cd{y / rxy, x / rxy};
            const cd eb = cd{z * rinvd, -rxy * rinvd};
            rotation_powers<G, ACC>(ea, eb, cd{1.0, 0.0}, q, [](cd a, cd b) { return cmul(a, b); },
                                    [&](int a, cd pa, cd pb) {
                                        tg.ca[a] = AR::from_d(pa.c);
                                        tg.sa[a] = AR::from_d(pa.s);
                                        tg.cb[a] = AR::from_d(pb.c);
                                        tg.sb[a] = AR::from_d(pb.s);
                                    });
        }
    }
};

// FIX selects block fixed-point swaps and beta rotations (float-float only).
// HBM: expansions in device memory (L2 prefetch and a 4x unrolled gather);
// false for host memory read over the link, where both cost end-to-end rate.
// WORK: tiles come from a work list (persistent launches of fused plans)
// instead of a fixed stride over the batch.
template <class A, int G, int ACC, bool FIX = false, bool HBM = true, bool WORK = false>
__global__ void __launch_bounds__(256) k_translate(KParams p)
{
    using AR = arith<A>;
    using T = typename AR::T;
    using S = typename AR::Stor;
    using Src = typename src_of<A>::type;
    static_assert(sizeof(S) == sizeof(Src), "buffer slots hold one source value");
    static_assert(32 % G == 0, "a translation's threads must share a warp");
    static_assert(!FIX || AR::split, "fixed-point swaps are a float-float variant");

    // Loads in flight per lane in the source gather and the target update,
    // measured on GB300 (M2L P=16, 10^6): 8 and 4 make the split kernel 2.2%
    // and the FP32 kernel 3.7% faster than 4 and 1, which the FP64 and
    // float-float kernels keep (1.5% and 0.7% slower with 8 and 4).
    constexpr bool kDeep = FIX || std::is_same<A, float>::value;
    // FP32-range arithmetics run every translation at the length scale of
    // its shift: lambda = 2^ks with |shift| / lambda in [2, 7), sources (and
    // the shift) divided by lambda^n (multipoles) or lambda^-(n+1) (locals),
    // results multiplied back -- the operators are homogeneous, and powers of
    // two are exact, so only the range changes.  With r = |shift| / lambda in
    // [2, 7) the edge factors (r^-(n+1) or r^n times the basis factors
    // sqrt((n-m)!(n+m)!) or their inverses, up to 5e35 at order 28) stay
    // inside the FP32 range at every geometry scale; shifts whose largest
    // component lies in [2, 4) run unscaled
    constexpr bool kScale = !std::is_same<A, double>::value;
    constexpr int kGatherUnroll = kDeep ? 8 : 4;
    constexpr int kAccUnroll = kDeep ? 4 : 1;

    extern __shared__ __align__(16) unsigned char smem[];
    const int TS = p.TS;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const int nwarps = blockDim.x >> 5;
    const int q = tid % G;
    const int slot = tid / G;
    const int P = p.P;
    const unsigned FULL = 0xffffffffu;

    S *buf0 = reinterpret_cast<S *>(smem);
    uint32_t *meta = reinterpret_cast<uint32_t *>(smem + (size_t)TS * p.spad * sizeof(S));
    uint32_t *m_sidx = meta;
    uint32_t *m_tidx = meta + TS;
    uint32_t *m_pin = meta + 2 * TS;
    uint32_t *m_pout = meta + 3 * TS;
    uint32_t *m_id = meta + 4 * TS;

    const T *W = reinterpret_cast<const T *>(p.W);
    const T *EIN = reinterpret_cast<const T *>(p.ein);
    const T *EOUT = reinterpret_cast<const T *>(p.eout);
    const T *H = reinterpret_cast<const T *>(p.H);
    const Src *src = reinterpret_cast<const Src *>(p.src);
    Src *dst = reinterpret_cast<Src *>(p.dst);
    const int op = p.op;

    for (long long tile = blockIdx.x;; tile += gridDim.x) {
        // this tile's range of the processing order: a fixed stride over the
        // batch, or the next entry of the work list (its two words after the
        // meta arrays: work-list launches carry 8 more bytes of shared memory)
        long long base = tile * TS;
        int cnt = TS;
        if constexpr (WORK) {
            uint32_t *wsh = meta + 5 * TS;
            if (tid == 0) {
                const unsigned w = atomicAdd(p.work_counter, 1u);
                const uint2 d = w < (unsigned long long)p.nwork ? p.work[w] : make_uint2(0u, 0xffffffffu);
                wsh[0] = d.x;
                wsh[1] = d.y;
            }
            __syncthreads();
            if (wsh[1] == 0xffffffffu) break;
            base = wsh[0];
            cnt = (int)wsh[1];
        } else if (base >= p.n) {
            break;
        }
        const long long i = base + slot;
        bool valid = i < p.n;
        if constexpr (WORK) valid = valid && slot < cnt;
        uint32_t t = 0, si = 0, ti = 0;
        if (valid) t = p.perm ? p.perm[i] : (uint32_t)i;
        int pin = 0, pout = 0;
        if (valid && t < p.nidx) {
            si = p.sidx ? p.sidx[t] : t;
            ti = p.tidx ? p.tidx[t] : t;
            pin = (int)p.pin[t];
            pout = (int)p.pout[t];
        }
        // malformed entries (the unchecked API's undefined behaviour) are
        // skipped and reported instead of touching memory out of bounds
        if (valid && (t >= p.nidx || si >= p.nsrc || ti >= p.ndst || pin > P || pout > P || pin < 0 || pout < 0)) {
            if (q == 0) atomicOr(p.status, 1);
            valid = false;
            pin = pout = 0;
        }
        double x = 0, y = 0, z = 1;
        if (valid) {
            x = p.shift[3 * (long long)t];
            y = p.shift[3 * (long long)t + 1];
            z = p.shift[3 * (long long)t + 2];
        }
        if (op == OP_M2M) {  // M2M translates by the negated shift (translations.cpp:331-333)
            x = -x;
            y = -y;
            z = -z;
        }
        const bool ident = valid && op != OP_M2L && (x * x + y * y + z * z) == 0.0;
        int ident_p = 0;
        if (ident) {  // zero shift: direct prefix add (translations.cpp:540-547)
            ident_p = min(pin, pout);
            pin = 0;
            pout = 0;
            x = 0;
            y = 0;
            z = 1;
        }
        if (op == OP_L2L) pout = min(pin, pout);  // output degrees >= P_in receive nothing (translations.cpp:412)
        int ks = 0;
        if constexpr (kScale) {
            const int e3 = max(exp_of(x), max(exp_of(y), exp_of(z)));  // |shift| in [2^e3, sqrt(3) 2^(e3+1))
            if (valid && !ident && e3 > -(1 << 19)) {
                ks = e3 - 1;
                x = d_scaled(x, -ks);
                y = d_scaled(y, -ks);
                z = d_scaled(z, -ks);
            }
        }
        if (q == 0) {
            m_sidx[slot] = valid ? si : 0;
            m_tidx[slot] = valid ? ti : 0;
            m_pin[slot] = (uint32_t)pin | ((uint32_t)(ks + 32768) << 16);  // order, and the scale above it
            m_pout[slot] = pout;
            m_id[slot] = ident_p;
        }
        __syncthreads();

        // 1. gather sources into the buffer (one warp per expansion, lanes over
        //    coefficients) in the arithmetic's storage format, zero past each
        //    source's order and in the padding (the swap loops read a few
        //    slots past a row and multiply them by zero coefficients).
        //    Sources and targets stream through with evict-first hints so the
        //    coefficient tables stay in the L1 left beside the buffers.
        for (int s = warp; s < TS; s += nwarps) {
            const int ps = (int)(m_pin[s] & 0xffffu);
            const int cnt = ps * (ps + 1);
            const Src *sp = p.src_ptr ? reinterpret_cast<const Src *>(p.src_ptr[m_sidx[s]])
                                      : src + (long long)m_sidx[s] * p.sstride;
            S *bp = buf0 + (long long)s * p.spad;
            if constexpr (kScale) {  // coefficient c of degree n times lambda^-n or lambda^(n+1)
                const int ksg = (int)(m_pin[s] >> 16) - 32768;
                const int es = op == OP_L2L ? ksg : -ksg;  // per degree
                const int e0 = op == OP_L2L ? ksg : 0;
#pragma unroll(kGatherUnroll)
                for (int c = lane; c < p.spad; c += 32)
                    AR::st(bp + c, c < cnt ? src_scaled(__ldcs(sp + c), es * degree_at(c) + e0, (const T *)nullptr)
                                           : AR::zero());
            } else if constexpr (HBM) {  // kGatherUnroll loads in flight per lane
#pragma unroll(kGatherUnroll)
                for (int c = lane; c < p.spad; c += 32)
                    AR::st(bp + c, c < cnt ? AR::from_src(__ldcs(sp + c)) : AR::zero());
            } else {
                for (int c = lane; c < p.spad; c += 32)
                    AR::st(bp + c, c < cnt ? AR::from_src(__ldcs(sp + c)) : AR::zero());
            }
        }
        __syncthreads();

        // L2 prefetch, spread over the group: this tile's targets (read at the
        // end of the tile) and the next tile's sources (read at its start),
        // so that both phases meet L2 instead of DRAM.  Device arrays only;
        // every address lies inside an expansion the entry may touch.
        if (HBM && !WORK && !p.src_ptr) {
            const int tc = max(pout * (pout + 1), ident_p * (ident_p + 1));
            if (valid && tc) {
                const char *dp = reinterpret_cast<const char *>(dst + (long long)ti * p.dstride);
                for (int o = q * 128; o < tc * (int)sizeof(Src); o += G * 128) prefetch_l2(dp + o);
            }
            const long long i2 = (tile + gridDim.x) * TS + slot;
            if (i2 < p.n) {
                const uint32_t t2 = p.perm ? p.perm[i2] : (uint32_t)i2;
                if (t2 < p.nidx) {
                    const uint32_t s2 = p.sidx ? p.sidx[t2] : t2;
                    const int pin2 = (int)p.pin[t2];
                    if (s2 < p.nsrc && pin2 > 0 && pin2 <= P) {
                        const char *sp2 = reinterpret_cast<const char *>(src + (long long)s2 * p.sstride);
                        for (int o = q * 128; o < pin2 * (pin2 + 1) * (int)sizeof(Src); o += G * 128)
                            prefetch_l2(sp2 + o);
                    }
                }
            }
        }

        S *b = buf0 + (long long)slot * p.spad;
        const int pin_w = __reduce_max_sync(FULL, pin);
        const int pout_w = __reduce_max_sync(FULL, pout);

        // geometry (euler, microkernel_generic.cpp:37-97)
        Geometry<AR, G, ACC, FIX> geo(x, y, z, q);
        const Trig<AR, ACC> &tg = geo.tg;
        const FixTrig<ACC> &tq = geo.tq;

        // 2. forward transforms, degree by degree
        const bool Lin = (op == OP_L2L);
        // r-power scale of degree n: r^n (L input) or r^-(n+1) (M input).
        // Float-float steps by repeated multiplication (FP32 pipe, error
        // ~n 2^-48); FP64 and FP32 take every power from the FP64 product.
        constexpr bool kFF = AR::split;
        double rp = Lin ? 1.0 : geo.rinvd;
        const double rpstep = Lin ? geo.rd : geo.rinvd;
        T f = Lin ? AR::from_d(1.0) : geo.rinv;
        const T rstep = Lin ? geo.r : geo.rinv;
        for (int n = 0; n < pin_w; ++n) {
            if (!kFF) f = AR::from_d(rp);
            const T *ein = EIN + n * (n + 1) / 2;
            if constexpr (FIX) {
                const int *WRq = p.Wq + __ldg(p.woff + n);
                dispatch<ACC>((n + G) / G, [&](auto na) {
                    forward_degree_fixed<G, decltype(na)::value, ACC>(b, n, WRq, ein, f, q, tg, tq);
                });
            } else {
                const T *WR = W + __ldg(p.woff + n);
                dispatch<ACC>((n + G) / G, [&](auto na) {
                    forward_degree<AR, G, decltype(na)::value, ACC>(b, n, WR, ein, f, q, tg);
                });
            }
            if (kFF) f = AR::mul(f, rstep);
            if (!kFF) rp *= rpstep;
        }

        // 3. z-translation, column by column.  Columns m >= min(P_in, P_out)
        //    of the outputs stay zero (trans2swap_buf, microkernel_generic.cpp:308-338):
        //    their rows beyond P_in were zero-filled by the gather.
        const int nout_w = pout_w;
        const int mend = min(pin_w, pout_w);
        for (int m = 0; m < mend; ++m) {
            const int HR = (p.Ptab - m + p.rowpad - 1) & ~(p.rowpad - 1);
            const T *Hm = H + __ldg(p.hoff + m);
            // M2M only needs inputs k <= n' and L2L only k >= n'
            const int kbeg = (op == OP_L2L) ? m + q : m;
            const int kend = (op == OP_M2M) ? min(pin_w, nout_w) : pin_w;
            dispatch<ACC>((nout_w - m + G - 1) / G, [&](auto na) {
                z_column<AR, G, decltype(na)::value>(b, Hm, HR, m, kbeg, kend, nout_w, q);
            });
        }

        // 4. backward transforms
        const bool Mout = (op == OP_M2M);
        double rq = Mout ? geo.rd : 1.0;  // r^(n+1) (M output) or r^-n (L output)
        const double rqstep = Mout ? geo.rd : geo.rinvd;
        T fo = Mout ? geo.r : AR::from_d(1.0);
        const T qstep = Mout ? geo.r : geo.rinv;
        for (int n = 0; n < nout_w; ++n) {
            if (!kFF) fo = AR::from_d(rq);
            const T f = fo;
            const T *eo = EOUT + n * (n + 1) / 2;
            if constexpr (FIX) {
                const int *WRq = p.Wq + __ldg(p.woff + n);
                dispatch<ACC>((n + G) / G, [&](auto na) {
                    backward_degree_fixed<G, decltype(na)::value, ACC>(b, n, WRq, eo, f, q, tg, tq);
                });
            } else {
                const T *WR = W + __ldg(p.woff + n);
                dispatch<ACC>((n + G) / G, [&](auto na) {
                    backward_degree<AR, G, decltype(na)::value, ACC>(b, n, WR, eo, f, q, tg);
                });
            }
            if (kFF) fo = AR::mul(fo, qstep);
            if (!kFF) rq *= rqstep;
        }
        __syncthreads();

        // 5. accumulate into the targets (one warp per expansion)
        for (int s = warp; s < TS; s += nwarps) {
            const int po = (int)m_pout[s];
            const int pid = (int)m_id[s];
            const int cnt = max(po * (po + 1), pid * (pid + 1));
            if (!cnt) continue;
            const S *bp = buf0 + (long long)s * p.spad;
            const Src *sp = p.src_ptr ? reinterpret_cast<const Src *>(p.src_ptr[m_sidx[s]])
                                      : src + (long long)m_sidx[s] * p.sstride;
            Src *dp = p.dst_ptr ? reinterpret_cast<Src *>(p.dst_ptr[m_tidx[s]]) : dst + (long long)m_tidx[s] * p.dstride;
            // back from the translation's length scale: output coefficient c of
            // degree j times lambda^j (multipoles) or lambda^-(j+1) (locals)
            const int ksa = (int)(m_pin[s] >> 16) - 32768;
            const int eo = op == OP_M2M ? ksa : -ksa, eo0 = op == OP_M2M ? 0 : -ksa;
#pragma unroll(kAccUnroll)
            for (int c = lane; c < cnt; c += 32) {
                const int j = kScale ? degree_at(c) : 0;
                if constexpr (AR::split) {
                    // hi and lo widen by exponent re-biasing; two FP64 additions
                    // (one FP64 addition after an integer-only hi + lo measured
                    // 2% slower: the kernel is issue bound, not FP64 bound)
                    double v = p.atomic ? 0.0 : (double)__ldcs(dp + c);
                    if (c < po * (po + 1)) {
                        const T t = AR::ld(bp + c);
                        const int e = eo * j + eo0;
                        const double hd = d_from_f_scaled(t.hi, e), lo = d_from_f_scaled(t.lo, e);
                        v = p.atomic ? hd + lo : (v + hd) + lo;
                    }
                    if (c < pid * (pid + 1)) v += (double)__ldcs(sp + c);
                    if (p.atomic) atomicAdd(dp + c, (Src)v);
                    else __stcs(dp + c, (Src)v);
                } else {
                    double v = 0;
                    if constexpr (kScale) {
                        if (c < po * (po + 1)) v = d_from_f_scaled(AR::ld(bp + c), eo * j + eo0);
                    } else if (c < po * (po + 1)) {
                        v = AR::to_d(AR::ld(bp + c));
                    }
                    if (c < pid * (pid + 1)) v += (double)__ldcs(sp + c);
                    if (p.atomic) atomicAdd(dp + c, (Src)v);
                    else __stcs(dp + c, (Src)((double)__ldcs(dp + c) + v));
                }
            }
        }
        __syncthreads();
    }
}

}  // namespace sfmm
