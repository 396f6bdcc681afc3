// Fused translation kernel: M2M, M2L and L2L over a batch of translations.
//
// One CTA processes tiles of TS translations; each translation is handled by
// G = 4 threads ("quad") that share its working expansion in a per-CTA
// buffer (shared memory, or a global scratch slice when the order is too
// large for shared memory).  Per tile:
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
// Thread q of a quad owns rows i = q + 4a (a < ACC) of every degree-n swap,
// rotation element m = q + 4a, and outputs n' = m + q + 4a of every
// z-translation column, so each stage keeps ACC accumulators in registers and
// reads its inputs from the buffer (quad members synchronise with
// __syncwarp).  Loop bounds are warp-uniform maxima over the warp's eight
// translations, exactly like the reference's lanes padded with zero orders
// (translations.cpp:504-514); inputs past a translation's own order read as
// zero and outputs past it are dropped.
#pragma once

#include <cstdint>

#include "sfmm_arith.cuh"
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

__device__ __forceinline__ long long woff_of(int n) { return (long long)n * (n + 1) * (2 * n + 1) / 3; }
__device__ __forceinline__ long long sq_sum(long long x) { return x * (x + 1) * (2 * x + 1) / 6; }
__device__ __forceinline__ long long hoff_of(int P, int m) { return sq_sum(P) - sq_sum(P - m); }

// complex helpers in FP64 for the per-translation geometry
struct cd {
    double c, s;
};
__device__ __forceinline__ cd cmul(cd a, cd b) { return cd{a.c * b.c - a.s * b.s, a.s * b.c + a.c * b.s}; }

template <class A, int ACC, bool GBUF>
__global__ void __launch_bounds__(256) k_translate(KParams p)
{
    using AR = arith<A>;
    using T = typename AR::T;
    using S = typename AR::Stor;
    using Acc = typename AR::Acc;
    using Src = typename src_of<A>::type;
    static_assert(sizeof(S) == sizeof(Src), "buffer slots hold one source value");

    extern __shared__ __align__(16) unsigned char smem[];
    const int TS = p.TS;
    const int tid = threadIdx.x;
    const int q = tid & 3;
    const int slot = tid >> 2;
    const int P = p.P;
    const int Scap = P * (P + 1);
    const unsigned FULL = 0xffffffffu;

    S *buf0;
    uint32_t *meta;
    if (GBUF) {
        buf0 = reinterpret_cast<S *>(p.scratch) + (long long)blockIdx.x * TS * p.spad;
        meta = reinterpret_cast<uint32_t *>(smem);
    } else {
        buf0 = reinterpret_cast<S *>(smem);
        meta = reinterpret_cast<uint32_t *>(smem + (size_t)TS * p.spad * sizeof(S));
    }
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

    for (long long tile = blockIdx.x; tile * TS < p.n; tile += gridDim.x) {
        const long long i = tile * TS + slot;
        bool valid = i < p.n;
        uint32_t t = 0, si = 0, ti = 0;
        if (valid) t = p.perm ? p.perm[i] : (uint32_t)i;
        int pin = 0, pout = 0;
        if (valid && t < p.n) {
            si = p.sidx ? p.sidx[t] : t;
            ti = p.tidx ? p.tidx[t] : t;
            pin = (int)p.pin[t];
            pout = (int)p.pout[t];
        }
        // malformed entries (the unchecked API's undefined behaviour) are
        // skipped and reported instead of touching memory out of bounds
        if (valid && (t >= p.n || si >= p.nsrc || ti >= p.ndst || pin > P || pout > P || pin < 0 || pout < 0)) {
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
        if (ident) {
            ident_p = min(pin, pout);
            pin = 0;
            pout = 0;
            x = 0;
            y = 0;
            z = 1;
        }
        if (op == OP_L2L) pout = min(pin, pout);  // output degrees >= P_in receive nothing (translations.cpp:412)
        if (q == 0) {
            m_sidx[slot] = valid ? si : 0;
            m_tidx[slot] = valid ? ti : 0;
            m_pin[slot] = pin;
            m_pout[slot] = pout;
            m_id[slot] = ident_p;
        }
        __syncthreads();

        // 1. gather sources into the buffer, zero past each source's order
        for (int e = tid; e < TS * Scap; e += blockDim.x) {
            int s = e / Scap;
            int c = e - s * Scap;
            int ps = (int)m_pin[s];
            Src v = 0;
            if (c < ps * (ps + 1)) v = src[(long long)m_sidx[s] * p.sstride + c];
            *reinterpret_cast<Src *>(buf0 + (long long)s * p.spad + c) = v;
        }
        __syncthreads();

        S *b = buf0 + (long long)slot * p.spad;
        const int pin_w = __reduce_max_sync(FULL, pin);
        const int pout_w = __reduce_max_sync(FULL, pout);

        // geometry in FP64 (euler, microkernel_generic.cpp:37-97)
        const double rxy = hypot(x, y);
        const double r = hypot(rxy, z);
        const double rinv = 1.0 / r;
        const cd ea = (rxy == 0) ? cd{1.0, 0.0} : cd{y / rxy, x / rxy};
        const cd eb = cd{z * rinv, -rxy * rinv};
        T ca[ACC], sa[ACC], cb[ACC], sb[ACC];
        {
            cd pa{1.0, 0.0}, pb{1.0, 0.0};
            for (int k = 0; k < q; ++k) {
                pa = cmul(pa, ea);
                pb = cmul(pb, eb);
            }
            cd a4 = cmul(cmul(ea, ea), cmul(ea, ea));
            cd b4 = cmul(cmul(eb, eb), cmul(eb, eb));
#pragma unroll
            for (int a = 0; a < ACC; ++a) {
                ca[a] = AR::from_d(pa.c);
                sa[a] = AR::from_d(pa.s);
                cb[a] = AR::from_d(pb.c);
                sb[a] = AR::from_d(pb.s);
                pa = cmul(pa, a4);
                pb = cmul(pb, b4);
            }
        }

        // 2. forward transforms, degree by degree
        const bool Lin = (op == OP_L2L);
        double rp = Lin ? 1.0 : rinv;          // r^n (L input) or r^-(n+1) (M input)
        const double rstep = Lin ? r : rinv;
        for (int n = 0; n < pin_w; ++n) {
            const int d = n + 1;
            S *bre = b + n * (n + 1);
            S *bim = b + (n + 1) * (n + 1);
            const T f = AR::from_d(rp);
            const T *ein = EIN + n * (n + 1) / 2;
#pragma unroll
            for (int a = 0; a < ACC; ++a) {
                const int m = q + 4 * a;
                if (m < d) {
                    T xr = AR::from_d((double)*reinterpret_cast<const Src *>(bre + m));
                    T xi = AR::from_d((double)*reinterpret_cast<const Src *>(bim + m));
                    T g = AR::mul(f, AR::ldt(ein + m));
                    T ur = AR::mul(g, AR::sub(AR::mul(ca[a], xr), AR::mul(sa[a], xi)));
                    T ui = AR::mul(g, AR::add(AR::mul(sa[a], xr), AR::mul(ca[a], xi)));
                    AR::st(bre + m, ur);
                    AR::st(bim + m, ui);
                }
            }
            __syncwarp();
            const T *WR = W + woff_of(n);
            const T *WI = WR + d * d;
#pragma unroll 1
            for (int pass = 0; pass < 2; ++pass) {
                Acc ar[ACC], ai[ACC];
#pragma unroll
                for (int a = 0; a < ACC; ++a) {
                    ar[a] = AR::acc0();
                    ai[a] = AR::acc0();
                }
                for (int j = (q + n) & 1; j < d; j += 2) {
                    const T xv = AR::ld(bre + j);
#pragma unroll
                    for (int a = 0; a < ACC; ++a) {
                        const int ii = q + 4 * a;
                        if (ii < d) AR::mac(ar[a], AR::ldt(WR + j * d + ii), xv);
                    }
                }
                for (int j = (q + n + 1) & 1; j < d; j += 2) {
                    const T xv = AR::ld(bim + j);
#pragma unroll
                    for (int a = 0; a < ACC; ++a) {
                        const int ii = q + 4 * a;
                        if (ii < d) AR::mac(ai[a], AR::ldt(WI + j * d + ii), xv);
                    }
                }
                __syncwarp();
#pragma unroll
                for (int a = 0; a < ACC; ++a) {
                    const int ii = q + 4 * a;
                    if (ii < d) {
                        T vr = AR::fin(ar[a]);
                        T vi = AR::fin(ai[a]);
                        if (pass == 0) {  // rotation by e^{+i m beta} between the two swaps
                            T wr = AR::sub(AR::mul(cb[a], vr), AR::mul(sb[a], vi));
                            T wi = AR::add(AR::mul(sb[a], vr), AR::mul(cb[a], vi));
                            vr = wr;
                            vi = wi;
                        }
                        AR::st(bre + ii, vr);
                        AR::st(bim + ii, vi);
                    }
                }
                __syncwarp();
            }
            rp *= rstep;
        }

        // 3. z-translation, column by column
        const int nout_w = pout_w;
        const int mend = min(pin_w, pout_w);
        const T *Hop = H;
        for (int m = 0; m < mend; ++m) {
            const int L = p.Ptab - m;
            const T *Hm = Hop + hoff_of(p.Ptab, m);
            Acc ar[ACC], ai[ACC];
#pragma unroll
            for (int a = 0; a < ACC; ++a) {
                ar[a] = AR::acc0();
                ai[a] = AR::acc0();
            }
            int kbeg = m, kend = pin_w;
            for (int k = kbeg; k < kend; ++k) {
                const T xr = AR::ld(b + k * (k + 1) + m);
                const T xi = AR::ld(b + (k + 1) * (k + 1) + m);
                const T *Hk = Hm + (long long)(k - m) * L;
#pragma unroll
                for (int a = 0; a < ACC; ++a) {
                    const int np = m + q + 4 * a;
                    if (np < nout_w) {
                        const T h = AR::ldt(Hk + (np - m));
                        AR::mac(ar[a], h, xr);
                        AR::mac(ai[a], h, xi);
                    }
                }
            }
            __syncwarp();
#pragma unroll
            for (int a = 0; a < ACC; ++a) {
                const int np = m + q + 4 * a;
                if (np < nout_w) {
                    AR::st(b + np * (np + 1) + m, AR::fin(ar[a]));
                    AR::st(b + (np + 1) * (np + 1) + m, AR::fin(ai[a]));
                }
            }
            __syncwarp();
        }
        // columns m >= min(P_in, P_out) of the outputs are zero (trans2swap_buf,
        // microkernel_generic.cpp:308-338); rows below P_in may still hold inputs
        for (int np = 0; np < nout_w; ++np) {
#pragma unroll
            for (int a = 0; a < ACC; ++a) {
                const int m = q + 4 * a;
                if (m >= mend && m <= np) {
                    AR::st(b + np * (np + 1) + m, AR::zero());
                    AR::st(b + (np + 1) * (np + 1) + m, AR::zero());
                }
            }
        }
        __syncwarp();

        // 4. backward transforms
        const bool Mout = (op == OP_M2M);
        double rq = Mout ? r : 1.0;            // r^(n+1) (M output) or r^-n (L output)
        const double qstep = Mout ? r : rinv;
        for (int n = 0; n < nout_w; ++n) {
            const int d = n + 1;
            S *bre = b + n * (n + 1);
            S *bim = b + (n + 1) * (n + 1);
            const T *WR = W + woff_of(n);
            const T *WI = WR + d * d;
            const T f = AR::from_d(rq);
            const T *eo = EOUT + n * (n + 1) / 2;
#pragma unroll 1
            for (int pass = 0; pass < 2; ++pass) {
                Acc ar[ACC], ai[ACC];
#pragma unroll
                for (int a = 0; a < ACC; ++a) {
                    ar[a] = AR::acc0();
                    ai[a] = AR::acc0();
                }
                for (int j = (q + n) & 1; j < d; j += 2) {
                    const T xv = AR::ld(bre + j);
#pragma unroll
                    for (int a = 0; a < ACC; ++a) {
                        const int ii = q + 4 * a;
                        if (ii < d) AR::mac(ar[a], AR::ldt(WR + j * d + ii), xv);
                    }
                }
                for (int j = (q + n + 1) & 1; j < d; j += 2) {
                    const T xv = AR::ld(bim + j);
#pragma unroll
                    for (int a = 0; a < ACC; ++a) {
                        const int ii = q + 4 * a;
                        if (ii < d) AR::mac(ai[a], AR::ldt(WI + j * d + ii), xv);
                    }
                }
                __syncwarp();
#pragma unroll
                for (int a = 0; a < ACC; ++a) {
                    const int ii = q + 4 * a;
                    if (ii < d) {
                        T vr = AR::fin(ar[a]);
                        T vi = AR::fin(ai[a]);
                        if (pass == 0) {  // e^{-i m beta}
                            T wr = AR::add(AR::mul(cb[a], vr), AR::mul(sb[a], vi));
                            T wi = AR::sub(AR::mul(cb[a], vi), AR::mul(sb[a], vr));
                            vr = wr;
                            vi = wi;
                        } else {  // e^{-i m alpha}, back to the solid basis, r-power scale
                            T g = AR::mul(f, AR::ldt(eo + ii));
                            T wr = AR::mul(g, AR::add(AR::mul(ca[a], vr), AR::mul(sa[a], vi)));
                            T wi = AR::mul(g, AR::sub(AR::mul(ca[a], vi), AR::mul(sa[a], vr)));
                            vr = wr;
                            vi = wi;
                        }
                        AR::st(bre + ii, vr);
                        AR::st(bim + ii, vi);
                    }
                }
                __syncwarp();
            }
            rq *= qstep;
        }
        __syncthreads();

        // 5. accumulate into the targets
        for (int e = tid; e < TS * Scap; e += blockDim.x) {
            int s = e / Scap;
            int c = e - s * Scap;
            int po = (int)m_pout[s];
            int pid = (int)m_id[s];
            if (c < po * (po + 1) || c < pid * (pid + 1)) {
                double v = 0;
                if (c < po * (po + 1)) v = AR::to_d(AR::ld(buf0 + (long long)s * p.spad + c));
                if (c < pid * (pid + 1)) v += (double)src[(long long)m_sidx[s] * p.sstride + c];
                Src *dp = dst + (long long)m_tidx[s] * p.dstride + c;
                if (p.atomic) atomicAdd(dp, (Src)v);
                else *dp = (Src)((double)*dp + v);
            }
        }
        __syncthreads();
    }
}

}  // namespace sfmm
