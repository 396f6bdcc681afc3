// Block fixed-point swaps and rotations for the split-precision path.
//
// Within one degree n the forward transform (swap, rotation by beta, swap)
// and the backward transform (swap, rotation by -beta, swap) run on int32
// mantissas that share one block exponent per translation and degree row:
// value = mantissa * 2^E with |mantissa| <= 2^30 after each renormalisation.
// The swap coefficients are the orthogonal W_R / W_I in Q1.30 (|w| <= 1), so
// a swap is an exact int64 multiply-accumulate (one IMAD.WIDE per term, no
// rounding) and only the renormalisation back to 30-bit mantissas rounds
// (error 2^-31 of the row's largest element); rotations multiply by cos/sin
// in Q1.30.  Every stage is norm-preserving, which bounds every partial sum
// of a swap (Cauchy-Schwarz with unit rows): |sum| <= 2^30 ||x||_2 <=
// 2^30 sqrt(2d) 2^30 (the rotation can leave one part of an element at
// sqrt(2) 2^30), below 2^63 for d <= 28; a rotated element stays below 2^31.
//
// The edges (scaling, rotation by alpha) and the z-translation stay in
// float-float; rows are converted to fixed point after the forward edge and
// back before the z-translation, and again around the backward swaps.
#pragma once

#include <cstdint>

#include "sfmm_arith.cuh"

namespace sfmm {

// maximum over the G threads of a translation (G a power of two <= 32)
template <int G>
__device__ __forceinline__ float group_max(float v)
{
#pragma unroll
    for (int o = 1; o < G; o <<= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Mantissa width after every renormalisation: |m| <= 2^kFixBits (the
// overflow bound above holds for kFixBits <= 30 and degrees below 28).
constexpr int kFixBits = 30;

// Block exponent for a row whose largest |hi| is mx: mantissas
// round(v * 2^-E) then satisfy |m| <= 2^kFixBits.  Zero rows get E = 0.
__device__ __forceinline__ int block_exponent(float mx)
{
    if (!(mx > 0.f)) return 0;
    const int e = ((__float_as_int(mx) >> 23) & 0xff) - 127;  // mx in [2^e, 2^(e+1))
    return e + 1 - kFixBits;
}

// float-float value -> mantissa at block exponent E (rounded, |error| <= 1)
__device__ __forceinline__ int ff_to_fixed(ff v, int E)
{
    return __float2int_rn(ldexp2(v.hi, -E)) + __float2int_rn(ldexp2(v.lo, -E));
}

// mantissa at block exponent E -> float-float (exact)
__device__ __forceinline__ ff fixed_to_ff(int m, int E)
{
    const float hi = __int2float_rn(m);
    const float lo = __int2float_rn(m - __float2int_rn(hi));
    return ff{ldexp2(hi, E), ldexp2(lo, E)};
}

// Shift that brings the int64 accumulators of one degree row (all G threads
// of the translation) to at most kFixBits bits; the block exponent grows by
// the shift.  The bit length comes from the OR of one's-complement
// magnitudes: v ^ (v >> 63) is |v| or |v| - 1, whose bit length can only
// undercount for v = -2^k, which then narrows to exactly -2^kFixBits.  The
// group maximum runs on the 32-bit bit lengths.
template <int G, int NA>
__device__ __forceinline__ int group_renorm_shift(const long long (&ar)[NA], const long long (&ai)[NA])
{
    unsigned long long o = 0;
#pragma unroll
    for (int a = 0; a < NA; ++a)
        o |= (unsigned long long)(ar[a] ^ (ar[a] >> 63)) | (unsigned long long)(ai[a] ^ (ai[a] >> 63));
    int used = 64 - __clzll((long long)o);
#pragma unroll
    for (int k = 1; k < G; k <<= 1) used = max(used, __shfl_xor_sync(0xffffffffu, used, k));
    return used > kFixBits ? used - kFixBits : 0;
}

__device__ __forceinline__ int round_shift(long long a, int s)
{
    return s ? (int)((a + (1ll << (s - 1))) >> s) : (int)a;
}

// (c*x - s*y) in Q1.30, rounded
__device__ __forceinline__ int rot_q30(int c, int x, int s, int y)
{
    const long long t = (long long)c * x - (long long)s * y;
    return (int)((t + (1ll << 29)) >> 30);
}

// Integer swap of one degree, both parts: rows i = q + G a (a < NA) of the
// Q1.30 matrices applied to the int32 mantissas stored in the buffer slots
// (low word of each 8-byte slot).  Same coefficient layout (slot t: R rows of
// W_R, then R rows of W_I), padding and software pipelining as the
// floating-point swap.
template <int G, int NA, int R>
__device__ __forceinline__ void swap_both_fixed(const int *__restrict__ W, const float2 *xre, const float2 *xim,
                                                int d, int n, int q, long long (&ar)[NA], long long (&ai)[NA])
{
    const int jr0 = (q + n) & 1, ji0 = jr0 ^ 1;
    const int cnt = (d + 1) >> 1;
    const int *w = W + q;
    const int *xr_p = reinterpret_cast<const int *>(xre + jr0);
    const int *xi_p = reinterpret_cast<const int *>(xim + ji0);
    int xrn = *xr_p, xin = *xi_p;
    int wrn[NA], win[NA];
#pragma unroll
    for (int a = 0; a < NA; ++a) {
        wrn[a] = __ldg(w + G * a);
        win[a] = __ldg(w + R + G * a);
    }
#pragma unroll 4  // measured on GB300: 4 beats 2 by 0.6% at P=16, 8 and 1 lose
    for (int t = 0; t < cnt; ++t) {
        const int xr = xrn, xi = xin;
        int wr[NA], wi[NA];
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            wr[a] = wrn[a];
            wi[a] = win[a];
        }
        xr_p += 4;  // two 8-byte slots
        xi_p += 4;
        w += 2 * R;
        xrn = *xr_p;
        xin = *xi_p;
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            wrn[a] = __ldg(w + G * a);
            win[a] = __ldg(w + R + G * a);
        }
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            ar[a] += (long long)wr[a] * xr;
            ai[a] += (long long)wi[a] * xi;
        }
    }
}

}  // namespace sfmm
