// Arithmetic policies for the translation kernels.
//
//   double : plain FP64 (DFMA pipe)
//   float  : plain FP32
//   ff     : double-FP32 ("float-float", hi + lo) on the FP32 pipe.  Products
//            are split exactly with an FMA (Dekker/Ogita-Rump-Oishi TwoProduct),
//            sums use Knuth's TwoSum; accumulations keep an unnormalised low
//            word and renormalise once at the end (Fast2Sum).  Every
//            intermediate carries ~44+ bits, which keeps the relative error of a
//            whole translation near 1e-13 although each operation runs on FP32.
//            __fmul_rn/__fadd_rn stop the compiler from contracting the
//            error-free transformations into FMAs.
#pragma once

#include <cuda_runtime.h>

namespace sfmm {

struct ff {
    float hi, lo;
};

template <class A>
struct arith;

template <>
struct arith<double> {
    static constexpr bool split = false;
    using T = double;
    using Stor = double;  // element type of the shared-memory buffer
    using Acc = double;
    static __device__ __forceinline__ T zero() { return 0.0; }
    static __device__ __forceinline__ T from_d(double x) { return x; }
    static __device__ __forceinline__ T from_src(double x) { return x; }
    static __device__ __forceinline__ double to_d(T x) { return x; }
    static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
    static __device__ __forceinline__ T add(T a, T b) { return a + b; }
    static __device__ __forceinline__ T sub(T a, T b) { return a - b; }
    static __device__ __forceinline__ T neg(T a) { return -a; }
    static __device__ __forceinline__ Acc acc0() { return 0.0; }
    static __device__ __forceinline__ void mac(Acc &acc, T w, T x) { acc = fma(w, x, acc); }
    static __device__ __forceinline__ T fin(Acc a) { return a; }
    static __device__ __forceinline__ T ld(const Stor *p) { return *p; }
    static __device__ __forceinline__ void st(Stor *p, T v) { *p = v; }
    static __device__ __forceinline__ T ldt(const T *p) { return __ldg(p); }
    // a1*b1 + a2*b2
    static __device__ __forceinline__ T dot2(T a1, T b1, T a2, T b2) { return fma(a1, b1, a2 * b2); }
};

template <>
struct arith<float> {
    static constexpr bool split = false;
    using T = float;
    using Stor = float;
    using Acc = float;
    static __device__ __forceinline__ T zero() { return 0.f; }
    static __device__ __forceinline__ T from_d(double x) { return (float)x; }
    static __device__ __forceinline__ T from_src(float x) { return x; }
    static __device__ __forceinline__ double to_d(T x) { return (double)x; }
    static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
    static __device__ __forceinline__ T add(T a, T b) { return a + b; }
    static __device__ __forceinline__ T sub(T a, T b) { return a - b; }
    static __device__ __forceinline__ T neg(T a) { return -a; }
    static __device__ __forceinline__ Acc acc0() { return 0.f; }
    static __device__ __forceinline__ void mac(Acc &acc, T w, T x) { acc = fmaf(w, x, acc); }
    static __device__ __forceinline__ T fin(Acc a) { return a; }
    static __device__ __forceinline__ T ld(const Stor *p) { return *p; }
    static __device__ __forceinline__ void st(Stor *p, T v) { *p = v; }
    static __device__ __forceinline__ T ldt(const T *p) { return __ldg(p); }
    static __device__ __forceinline__ T dot2(T a1, T b1, T a2, T b2) { return fmaf(a1, b1, a2 * b2); }
};

// Fast2Sum: |a| >= |b| assumed (or a == 0)
__device__ __forceinline__ ff ff_norm(float a, float b)
{
    float s = __fadd_rn(a, b);
    float e = __fsub_rn(b, __fsub_rn(s, a));
    return ff{s, e};
}

__device__ __forceinline__ ff ff_from_d(double x)
{
    float h = __double2float_rn(x);
    float l = __double2float_rn(x - (double)h);
    return ff{h, l};
}

__device__ __forceinline__ double ff_to_d(ff a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ ff ff_add(ff a, ff b)
{
    float s = __fadd_rn(a.hi, b.hi);
    float v = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return ff_norm(s, e);
}

__device__ __forceinline__ ff ff_mul(ff a, ff b)
{
    float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return ff_norm(p, e);
}

// 2^e (|e| <= 126) as a float, and x * 2^e as two exact power-of-two
// multiplications (the first never leaves the normal range for the
// exponents used here, so only the final product rounds).
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }
__device__ __forceinline__ float ldexp2(float x, int e)
{
    const int e1 = e / 2;
    return __fmul_rn(__fmul_rn(x, pow2f(e1)), pow2f(e - e1));
}

// x 2^sh as float-float with integer and FP32 operations only (the FP64
// pipe is 1/64 of the FP32 rate).  The 53-bit significand M splits into its
// top 24 bits A (exact in a float) and the remaining 29 bits B (rounded to 24
// bits); x 2^sh = A 2^k + B 2^(k-29), the shift folded into k, then one
// Fast2Sum.  The pair represents x 2^sh to about 2^-48 relative; results
// below 2^-151 become 0, from 2^128 they overflow.
__device__ __forceinline__ ff ff_from_d_scaled(double x, int sh)
{
    const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
    const int e = (int)((hw >> 20) & 0x7ffu);
    const unsigned A = 0x800000u | ((hw & 0xfffffu) << 3) | (lw >> 29);
    const unsigned B = lw & 0x1fffffffu;
    const int k = min(e - 1023 - 23 + sh, 106);
    float h = ldexp2(__uint2float_rn(A), k);
    float l = ldexp2(__uint2float_rn(B), k - 29);
    if (e - 1023 + sh < -151) h = l = 0.f;  // zero and subnormal x too, for |sh| < 872
    if (hw >> 31) {
        h = -h;
        l = -l;
    }
    return ff_norm(h, l);
}

// double -> float-float without FP64 instructions
__device__ __forceinline__ ff ff_from_d_int(double x) { return ff_from_d_scaled(x, 0); }

// ff_from_d_scaled for shifts of any size: zero and subnormal x give 0
// (above a shift of 872 the range test alone would miss them)
__device__ __forceinline__ ff ff_from_d_scaled0(double x, int sh)
{
    if ((((unsigned)__double2hiint(x) >> 20) & 0x7ffu) == 0u) return ff{0.f, 0.f};
    return ff_from_d_scaled(x, sh);
}

// float -> double by re-biasing the exponent (exact); zero included, other
// non-normal values take the conversion instruction.
__device__ __forceinline__ double d_from_f_int(float f)
{
    const unsigned w = __float_as_uint(f);
    const unsigned ex = (w >> 23) & 0xffu;
    if ((w << 1) == 0u) return __hiloint2double((int)(w & 0x80000000u), 0);
    if (ex == 0u || ex == 0xffu) return (double)f;
    const unsigned hi = (w & 0x80000000u) | ((ex + 896u) << 20) | ((w & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)(w << 29));
}

// binary exponent of x (x = f 2^e, f in [1, 2)); zero and subnormals give a
// value below every other
__device__ __forceinline__ int exp_of(double x)
{
    const int e = (int)(((unsigned)__double2hiint(x) >> 20) & 0x7ffu);
    return e ? e - 1023 : -(1 << 20);
}
__device__ __forceinline__ int exp_of(float x)
{
    const int e = (int)((__float_as_uint(x) >> 23) & 0xffu);
    return e ? e - 127 : -(1 << 20);
}

// x 2^e through the exponent field (exact): zero and subnormal x give zero,
// results beyond the normal range zero or infinity
__device__ __forceinline__ float f_scaled(float x, int e)
{
    const unsigned w = __float_as_uint(x);
    const int ex = (int)((w >> 23) & 0xffu);
    if (ex == 0 || ex == 0xff) return ex ? x : __uint_as_float(w & 0x80000000u);
    const int ne = ex + e;
    if (ne <= 0) return __uint_as_float(w & 0x80000000u);
    if (ne >= 0xff) return __uint_as_float((w & 0x80000000u) | 0x7f800000u);
    return __uint_as_float((w & 0x807fffffu) | ((unsigned)ne << 23));
}

// double x 2^e through the exponent field (exact): zero and subnormal x
// give zero, results beyond the normal range zero or infinity
__device__ __forceinline__ double d_scaled(double x, int e)
{
    const int h = __double2hiint(x);
    const int ex = (int)(((unsigned)h >> 20) & 0x7ffu);
    const int sg = h & (int)0x80000000u;
    if (ex == 0) return __hiloint2double(sg, 0);
    if (ex == 0x7ff) return x;
    const int ne = ex + e;
    if (ne <= 0) return __hiloint2double(sg, 0);
    if (ne >= 0x7ff) return __hiloint2double(sg | 0x7ff00000, 0);
    return __hiloint2double((h & (int)0x800fffffu) | (ne << 20), __double2loint(x));
}

// d_from_f_scaled for the rare inputs: zero, subnormal f (normalised
// first), infinity and NaN, and results beyond the double range (zero below,
// infinity above)
__device__ __forceinline__ double d_from_f_scaled_rare(float f, int e)
{
    unsigned w = __float_as_uint(f);
    int ex = (int)((w >> 23) & 0xffu);
    const unsigned sg = w & 0x80000000u;
    if (ex == 0) {
        if ((w << 1) == 0u) return __hiloint2double((int)sg, 0);
        w = __float_as_uint(f * 16777216.f);  // exact: 2^24
        ex = (int)((w >> 23) & 0xffu);
        e -= 24;
    }
    if (ex == 0xff) return (double)f;
    const int ne = ex + 896 + e;
    if (ne <= 0) return __hiloint2double((int)sg, 0);
    if (ne >= 2047) return __hiloint2double((int)(sg | 0x7ff00000u), 0);
    const unsigned hi = sg | ((unsigned)ne << 20) | ((w & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)(w << 29));
}

// float -> double times 2^e by re-biasing the exponent (exact; d_from_f_int
// with a shift): one range test for normal inputs with normal results, the
// other cases out of line
__device__ __forceinline__ double d_from_f_scaled(float f, int e)
{
    const unsigned w = __float_as_uint(f);
    const int ex = (int)((w >> 23) & 0xffu);
    const int ne = ex + 896 + e;
    if (__builtin_expect((unsigned)(ex - 1) < 254u && (unsigned)(ne - 1) < 2046u, 1)) {
        const unsigned hi = (w & 0x80000000u) | ((unsigned)ne << 20) | ((w & 0x7fffffu) >> 3);
        return __hiloint2double((int)hi, (int)(w << 29));
    }
    return d_from_f_scaled_rare(f, e);
}

// float-float square root and reciprocal: one Newton step from the FP32
// result (error ~2^-44 relative).
__device__ __forceinline__ ff ff_sqrt(ff a)
{
    if (!(a.hi > 0.f)) return ff{0.f, 0.f};
    const float s = __fsqrt_rn(a.hi);
    const float p = __fmul_rn(s, s);
    const float pe = __fmaf_rn(s, s, -p);
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), pe), a.lo);  // a - s^2
    return ff_norm(s, __fmul_rn(r, __fdiv_rn(0.5f, s)));
}

__device__ __forceinline__ ff ff_rcp(ff b)
{
    const float r = __frcp_rn(b.hi);
    // 1 - b r, with the b.hi r product split exactly
    const float e = __fsub_rn(__fmaf_rn(-b.hi, r, 1.f), __fmul_rn(b.lo, r));
    return ff_norm(r, __fmul_rn(r, e));
}

// unnormalised accumulator: value = hi + lo, lo collects every rounding error
struct ffacc {
    float hi, lo;
};

template <>
struct arith<ff> {
    static constexpr bool split = true;
    using T = ff;
    using Stor = float2;
    using Acc = ffacc;
    static __device__ __forceinline__ T zero() { return ff{0.f, 0.f}; }
    static __device__ __forceinline__ T from_d(double x) { return ff_from_d(x); }
    // source coefficients: converted without FP64 instructions
    static __device__ __forceinline__ T from_src(double x) { return ff_from_d_int(x); }
    static __device__ __forceinline__ double to_d(T x) { return ff_to_d(x); }
    static __device__ __forceinline__ T mul(T a, T b) { return ff_mul(a, b); }
    static __device__ __forceinline__ T add(T a, T b) { return ff_add(a, b); }
    static __device__ __forceinline__ T sub(T a, T b) { return ff_add(a, ff{-b.hi, -b.lo}); }
    static __device__ __forceinline__ T neg(T a) { return ff{-a.hi, -a.lo}; }
    static __device__ __forceinline__ Acc acc0() { return ffacc{0.f, 0.f}; }
    // acc += w * x, 11 FP32 operations
    static __device__ __forceinline__ void mac(Acc &acc, T w, T x)
    {
        float p = __fmul_rn(w.hi, x.hi);
        float e = __fmaf_rn(w.hi, x.hi, -p);
        e = __fmaf_rn(w.hi, x.lo, e);
        e = __fmaf_rn(w.lo, x.hi, e);
        float s = __fadd_rn(acc.hi, p);
        float v = __fsub_rn(s, acc.hi);
        float t = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, v)), __fsub_rn(p, v));
        acc.lo = __fadd_rn(acc.lo, __fadd_rn(t, e));
        acc.hi = s;
    }
    static __device__ __forceinline__ T fin(Acc a)
    {
        // two-sum renormalisation (lo may exceed hi after cancellation)
        float s = __fadd_rn(a.hi, a.lo);
        float v = __fsub_rn(s, a.hi);
        float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(a.lo, v));
        return ff{s, e};
    }
    static __device__ __forceinline__ T ld(const Stor *p)
    {
        float2 v = *p;
        return ff{v.x, v.y};
    }
    static __device__ __forceinline__ void st(Stor *p, T v) { *p = make_float2(v.hi, v.lo); }
    static __device__ __forceinline__ T ldt(const T *p)
    {
        float2 v = __ldg(reinterpret_cast<const float2 *>(p));
        return ff{v.x, v.y};
    }
    // a1*b1 + a2*b2 with both products split exactly and one TwoSum (19 FP32 operations)
    static __device__ __forceinline__ T dot2(T a1, T b1, T a2, T b2)
    {
        float p1 = __fmul_rn(a1.hi, b1.hi);
        float e1 = __fmaf_rn(a1.hi, b1.hi, -p1);
        e1 = __fmaf_rn(a1.hi, b1.lo, e1);
        e1 = __fmaf_rn(a1.lo, b1.hi, e1);
        float p2 = __fmul_rn(a2.hi, b2.hi);
        float e2 = __fmaf_rn(a2.hi, b2.hi, -p2);
        e2 = __fmaf_rn(a2.hi, b2.lo, e2);
        e2 = __fmaf_rn(a2.lo, b2.hi, e2);
        float s = __fadd_rn(p1, p2);
        float v = __fsub_rn(s, p1);
        float t = __fadd_rn(__fsub_rn(p1, __fsub_rn(s, v)), __fsub_rn(p2, v));
        t = __fadd_rn(t, __fadd_rn(e1, e2));
        return ff_norm(s, t);
    }
};

}  // namespace sfmm
