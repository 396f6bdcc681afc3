// Tensor-core translation kernel (tcgen05): M2M, M2L and L2L for order
// bounds up to 16, one thread per translation.
//
// A CTA of 128 threads (one warpgroup) owns one SM and walks tiles of 128
// translations; thread t holds translation t of the tile, which is row t of
// every MMA (M = 128) and lane t of tensor memory.  Every constant matrix of
// the rotation method multiplies the stacked rows of a whole tile at once:
//
//   swap of degree n   D[t][i] = sum_j X[t][j] W[i][j]     (W_R on real parts,
//                                                            W_I on imaginary)
//   z-translation, m   D[t][n'-m] = sum_k X[t][k-m] H_m[k][n']
//
// with N = K = 16.  Degrees are paired so that every MMA is full: degree
// P-1 alone, then (n, P-2-n) with n + 1 + P-1-n = P <= 16 rows, B the
// block-diagonal of the two swap matrices; z-columns likewise: column 0
// alone, then (m, P-m) with (P-m) + m = P rows.  A stage therefore takes
// (P+2)/2 (swaps) or P/2+1 (z-translation) groups instead of P.
//
// The operands are split into two pieces each (hi + lo) and multiplied as
// hi*hi + hi*lo + lo*hi, accumulated in FP32 in tensor memory: 3xTF32
// (kind::tf32) or 3xBF16 (kind::f16 with BF16 operands).  The constant
// matrices (orthogonal swap matrices W_R/W_I, z-translation matrices H_m,
// built in FP64 on the host and split there) stay in shared memory for the
// whole launch; each thread writes its row of the split A operand to shared
// memory and reads its row of D from tensor memory, so the per-element work
// around the contractions (edge scaling, azimuthal and polar rotations, the
// splits) runs in registers with no exchange between threads.
//
// Per tile (the rotation method, translations.cpp:37-316 and :319-471):
//   forward, group by group: edge (r-power, e^{i m alpha}, change to the
//     orthogonal basis), swap, e^{i m beta}, swap -> state;
//   z-translation group by group on the state, in place;
//   backward, group by group: swap, e^{-i m beta}, swap, edge -> target +=.
// Each stage is software-pipelined over two groups in flight (three A
// operand slots in shared memory, two accumulator slots in tensor memory,
// one CTA barrier per step): each step first prepares the next group's
// operand, which depends on nothing in flight, and only then waits for the
// tensor core's results of the step before.  The state (the rotated expansion, FP32) lives in
// tensor memory ordered by z-group, so that a z-group is one vector load.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

#include "sfmm_arith.cuh"
#include "sfmm_params.hpp"
#include "sfmm_tc.cuh"

namespace sfmm {

constexpr int kTcRows = 128;  // translations per tile = MMA M
constexpr int kTcMaxOrder = 16;
constexpr int kTcNodes = 16;  // MMA N and K

// Tensor-memory columns: state re / im (136 each at order 16), two
// accumulator slots of 32 columns (re, im).
constexpr uint32_t kTcStateRe = 0, kTcStateIm = 136, kTcD = 288, kTcCols = 512;

__host__ __device__ constexpr int tc_deg_groups(int P) { return (P + 2) / 2; }
__host__ __device__ constexpr int tc_z_groups(int P) { return P / 2 + 1; }

// Two degrees (or two z-columns) sharing one MMA: lanes [0, d1) belong to
// the first, [d1, d1 + d2) to the second (d2 = 0: alone).
struct TcGroup {
    int n1, n2, d1, d2;
};

// swap group g of order bound P: degree P-1, then (g-1, P-1-g)
__host__ __device__ inline TcGroup tc_deg_group(int P, int g)
{
    if (g == 0) return TcGroup{P - 1, 0, P, 0};
    const int a = g - 1, b = P - 1 - g;
    return a < b ? TcGroup{a, b, a + 1, b + 1} : TcGroup{a, 0, a + 1, 0};
}

// z group g: column 0 (P rows), then columns (g, P-g) with P-g and g rows;
// it spans state columns [g P, g P + d1 + d2)
__host__ __device__ inline TcGroup tc_z_group(int P, int g)
{
    if (g == 0) return TcGroup{0, 0, P, 0};
    const int b = P - g;
    return g < b ? TcGroup{g, b, P - g, g} : TcGroup{g, 0, P - g, 0};
}

// state column of element (n, m), m <= n < P
__host__ __device__ inline int tc_state_col(int P, int n, int m)
{
    if (m == 0) return n;
    const int g = m < P - m ? m : P - m;
    return g * P + (m == g ? 0 : P - g) + (n - m);
}

// Operand formats: 0 = 3xTF32, 1 = 3xBF16 (two pieces per operand, the three
// products hi*hi + hi*lo + lo*hi), 2 = BF16x6 (three BF16 pieces per operand,
// the six products whose pieces sum to at most 2, issued smallest first so
// that the FP32 accumulator rounds the sum about once; the edges of this
// mode run in float-float and feed the split directly).
template <int MODE>
struct TcFmt;
template <>
struct TcFmt<0> {
    static constexpr int ESZ = 4;
    static constexpr int KC = 4;      // core matrices along K = 16
    static constexpr int KSTEPS = 2;  // MMA instructions along K (K = 8 each)
    static constexpr int PIECES = 2;
    static constexpr bool FF = false;  // float-float edges
    static constexpr uint32_t FMT = tc::FMT_TF32;
};
template <>
struct TcFmt<1> {
    static constexpr int ESZ = 2;
    static constexpr int KC = 2;
    static constexpr int KSTEPS = 1;  // K = 16 in one instruction
    static constexpr int PIECES = 2;
    static constexpr bool FF = false;
    static constexpr uint32_t FMT = tc::FMT_BF16;
};
template <>
struct TcFmt<2> {
    static constexpr int ESZ = 2;
    static constexpr int KC = 2;
    static constexpr int KSTEPS = 1;
    static constexpr int PIECES = 3;
    static constexpr bool FF = true;
    static constexpr uint32_t FMT = tc::FMT_BF16;
};

template <int MODE>
struct TcLayout {
    static constexpr int IMG_A = kTcRows * kTcNodes * TcFmt<MODE>::ESZ;  // one piece of one part
    static constexpr int IMG_B = kTcNodes * kTcNodes * TcFmt<MODE>::ESZ;
    static constexpr int SBO = TcFmt<MODE>::KC * 128;
    static constexpr int PART_A = TcFmt<MODE>::PIECES * IMG_A;  // A operand of one part: [piece]
    static constexpr int SLOT = 2 * PART_A;                     // A operand of one group: [part][piece]
    static constexpr int PART_B = TcFmt<MODE>::PIECES * IMG_B;  // B operand of one part: [piece]
    static constexpr int GRP_W = 2 * PART_B;                    // swap group: [part][piece]
    static constexpr int GRP_H = PART_B;                        // z group: [piece] (both parts)
};

// Kernel arguments beyond the translation batch: the B images of this
// launch's order bound and op, and the edge factors.
struct TcTables {
    const unsigned char *W;  // [swap group][part][piece] images
    const unsigned char *H;  // [z group][piece] images
    const float *ein, *eout;  // edge factors of this op, n(n+1)/2 + m, n < 16 (float-float pairs
                              // for the float-float-edge formats)
    uint32_t wait_limit;      // mbarrier polls before a wait is declared failed
};

// shared-memory plan of one CTA (byte offsets), for order bound P and
// operand format MODE
struct TcSmem {
    int w, h, a, pw, rp, ein, eout, bar, total;
    template <int MODE>
    __host__ __device__ static TcSmem of(int P)
    {
        using L = TcLayout<MODE>;
        constexpr int ff = TcFmt<MODE>::FF ? 2 : 1;  // hi (and lo) words per value
        TcSmem s;
        int o = 0;
        s.w = o;
        o += tc_deg_groups(P) * L::GRP_W;
        s.h = o;
        o += tc_z_groups(P) * L::GRP_H;
        s.a = o;  // three A slots: a group's operand is written two steps after the
                  // previous occupant's last MMA was issued, which by then has completed
        o += 3 * L::SLOT;
        s.pw = o;  // cos/sin m alpha, cos/sin m beta (hi, then lo): [word][m][thread]
        o += 4 * ff * kTcMaxOrder * kTcRows * 4;
        s.rp = o;  // forward and backward r-power of degree n (hi, then lo): [word][n][thread]
        o += 2 * ff * kTcMaxOrder * kTcRows * 4;
        s.ein = o;
        o += ff * kTcMaxOrder * (kTcMaxOrder + 1) / 2 * 4;
        s.eout = o;
        o += ff * kTcMaxOrder * (kTcMaxOrder + 1) / 2 * 4;
        o = (o + 15) & ~15;
        s.bar = o;
        o += 48;  // four mbarriers + tensor-memory address
        s.total = o;
        return s;
    }
};

namespace tcd {

__device__ __forceinline__ float tf32_rna(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// FP64 x 2^e -> FP32 with integer operations (round half up; results below
// 2^-126, zero and subnormal x -> 0, above the FP32 range -> infinity; the
// FP64 pipe runs at 1/64 of the FP32 rate)
__device__ __forceinline__ float f32_from_d(double x, int e = 0)
{
    const uint32_t hw = (uint32_t)__double2hiint(x), lw = (uint32_t)__double2loint(x);
    const int ed = (int)((hw >> 20) & 0x7ffu);
    const int ef = ed - 1023 + 127 + e;
    uint32_t b = ((uint32_t)ef << 23) + (((hw & 0xfffffu) << 3) | (lw >> 29)) + ((lw >> 28) & 1u);
    if (ef <= 0 || ed == 0) b = 0;
    if (ef >= 255) b = 0x7f800000u;
    return __uint_as_float(b | (hw & 0x80000000u));
}

// D (+)= A * B^T over the split products of one part: A pieces at
// a + i IMG_A, B pieces at b + j IMG_B, products (i, j) with i + j below the
// piece count, the smallest first (they sum almost exactly before the
// largest, hi*hi, is added: the FP32 accumulator then rounds about once).
template <int MODE>
__device__ __forceinline__ void mma_part(uint32_t dt, uint32_t a, uint32_t b)
{
    using L = TcLayout<MODE>;
    constexpr uint32_t ID = tc::idesc(TcFmt<MODE>::FMT, kTcRows, kTcNodes);
    constexpr int NP = TcFmt<MODE>::PIECES == 3 ? 6 : 3;
    constexpr int pi[6] = {2, 1, 0, 1, 0, 0}, pj[6] = {0, 1, 2, 0, 1, 0};  // 3 pieces
    constexpr int qi[3] = {1, 0, 0}, qj[3] = {0, 1, 0};                    // 2 pieces
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const int i = NP == 6 ? pi[p] : qi[p], j = NP == 6 ? pj[p] : qj[p];
#pragma unroll
        for (int c = 0; c < TcFmt<MODE>::KSTEPS; ++c) {
            const uint64_t da = tc::sdesc(a + i * L::IMG_A + c * 256, 128, L::SBO);
            const uint64_t db = tc::sdesc(b + j * L::IMG_B + c * 256, 128, L::SBO);
            if constexpr (MODE == 0) tc::mma_tf32(dt, da, db, ID, (p | c) != 0);
            else tc::mma_f16(dt, da, db, ID, (p | c) != 0);
        }
    }
}

// both parts of one group: A slot at a, B images at b (real part) and
// b + boff (imaginary part), D at dt (real) and dt + 16 (imaginary)
template <int MODE>
__device__ __forceinline__ void mma_group(uint32_t dt, uint32_t a, uint32_t b, uint32_t boff)
{
    mma_part<MODE>(dt, a, b);
    mma_part<MODE>(dt + 16, a + TcLayout<MODE>::PART_A, b + boff);
}

// Tie registers written by tcgen05.ld to the preceding tcgen05.wait::ld:
// empty volatile asm statements stay after the wait (volatile asm is not
// reordered), and every later use depends on them.
__device__ __forceinline__ void reg_fence(uint32_t &r) { asm volatile("" : "+r"(r)); }

// two 16-column rows of this thread's lane (re and im), complete on return
__device__ __forceinline__ void ld_pair_u(uint32_t a, uint32_t b, uint32_t (&x)[16], uint32_t (&y)[16])
{
    tc::tmem_ld16(a, x);
    tc::tmem_ld16(b, y);
    tc::tmem_wait_ld();
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        reg_fence(x[j]);
        reg_fence(y[j]);
    }
}

__device__ __forceinline__ void ld_pair(uint32_t a, uint32_t b, float (&x)[16], float (&y)[16])
{
    uint32_t rx[16], ry[16];
    ld_pair_u(a, b, rx, ry);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        x[j] = __uint_as_float(rx[j]);
        y[j] = __uint_as_float(ry[j]);
    }
}

// lane j of a group: (degree n, order m), and whether it is used
struct TcLane {
    int n, m;
    bool on;
};
__device__ __forceinline__ TcLane deg_lane(const TcGroup &g, int j)
{
    return TcLane{j < g.d1 ? g.n1 : g.n2, j < g.d1 ? j : j - g.d1, j < g.d1 + g.d2};
}

}  // namespace tcd

// Per-CTA pipeline barriers: barrier (kind, slot) tracks the first (kind 0)
// or second (kind 1) MMA of the group held in that slot.  A failed wait (the
// tensor core never completed) marks the thread; the CTA stops at the next
// tile boundary.
struct TcSync {
    uint64_t *bar;   // [kind][slot]
    uint32_t phase;  // bit 2 kind + slot
    uint32_t limit;
    bool failed;

    __device__ __forceinline__ void wait(int kind, int slot)
    {
        const int b = 2 * kind + slot;
        if (!failed && !tc::mbar_wait(bar + b, (phase >> b) & 1u, limit)) failed = true;
        phase ^= 1u << b;
        tc::fence_after_sync();
    }
    // all threads' A rows written and tensor-memory reads complete: barrier,
    // then thread 0 issues (f)
    template <class F>
    __device__ __forceinline__ void step(F f)
    {
        tc::fence_proxy_async();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (threadIdx.x == 0) f();
    }
    __device__ __forceinline__ void commit(int kind, int slot) { tc::commit(bar + 2 * kind + slot); }
};


namespace tcd {

// LPT consecutive tensor-memory columns of this thread's lane
template <int LPT>
__device__ __forceinline__ void ldn(uint32_t taddr, uint32_t (&r)[LPT])
{
    if constexpr (LPT == 4) tc::tmem_ld4(taddr, r);
    else if constexpr (LPT == 8) tc::tmem_ld8(taddr, r);
    else tc::tmem_ld16(taddr, r);
}

template <int LPT>
__device__ __forceinline__ void stn(uint32_t taddr, const uint32_t (&r)[LPT])
{
    if constexpr (LPT == 4) tc::tmem_st4(taddr, r);
    else if constexpr (LPT == 8) tc::tmem_st8(taddr, r);
    else tc::tmem_st16(taddr, r);
}

// re and im columns [c, c + LPT) of this lane, complete on return
template <int LPT>
__device__ __forceinline__ void ld_pair_n(uint32_t a, uint32_t b, float (&x)[LPT], float (&y)[LPT])
{
    uint32_t rx[LPT], ry[LPT];
    ldn<LPT>(a, rx);
    ldn<LPT>(b, ry);
    tc::tmem_wait_ld();
#pragma unroll
    for (int j = 0; j < LPT; ++j) {
        reg_fence(rx[j]);
        reg_fence(ry[j]);
        x[j] = __uint_as_float(rx[j]);
        y[j] = __uint_as_float(ry[j]);
    }
}

// Elements [LPT q, LPT q + LPT) of row t of the split A operand: the
// pieces of v (+ lo, a float-float low word, or none) into the images at
// img + i IMG_A.  Each piece is the input format's rounding of what the
// earlier pieces left; the remainders are exact in FP32, so the pieces sum
// to v + lo up to the last piece's rounding.
template <int MODE, int LPT>
__device__ __forceinline__ void put_part(unsigned char *img, int t, int q, const float (&v)[LPT],
                                         const float *lo = nullptr)
{
    constexpr int IA = TcLayout<MODE>::IMG_A;
    constexpr int NPC = TcFmt<MODE>::PIECES;
    unsigned char *row = img + (t >> 3) * TcFmt<MODE>::KC * 128 + (t & 7) * 16;
    if constexpr (MODE == 0) {  // 4 TF32 elements per core-matrix row
#pragma unroll
        for (int c = 0; c < LPT / 4; ++c) {
            float h[4], l[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                h[e] = tf32_rna(v[4 * c + e]);
                l[e] = tf32_rna(v[4 * c + e] - h[e]);
            }
            unsigned char *d = row + ((LPT * q) / 4 + c) * 128;
            *reinterpret_cast<float4 *>(d) = make_float4(h[0], h[1], h[2], h[3]);
            *reinterpret_cast<float4 *>(d + IA) = make_float4(l[0], l[1], l[2], l[3]);
        }
    } else {  // 8 BF16 elements per core-matrix row
        uint32_t pc[NPC][LPT / 2];
#pragma unroll
        for (int e = 0; e < LPT / 2; ++e) {
            float a = v[2 * e], b = v[2 * e + 1];
            const float la = lo ? lo[2 * e] : 0.f, lb = lo ? lo[2 * e + 1] : 0.f;
#pragma unroll
            for (int k = 0; k < NPC; ++k) {
                const __nv_bfloat162 hb = __floats2bfloat162_rn(a, b);
                pc[k][e] = *reinterpret_cast<const uint32_t *>(&hb);
                a -= __low2float(hb);  // exact
                b -= __high2float(hb);
                if (k == 0 && lo) {  // the low word joins the remainder (rounding ~2^-24 of it)
                    a += la;
                    b += lb;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < NPC; ++k) {
            if constexpr (LPT == 4) {
                *reinterpret_cast<uint2 *>(row + (q >> 1) * 128 + (q & 1) * 8 + k * IA) = make_uint2(pc[k][0], pc[k][1]);
            } else {
#pragma unroll
                for (int c = 0; c < LPT / 8; ++c)
                    *reinterpret_cast<uint4 *>(row + ((LPT * q) / 8 + c) * 128 + k * IA) =
                        make_uint4(pc[k][4 * c], pc[k][4 * c + 1], pc[k][4 * c + 2], pc[k][4 * c + 3]);
            }
        }
    }
}

__device__ __forceinline__ void prefetch_l2(const void *ptr) { asm volatile("prefetch.global.L2 [%0];" ::"l"(ptr)); }

// complex float-float product
__device__ __forceinline__ void cmul_ff(ff &c, ff &s, ff bc, ff bs)
{
    using A = arith<ff>;
    const ff nc = A::dot2(c, bc, A::neg(s), bs), ns = A::dot2(s, bc, c, bs);
    c = nc;
    s = ns;
}

}  // namespace tcd

// NWG warpgroups share a tile: thread (q, t) = (warpgroup, row) handles
// lanes [LPT q, LPT q + LPT) of every group of translation t, LPT = 16/NWG;
// the warps of every warpgroup reach tensor-memory lanes 0..127.
template <int MODE, int NWG>
__global__ void __launch_bounds__(kTcRows *NWG, 1) k_translate_tc(KParams p, TcTables tt)
{
    using L = TcLayout<MODE>;
    using A = arith<ff>;
    constexpr int LPT = kTcNodes / NWG;
    constexpr bool FF = TcFmt<MODE>::FF;
    constexpr int kNE = kTcMaxOrder * (kTcMaxOrder + 1) / 2;  // stride of the edge tables' low words
    extern __shared__ __align__(1024) unsigned char smem[];
    const int P = p.P;
    const TcSmem sm = TcSmem::of<MODE>(P);
    const int tid = threadIdx.x;
    const int t = tid & (kTcRows - 1);  // translation of the tile, tensor-memory lane
    const int q = tid >> 7;             // lanes [LPT q, LPT q + LPT) of every group
    const int warp = tid >> 5;
    const int j0 = LPT * q;
    const int NG = tc_deg_groups(P), NZ = tc_z_groups(P);
    unsigned char *sA = smem + sm.a;
    float *pw = reinterpret_cast<float *>(smem + sm.pw) + t;   // [q][m][row], this row's column
    float *rpw = reinterpret_cast<float *>(smem + sm.rp) + t;  // [dir][n][row]
    float *sEin = reinterpret_cast<float *>(smem + sm.ein);
    float *sEout = reinterpret_cast<float *>(smem + sm.eout);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + sm.bar);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + sm.bar + 32);
    __shared__ int red[2];
#define PW(k, m) pw[((k) * kTcMaxOrder + (m)) * kTcRows]
#define RPW(dir, n) rpw[((dir) * kTcMaxOrder + (n)) * kTcRows]

    // constant operands (this order bound's groups) and edge factors, once per CTA
    {
        const int nw = NG * L::GRP_W / 16, nh = NZ * L::GRP_H / 16;
        const uint4 *gw = reinterpret_cast<const uint4 *>(tt.W);
        const uint4 *gh = reinterpret_cast<const uint4 *>(tt.H);
        for (int i = tid; i < nw; i += kTcRows * NWG) reinterpret_cast<uint4 *>(smem + sm.w)[i] = gw[i];
        for (int i = tid; i < nh; i += kTcRows * NWG) reinterpret_cast<uint4 *>(smem + sm.h)[i] = gh[i];
        for (int i = tid; i < P * (P + 1) / 2; i += kTcRows * NWG) {
            sEin[i] = tt.ein[i];
            sEout[i] = tt.eout[i];
            if constexpr (FF) {  // low words at a fixed stride
                sEin[kNE + i] = tt.ein[kNE + i];
                sEout[kNE + i] = tt.eout[kNE + i];
            }
        }
    }
    if (tid == 0) {
        for (int b = 0; b < 4; ++b) tc::mbar_init(bars + b, 1);
        tc::fence_mbar_init();
    }
    if (warp == 0) tc::tmem_alloc(tslot, kTcCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = *tslot;
    const uint32_t lb = tbase + ((uint32_t)((warp & 3) * 32) << 16);  // this warp's lanes
    const uint32_t a0 = tc::smem_u32(sA), w0 = tc::smem_u32(smem + sm.w), h0 = tc::smem_u32(smem + sm.h);
    TcSync sy{bars, 0u, tt.wait_limit, false};
    const double *src = reinterpret_cast<const double *>(p.src);
    double *dst = reinterpret_cast<double *>(p.dst);
    const int op = p.op;
    bool range_ok = true;

    for (long long tile = blockIdx.x; tile * kTcRows < p.n; tile += gridDim.x) {
        // ---- per-translation setup (validation as in k_translate) ----
        const long long i = tile * kTcRows + t;
        bool valid = i < p.n;
        uint32_t tr = 0, si = 0, ti = 0;
        if (valid) tr = p.perm ? p.perm[i] : (uint32_t)i;
        int pin = 0, pout = 0;
        if (valid && tr < p.nidx) {
            si = p.sidx ? p.sidx[tr] : tr;
            ti = p.tidx ? p.tidx[tr] : tr;
            pin = (int)p.pin[tr];
            pout = (int)p.pout[tr];
        }
        if (valid && (tr >= p.nidx || si >= p.nsrc || ti >= p.ndst || pin > P || pout > P || pin < 0 || pout < 0)) {
            if (q == 0) atomicOr(p.status, 1);
            valid = false;
        }
        if (!valid) pin = pout = 0;
        double x = 0, y = 0, z = 1;
        if (valid) {
            x = p.shift[3 * (long long)tr];
            y = p.shift[3 * (long long)tr + 1];
            z = p.shift[3 * (long long)tr + 2];
        }
        if (op == OP_M2M) {  // M2M translates by the negated shift (translations.cpp:331-333)
            x = -x;
            y = -y;
            z = -z;
        }
        int ident_p = 0;
        if (valid && op != OP_M2L && (x * x + y * y + z * z) == 0.0) {  // translations.cpp:540-547
            ident_p = min(pin, pout);
            pin = pout = 0;
            x = y = 0;
            z = 1;
        }
        if (op == OP_L2L) pout = min(pin, pout);  // translations.cpp:412
        // the translation's length scale lambda = 2^ks, |shift| / lambda in
        // [2, 7): sources times lambda^-n (multipoles) or lambda^(n+1)
        // (locals), results back, all exact in the conversions, so that the
        // edge factors r^n and r^-(n+1) stay in range at any geometry scale
        int ks = 0;
        {
            const int e3 = max(exp_of(x), max(exp_of(y), exp_of(z)));  // |shift| in [2^e3, sqrt(3) 2^(e3+1))
            if (valid && !ident_p && e3 > -(1 << 19)) {
                ks = e3 - 1;
                x = d_scaled(x, -ks);
                y = d_scaled(y, -ks);
                z = d_scaled(z, -ks);
            }
        }
        const int es = op == OP_L2L ? ks : -ks, es0 = op == OP_L2L ? ks : 0;   // source degree n: es n + es0
        const int eo = op == OP_M2M ? ks : -ks, eo0 = op == OP_M2M ? 0 : -ks;  // output degree j: eo j + eo0
        // pointer mode: per-translation addresses (host solids the GPU reads in place)
        const double *sp = p.src_ptr ? reinterpret_cast<const double *>(p.src_ptr[si]) : src + (long long)si * p.sstride;
        double *dp = p.dst_ptr ? reinterpret_cast<double *>(p.dst_ptr[ti]) : dst + (long long)ti * p.dstride;

        // geometry (euler, microkernel_generic.cpp:37-97) and its powers in
        // float-float (FP32 and integer pipes; the FP64 pipe runs at 1/64 of
        // the FP32 rate), this thread's orders m in [j0, j0 + LPT), stored as FP32
        {
            const ff fx = ff_from_d_int(x), fy = ff_from_d_int(y), fz = ff_from_d_int(z);
            const ff rxy2 = A::dot2(fx, fx, fy, fy);
            const ff rxy = ff_sqrt(rxy2);
            const ff rr = ff_sqrt(A::add(rxy2, A::mul(fz, fz)));
            const ff ri = ff_rcp(rr), one{1.f, 0.f}, zero{0.f, 0.f};
            ff e1c = one, e1s = zero;
            if (rxy.hi > 0.f) {
                const ff rq = ff_rcp(rxy);
                e1c = A::mul(fy, rq);
                e1s = A::mul(fx, rq);
            }
            const ff b1c = A::mul(fz, ri), b1s = A::neg(A::mul(rxy, ri));
            ff eac = e1c, eas = e1s, ebc = b1c, ebs = b1s;
            // forward scale r^n (local input) or r^-(n+1) (multipole input);
            // backward r^(n+1) (multipole output) or r^-n (local output)
            ff f = op == OP_L2L ? one : ri, g = op == OP_M2M ? rr : one;
            ff fs = op == OP_L2L ? rr : ri, gs = op == OP_M2M ? rr : ri;
            // powers j0: binary exponentiation
            ff ac = one, as = zero, bc = one, bs = zero;
            for (int k = j0; k; k >>= 1) {
                if (k & 1) {
                    tcd::cmul_ff(ac, as, eac, eas);
                    tcd::cmul_ff(bc, bs, ebc, ebs);
                    f = A::mul(f, fs);
                    g = A::mul(g, gs);
                }
                tcd::cmul_ff(eac, eas, eac, eas);
                tcd::cmul_ff(ebc, ebs, ebc, ebs);
                fs = A::mul(fs, fs);
                gs = A::mul(gs, gs);
            }
            // eac.. and fs.. now hold e^{i 2^k alpha} etc.; the single steps
            const ff f1 = op == OP_L2L ? rr : ri, g1 = op == OP_M2M ? rr : ri;
#pragma unroll
            for (int jj = 0; jj < LPT; ++jj) {
                const int m = j0 + jj;
                if (m < P) {
                    PW(0, m) = ac.hi;
                    PW(1, m) = as.hi;
                    PW(2, m) = bc.hi;
                    PW(3, m) = bs.hi;
                    RPW(0, m) = f.hi;
                    RPW(1, m) = g.hi;
                    if constexpr (FF) {
                        PW(4, m) = ac.lo;
                        PW(5, m) = as.lo;
                        RPW(2, m) = f.lo;
                        RPW(3, m) = g.lo;
                    }
                    if (m < max(pin, pout) && !(isfinite(f.hi) && isfinite(g.hi) && f.hi != 0.f && g.hi != 0.f))
                        range_ok = false;
                }
                tcd::cmul_ff(ac, as, e1c, e1s);
                tcd::cmul_ff(bc, bs, b1c, b1s);
                f = A::mul(f, f1);
                g = A::mul(g, g1);
            }
        }
        // L2 prefetch: this tile's targets (read in the backward stage) and the
        // next tile's sources (read at its start), spread over the warpgroups;
        // device arrays only, every address inside an expansion the entry may touch
        if (p.in_hbm && !p.src_ptr) {
            const int tcnt = max(pout * (pout + 1), ident_p * (ident_p + 1));
            for (int o = q * 128; o < tcnt * 8; o += NWG * 128) tcd::prefetch_l2(reinterpret_cast<const char *>(dp) + o);
            const long long i2 = (tile + gridDim.x) * kTcRows + t;
            if (i2 < p.n) {
                const uint32_t t2 = p.perm ? p.perm[i2] : (uint32_t)i2;
                if (t2 < p.nidx) {
                    const uint32_t s2 = p.sidx ? p.sidx[t2] : t2;
                    const int pin2 = (int)p.pin[t2];
                    if (s2 < p.nsrc && pin2 > 0 && pin2 <= P) {
                        const char *sp2 = reinterpret_cast<const char *>(src + (long long)s2 * p.sstride);
                        for (int o = q * 128; o < pin2 * (pin2 + 1) * 8; o += NWG * 128) tcd::prefetch_l2(sp2 + o);
                    }
                }
            }
        }
        if (tid == 0) red[0] = 0;
        __syncthreads();
        if (q == 0) atomicMax(&red[0], pin);
        __syncthreads();
        const int pin_w = red[0];

        // ---- forward transforms (pipelined over swap groups) ----
        double xr_n[LPT], xi_n[LPT];  // sources of the next group, in flight
        auto fetch = [&](int gi) {
            const TcGroup gr = tc_deg_group(P, gi);
#pragma unroll
            for (int jj = 0; jj < LPT; ++jj) {
                const tcd::TcLane ln = tcd::deg_lane(gr, j0 + jj);
                xr_n[jj] = xi_n[jj] = 0.0;
                if (ln.on && ln.n < pin) {
                    xr_n[jj] = sp[ln.n * (ln.n + 1) + ln.m];
                    xi_n[jj] = sp[(ln.n + 1) * (ln.n + 1) + ln.m];
                }
            }
        };
        fetch(0);
        for (int s = 0; s <= NG + 1; ++s) {
            const int sl = s & 1;
            if (s < NG) {  // group s: edge (r-power, e^{+i m alpha}, basis) -> A
                const TcGroup gr = tc_deg_group(P, s);
                float vr[LPT], vi[LPT], vr_lo[LPT], vi_lo[LPT];
#pragma unroll
                for (int jj = 0; jj < LPT; ++jj) {
                    const tcd::TcLane ln = tcd::deg_lane(gr, j0 + jj);
                    vr[jj] = vi[jj] = vr_lo[jj] = vi_lo[jj] = 0.f;
                    if (ln.on) {
                        const int e = ln.n * (ln.n + 1) / 2 + ln.m;
                        if constexpr (FF) {  // float-float edge, split without rounding to FP32
                            const int esh = es * ln.n + es0;
                            const ff xr = ff_from_d_scaled0(xr_n[jj], esh), xi = ff_from_d_scaled0(xi_n[jj], esh);
                            const ff gg = A::mul(ff{RPW(0, ln.n), RPW(2, ln.n)}, ff{sEin[e], sEin[kNE + e]});
                            const ff gc = A::mul(gg, ff{PW(0, ln.m), PW(4, ln.m)});
                            const ff gs = A::mul(gg, ff{PW(1, ln.m), PW(5, ln.m)});
                            const ff yr = A::dot2(gc, xr, A::neg(gs), xi), yi = A::dot2(gs, xr, gc, xi);
                            vr[jj] = yr.hi;
                            vr_lo[jj] = yr.lo;
                            vi[jj] = yi.hi;
                            vi_lo[jj] = yi.lo;
                        } else {
                            const int esh = es * ln.n + es0;
                            const float xr = tcd::f32_from_d(xr_n[jj], esh), xi = tcd::f32_from_d(xi_n[jj], esh);
                            const float gg = RPW(0, ln.n) * sEin[e];
                            const float gc = gg * PW(0, ln.m), gs = gg * PW(1, ln.m);
                            vr[jj] = gc * xr - gs * xi;
                            vi[jj] = gs * xr + gc * xi;
                        }
                    }
                }
                if (s + 1 < NG) fetch(s + 1);
                unsigned char *slot = sA + (s % 3) * L::SLOT;
                tcd::put_part<MODE, LPT>(slot, t, q, vr, FF ? vr_lo : nullptr);
                tcd::put_part<MODE, LPT>(slot + L::PART_A, t, q, vi, FF ? vi_lo : nullptr);
            }
            if (s >= 2) {  // group s-2: second swap -> state
                sy.wait(1, sl);
                float ur[LPT], ui[LPT];
                tcd::ld_pair_n<LPT>(lb + kTcD + 32 * sl + j0, lb + kTcD + 32 * sl + 16 + j0, ur, ui);
                const TcGroup gr = tc_deg_group(P, s - 2);
#pragma unroll
                for (int jj = 0; jj < LPT; ++jj) {
                    const tcd::TcLane ln = tcd::deg_lane(gr, j0 + jj);
                    if (ln.on) {
                        const uint32_t col = (uint32_t)tc_state_col(P, ln.n, ln.m);
                        tc::tmem_st1(lb + kTcStateRe + col, __float_as_uint(ur[jj]));
                        tc::tmem_st1(lb + kTcStateIm + col, __float_as_uint(ui[jj]));
                    }
                }
            }
            if (s >= 1 && s <= NG) {  // group s-1: first swap -> e^{+i m beta} -> A
                sy.wait(0, sl ^ 1);
                float vr[LPT], vi[LPT];
                tcd::ld_pair_n<LPT>(lb + kTcD + 32 * (sl ^ 1) + j0, lb + kTcD + 32 * (sl ^ 1) + 16 + j0, vr, vi);
                const TcGroup gr = tc_deg_group(P, s - 1);
#pragma unroll
                for (int jj = 0; jj < LPT; ++jj) {
                    const tcd::TcLane ln = tcd::deg_lane(gr, j0 + jj);
                    const float c = ln.on ? PW(2, ln.m) : 0.f, sn = ln.on ? PW(3, ln.m) : 0.f;
                    const float a = vr[jj], b = vi[jj];
                    vr[jj] = c * a - sn * b;
                    vi[jj] = sn * a + c * b;
                }
                unsigned char *slot = sA + ((s + 2) % 3) * L::SLOT;
                tcd::put_part<MODE, LPT>(slot, t, q, vr);
                tcd::put_part<MODE, LPT>(slot + L::PART_A, t, q, vi);
            }
            sy.step([&] {
                if (s >= 1 && s <= NG) {
                    tcd::mma_group<MODE>(tbase + kTcD + 32 * (sl ^ 1), a0 + ((s + 2) % 3) * L::SLOT,
                                         w0 + (s - 1) * L::GRP_W, L::PART_B);
                    sy.commit(1, sl ^ 1);
                }
                if (s < NG) {
                    tcd::mma_group<MODE>(tbase + kTcD + 32 * sl, a0 + (s % 3) * L::SLOT, w0 + s * L::GRP_W, L::PART_B);
                    sy.commit(0, sl);
                }
            });
        }
        tc::tmem_wait_st();

        // ---- z-translation (pipelined over z groups, in place) ----
        for (int s = 0; s <= NZ; ++s) {
            const int sl = s & 1;
            if (s < NZ) {  // group s: state -> A (rows at or above the tile's input order are zero)
                const TcGroup gr = tc_z_group(P, s);
                float vr[LPT], vi[LPT];
                tcd::ld_pair_n<LPT>(lb + kTcStateRe + s * P + j0, lb + kTcStateIm + s * P + j0, vr, vi);
#pragma unroll
                for (int jj = 0; jj < LPT; ++jj) {
                    const int j = j0 + jj;
                    const int k = j < gr.d1 ? gr.n1 + j : gr.n2 + j - gr.d1;
                    if (j >= gr.d1 + gr.d2 || k >= pin_w) vr[jj] = vi[jj] = 0.f;
                }
                unsigned char *slot = sA + (s % 3) * L::SLOT;
                tcd::put_part<MODE, LPT>(slot, t, q, vr);
                tcd::put_part<MODE, LPT>(slot + L::PART_A, t, q, vi);
            }
            if (s >= 1) {  // group s-1: output -> state
                sy.wait(0, sl ^ 1);
                uint32_t ur[LPT], ui[LPT];
                tcd::ldn<LPT>(lb + kTcD + 32 * (sl ^ 1) + j0, ur);
                tcd::ldn<LPT>(lb + kTcD + 32 * (sl ^ 1) + 16 + j0, ui);
                tc::tmem_wait_ld();
#pragma unroll
                for (int jj = 0; jj < LPT; ++jj) {
                    tcd::reg_fence(ur[jj]);
                    tcd::reg_fence(ui[jj]);
                }
                const TcGroup gr = tc_z_group(P, s - 1);
                const int w = gr.d1 + gr.d2;
                const uint32_t col = (uint32_t)((s - 1) * P + j0);
                if (j0 + LPT <= w) {
                    tcd::stn<LPT>(lb + kTcStateRe + col, ur);
                    tcd::stn<LPT>(lb + kTcStateIm + col, ui);
                } else {
#pragma unroll
                    for (int jj = 0; jj < LPT; ++jj)
                        if (j0 + jj < w) {
                            tc::tmem_st1(lb + kTcStateRe + col + jj, ur[jj]);
                            tc::tmem_st1(lb + kTcStateIm + col + jj, ui[jj]);
                        }
                }
            }
            sy.step([&] {
                if (s < NZ) {
                    tcd::mma_group<MODE>(tbase + kTcD + 32 * sl, a0 + (s % 3) * L::SLOT, h0 + s * L::GRP_H, 0);
                    sy.commit(0, sl);
                }
            });
        }
        tc::tmem_wait_st();

        // ---- backward transforms and accumulation (pipelined over swap groups) ----
        double tr_n[LPT], ti_n[LPT];  // targets of the group in the middle stage, in flight
        for (int s = 0; s <= NG + 1; ++s) {
            const int sl = s & 1;
            if (s < NG) {  // group s: state -> A
                const TcGroup gr = tc_deg_group(P, s);
                uint32_t ur[LPT], ui[LPT];
#pragma unroll
                for (int jj = 0; jj < LPT; ++jj) {
                    const tcd::TcLane ln = tcd::deg_lane(gr, j0 + jj);
                    ur[jj] = ui[jj] = 0u;
                    if (ln.on) {
                        const uint32_t col = (uint32_t)tc_state_col(P, ln.n, ln.m);
                        ur[jj] = tc::tmem_ld1(lb + kTcStateRe + col);
                        ui[jj] = tc::tmem_ld1(lb + kTcStateIm + col);
                    }
                }
                tc::tmem_wait_ld();
                float vr[LPT], vi[LPT];
#pragma unroll
                for (int jj = 0; jj < LPT; ++jj) {
                    tcd::reg_fence(ur[jj]);
                    tcd::reg_fence(ui[jj]);
                    const bool on = j0 + jj < gr.d1 + gr.d2;
                    vr[jj] = on ? __uint_as_float(ur[jj]) : 0.f;
                    vi[jj] = on ? __uint_as_float(ui[jj]) : 0.f;
                }
                unsigned char *slot = sA + (s % 3) * L::SLOT;
                tcd::put_part<MODE, LPT>(slot, t, q, vr);
                tcd::put_part<MODE, LPT>(slot + L::PART_A, t, q, vi);
            }
            if (s >= 2) {  // group s-2: second swap -> e^{-i m alpha}, basis, r-power -> target +=
                sy.wait(1, sl);
                float ur[LPT], ui[LPT];
                tcd::ld_pair_n<LPT>(lb + kTcD + 32 * sl + j0, lb + kTcD + 32 * sl + 16 + j0, ur, ui);
                const TcGroup gr = tc_deg_group(P, s - 2);
#pragma unroll
                for (int jj = 0; jj < LPT; ++jj) {
                    const tcd::TcLane ln = tcd::deg_lane(gr, j0 + jj);
                    if (ln.on && ln.n < pout) {
                        const int e = ln.n * (ln.n + 1) / 2 + ln.m;
                        double orr, oi;
                        if constexpr (FF) {  // float-float edge
                            const ff gg = A::mul(ff{RPW(1, ln.n), RPW(3, ln.n)}, ff{sEout[e], sEout[kNE + e]});
                            const ff gc = A::mul(gg, ff{PW(0, ln.m), PW(4, ln.m)});
                            const ff gs = A::mul(gg, ff{PW(1, ln.m), PW(5, ln.m)});
                            const ff xr{ur[jj], 0.f}, xi{ui[jj], 0.f};
                            const ff yr = A::dot2(gc, xr, gs, xi), yi = A::dot2(gc, xi, A::neg(gs), xr);
                            const int esh = eo * ln.n + eo0;
                            orr = d_from_f_scaled(yr.hi, esh) + d_from_f_scaled(yr.lo, esh);
                            oi = d_from_f_scaled(yi.hi, esh) + d_from_f_scaled(yi.lo, esh);
                        } else {
                            const float gg = RPW(1, ln.n) * sEout[e];
                            const float gc = gg * PW(0, ln.m), gs = gg * PW(1, ln.m);
                            const int esh = eo * ln.n + eo0;
                            orr = d_from_f_scaled(gc * ur[jj] + gs * ui[jj], esh);
                            oi = d_from_f_scaled(gc * ui[jj] - gs * ur[jj], esh);
                        }
                        double *pr = dp + ln.n * (ln.n + 1) + ln.m, *pi = dp + (ln.n + 1) * (ln.n + 1) + ln.m;
                        if (p.atomic) {
                            atomicAdd(pr, orr);
                            atomicAdd(pi, oi);
                        } else {
                            *pr = tr_n[jj] + orr;
                            *pi = ti_n[jj] + oi;
                        }
                    }
                }
            }
            if (s >= 1 && s <= NG) {  // group s-1: first swap -> e^{-i m beta} -> A; fetch its targets
                sy.wait(0, sl ^ 1);
                float vr[LPT], vi[LPT];
                tcd::ld_pair_n<LPT>(lb + kTcD + 32 * (sl ^ 1) + j0, lb + kTcD + 32 * (sl ^ 1) + 16 + j0, vr, vi);
                const TcGroup gr = tc_deg_group(P, s - 1);
#pragma unroll
                for (int jj = 0; jj < LPT; ++jj) {
                    const tcd::TcLane ln = tcd::deg_lane(gr, j0 + jj);
                    const float c = ln.on ? PW(2, ln.m) : 0.f, sn = ln.on ? PW(3, ln.m) : 0.f;
                    const float a = vr[jj], b = vi[jj];
                    vr[jj] = c * a + sn * b;
                    vi[jj] = c * b - sn * a;
                    tr_n[jj] = ti_n[jj] = 0.0;
                    if (!p.atomic && ln.on && ln.n < pout) {
                        tr_n[jj] = dp[ln.n * (ln.n + 1) + ln.m];
                        ti_n[jj] = dp[(ln.n + 1) * (ln.n + 1) + ln.m];
                    }
                }
                unsigned char *slot = sA + ((s + 2) % 3) * L::SLOT;
                tcd::put_part<MODE, LPT>(slot, t, q, vr);
                tcd::put_part<MODE, LPT>(slot + L::PART_A, t, q, vi);
            }
            sy.step([&] {
                if (s >= 1 && s <= NG) {
                    tcd::mma_group<MODE>(tbase + kTcD + 32 * (sl ^ 1), a0 + ((s + 2) % 3) * L::SLOT,
                                         w0 + (s - 1) * L::GRP_W, L::PART_B);
                    sy.commit(1, sl ^ 1);
                }
                if (s < NG) {
                    tcd::mma_group<MODE>(tbase + kTcD + 32 * sl, a0 + (s % 3) * L::SLOT, w0 + s * L::GRP_W, L::PART_B);
                    sy.commit(0, sl);
                }
            });
        }
        // zero shift (M2M, L2L): direct prefix add (translations.cpp:540-547)
        for (int c = q; c < ident_p * (ident_p + 1); c += NWG) {
            if (p.atomic) atomicAdd(dp + c, sp[c]);
            else dp[c] += sp[c];
        }
        if (__syncthreads_or(sy.failed)) break;
    }
    const int any_failed = __syncthreads_or(sy.failed);
    if (tid == 0 && any_failed) atomicOr(p.status, 2);  // a tensor-core wait ran out
    if (!range_ok) atomicOr(p.status, 4);                // an r-power left the FP32 range
#undef PW
#undef RPW
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tbase, kTcCols);
}

}  // namespace sfmm
