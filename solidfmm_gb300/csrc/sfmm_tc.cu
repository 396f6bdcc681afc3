// Tensor-core translation path: operand images of the constant matrices
// (built on the host in FP64, split into two pieces in the MMA's input
// format, laid out as the kernel's shared-memory B operands), their upload,
// and the launch of k_translate_tc.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "sfmm_launch.hpp"
#include "sfmm_tables.hpp"
#include "sfmm_tc_kernel.cuh"

namespace sfmm {

namespace {

// round to TF32 (10 explicit mantissa bits), to nearest with ties away from
// zero, as cvt.rna.tf32.f32 does on the device
float tf32_rna_host(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7f800000u) != 0x7f800000u) {
        u += 0x1000u;
        u &= 0xffffe000u;
    }
    std::memcpy(&f, &u, 4);
    return f;
}

// round to BF16, to nearest even (finite inputs)
uint16_t bf16_rn_host(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

float bf16_float(uint16_t h)
{
    const uint32_t u = (uint32_t)h << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

int pieces_of(int mode) { return mode == 2 ? 3 : 2; }

// Entry (r, k) of a 16 x 16 B operand (K-major core matrices) in format
// `mode`: piece i at img + i * image size, each piece the rounding of what the
// earlier ones left of v (computed in FP64).
void put_b(unsigned char *img, int mode, int r, int k, double v)
{
    const int esz = mode == 0 ? 4 : 2, KC = 16 * esz / 16, ib = 16 * 16 * esz;
    const size_t off = (size_t)((r / 8) * KC + (k * esz) / 16) * 128 + (r % 8) * 16 + (k * esz) % 16;
    double rem = v;
    for (int i = 0; i < pieces_of(mode); ++i) {
        if (mode == 0) {
            const float pc = tf32_rna_host((float)rem);
            std::memcpy(img + i * ib + off, &pc, 4);
            rem -= (double)pc;
        } else {
            const uint16_t pc = bf16_rn_host((float)rem);
            std::memcpy(img + i * ib + off, &pc, 2);
            rem -= (double)bf16_float(pc);
        }
    }
}

template <class T>
cudaError_t upload_vec(void **dst, const std::vector<T> &v)
{
    const size_t bytes = v.size() * sizeof(T);
    cudaError_t e = cudaMalloc(dst, bytes ? bytes : 16);
    if (e == cudaSuccess && bytes) e = cudaMemcpy(*dst, v.data(), bytes, cudaMemcpyHostToDevice);
    return e;
}

// warpgroups per CTA (each thread handles 16 / kTcGroups lanes of a group)
constexpr int kTcGroups = 4;

template <int MODE>
int smem_bytes(int P)
{
    const TcSmem sm = TcSmem::of<MODE>(P);
    // at least 116 KB: two CTAs never share an SM (each allocates all of
    // its tensor memory)
    return sm.total < 116 * 1024 ? 116 * 1024 : sm.total;
}

}  // namespace

struct TcDevTables {
    int mode = 0;
    int Pt = 0;
    void *W = nullptr;
    void *H[3] = {nullptr, nullptr, nullptr};
    void *e[4] = {nullptr, nullptr, nullptr, nullptr};  // e_in_M, e_in_L, e_out_L, e_out_M (FP32)
    size_t offW[kTcMaxOrder + 1] = {}, offH[kTcMaxOrder + 1] = {};  // images of order bound P
};

void tc_release(TcDevTables *t)
{
    if (!t) return;
    if (t->W) cudaFree(t->W);
    for (void *p : t->H)
        if (p) cudaFree(p);
    for (void *p : t->e)
        if (p) cudaFree(p);
    delete t;
}

int tc_max_order() { return kTcMaxOrder; }

// Images for every order bound P <= min(context order, 16): the swap groups
// of P (block-diagonal pairs of W_R and of W_I) and its z groups (pairs of
// H_m) for each op, split into two pieces in the MMA's input format.
cudaError_t tc_prepare(TcDevTables **out, int mode, const HostTables &host)
{
    *out = nullptr;
    auto *t = new (std::nothrow) TcDevTables;
    if (!t) return cudaErrorMemoryAllocation;
    t->mode = mode;
    t->Pt = host.P < kTcMaxOrder ? host.P : kTcMaxOrder;
    const int Pt = t->Pt;
    const int ib = mode == 0 ? TcLayout<0>::IMG_B : TcLayout<1>::IMG_B;
    const int np = pieces_of(mode);  // group image: [part][piece] (swaps), [piece] (z)
    std::vector<unsigned char> W, H[3];
    for (int P = 1; P <= Pt; ++P) {
        t->offW[P] = W.size();
        t->offH[P] = H[0].size();
        const int NG = tc_deg_groups(P), NZ = tc_z_groups(P);
        W.resize(W.size() + (size_t)NG * 2 * np * ib, 0);
        for (int g = 0; g < NG; ++g) {
            const TcGroup gr = tc_deg_group(P, g);
            for (int part = 0; part < 2; ++part) {
                unsigned char *img = &W[t->offW[P] + ((size_t)g * 2 + part) * np * ib];
                for (int blk = 0; blk < 2; ++blk) {
                    const int n = blk ? gr.n2 : gr.n1, d = blk ? gr.d2 : gr.d1, o = blk ? gr.d1 : 0;
                    for (int i = 0; i < d; ++i)
                        for (int j = 0; j < d; ++j) put_b(img, mode, o + i, o + j, w_entry(host, n, part, i, j));
                }
            }
        }
        for (int op = 0; op < 3; ++op) {
            H[op].resize(H[op].size() + (size_t)NZ * np * ib, 0);
            for (int g = 0; g < NZ; ++g) {
                const TcGroup gr = tc_z_group(P, g);
                unsigned char *img = &H[op][t->offH[P] + (size_t)g * np * ib];
                for (int blk = 0; blk < 2; ++blk) {
                    const int m = blk ? gr.n2 : gr.n1, L = blk ? gr.d2 : gr.d1, o = blk ? gr.d1 : 0;
                    if (!L) continue;
                    const int HR = hrows(host.P - m, host.pad);
                    // B row = output n' - m, column = input k - m
                    for (int a = 0; a < L; ++a)
                        for (int k = 0; k < L; ++k)
                            put_b(img, mode, o + a, o + k, host.H[op][host.hoff[m] + (size_t)k * HR + a]);
                }
            }
        }
    }
    const size_t ne = (size_t)Pt * (Pt + 1) / 2;
    const std::vector<double> *ev[4] = {&host.e_in_M, &host.e_in_L, &host.e_out_L, &host.e_out_M};
    cudaError_t e = upload_vec(&t->W, W);
    for (int op = 0; op < 3 && e == cudaSuccess; ++op) e = upload_vec(&t->H[op], H[op]);
    // edge factors in FP32; the float-float-edge format keeps the low words
    // after a fixed stride of 136 (order 16)
    const size_t kNE = (size_t)kTcMaxOrder * (kTcMaxOrder + 1) / 2;
    for (int k = 0; k < 4 && e == cudaSuccess; ++k) {
        std::vector<float> f(mode == 2 ? 2 * kNE : ne, 0.f);
        for (size_t i = 0; i < ne; ++i) {
            f[i] = (float)(*ev[k])[i];
            if (mode == 2) f[kNE + i] = (float)((*ev[k])[i] - (double)f[i]);
        }
        e = upload_vec(&t->e[k], f);
    }
    if (e == cudaSuccess) {
        const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
        if (mode == 0) e = cudaFuncSetAttribute(k_translate_tc<0, kTcGroups>, at, smem_bytes<0>(Pt));
        else if (mode == 1) e = cudaFuncSetAttribute(k_translate_tc<1, kTcGroups>, at, smem_bytes<1>(Pt));
        else e = cudaFuncSetAttribute(k_translate_tc<2, kTcGroups>, at, smem_bytes<2>(Pt));
    }
    if (e != cudaSuccess) {
        tc_release(t);
        return e;
    }
    *out = t;
    return cudaSuccess;
}

// One persistent CTA per SM (at most one per tile).  The kernel's waits on
// the tensor core give up after ~2^22 polls (seconds), flag bit 1 of the
// status word and return; bit 2 marks translations whose r-powers left the
// FP32 range.
cudaError_t launch_translate_tc(const KParams &p, const TcDevTables *t, int num_sms, cudaStream_t st)
{
    if (p.P < 1 || p.P > t->Pt) return cudaErrorInvalidValue;
    TcTables tt;
    tt.W = static_cast<const unsigned char *>(t->W) + t->offW[p.P];
    tt.H = static_cast<const unsigned char *>(t->H[p.op]) + t->offH[p.P];
    tt.ein = static_cast<const float *>(t->e[p.op == OP_L2L ? 1 : 0]);
    tt.eout = static_cast<const float *>(t->e[p.op == OP_M2M ? 3 : 2]);
    tt.wait_limit = 1u << 22;
    const long long tiles = (p.n + kTcRows - 1) / kTcRows;
    const int grid = (int)(tiles < num_sms ? tiles : num_sms);
    const int nt = kTcRows * kTcGroups;
    clear_stale_error();
    if (t->mode == 0) k_translate_tc<0, kTcGroups><<<grid, nt, smem_bytes<0>(p.P), st>>>(p, tt);
    else if (t->mode == 1) k_translate_tc<1, kTcGroups><<<grid, nt, smem_bytes<1>(p.P), st>>>(p, tt);
    else k_translate_tc<2, kTcGroups><<<grid, nt, smem_bytes<2>(p.P), st>>>(p, tt);
    return cudaGetLastError();
}

}  // namespace sfmm
