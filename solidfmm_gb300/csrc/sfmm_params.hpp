// Kernel parameter block shared by the C ABI (host C++) and the kernels.
#pragma once

#include <cstdint>

#include <vector_types.h>

namespace sfmm {

enum { OP_M2M = 0, OP_M2L = 1, OP_L2L = 2 };

// buffer slots per translation covered by the FP32-range kernels' table of
// coefficient degrees (every order up to 28 with its padding)
constexpr int kDegreeTableSize = 1024;

struct KParams {
    int op;
    int P;          // order bound of this batch: every p_in/p_out <= P
    int Ptab;       // order the tables were built for (>= P)
    long long n;
    const void *src;
    long long sstride;
    long long nsrc;     // expansions addressable through src
    const uint32_t *sidx;
    void *dst;
    long long dstride;
    long long ndst;     // expansions addressable through dst
    const uint32_t *tidx;
    const uint32_t *pin;
    const uint32_t *pout;
    const double *shift;
    const uint32_t *perm;
    long long nidx;     // entries of pin/pout/shift/sidx/tidx (perm values index these)
    int atomic;
    int in_hbm;    // expansions in device memory (0: host memory read over the link)
    const void *W;      // arith-typed swap matrices (padded, see sfmm_tables.hpp)
    const int *Wq;      // swap matrices in Q1.30 (fixed-point variant), same layout as W
    const int *woff;    // offset of degree n's W blocks
    const int *hoff;    // offset of column m's z matrix
    int rowpad;         // row padding of W and H blocks (8 or 32)
    const void *ein;    // arith-typed forward edge factors (op dependent)
    const void *eout;   // arith-typed backward edge factors (op dependent)
    const void *H;      // arith-typed z matrices of this op
    int spad;           // buffer elements per translation
    int TS;             // translations per CTA tile
    void *scratch;      // global buffer (GBUF kernels)
    int *status;        // device error word: bit 0 = a translation had an out-of-range index or order
    // pointer mode (both null otherwise): translation t reads its source at
    // src_ptr[t] and accumulates into dst_ptr[t] (addresses the GPU can use,
    // e.g. host solids on a GPU that walks the host page tables); sidx/tidx
    // are then null and nsrc = ndst = nidx
    const unsigned long long *src_ptr;
    const unsigned long long *dst_ptr;
    // work-list mode (non-null work): CTAs take tiles in the list's order from
    // the counter (zero at launch); tile k covers entries [work[k].x,
    // work[k].x + work[k].y) of the processing order, at most TS of them
    const uint2 *work;
    unsigned *work_counter;
    long long nwork;
};

}  // namespace sfmm
