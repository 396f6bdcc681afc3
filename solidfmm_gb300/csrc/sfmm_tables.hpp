// Host-side operator tables for the GPU translation kernels.
//
// Plays the role of the reference's operator_data<real> (factorials and the
// packed real/imag swap matrices, solidfmm/operator_data.cpp:48-244), built
// once per context in FP64 and uploaded.  The kernels work in an orthogonal
// basis of each degree-n subspace:
//
//   D_m   = sqrt((n-m)! (n+m)!),   s_0 = sqrt(2), s_m = 1 (m > 0)
//   E_m   = D_m / s_m,             F_m = D_m * s_m
//   W_R   = E Rf E^-1 = F^-1 Rt F  (Rf, Rt: the reference's real swap matrix and its
//                                   transposed variant, operator_data.cpp:48-122)
//   W_I   = D If D^-1 = D^-1 It D  (imag swap matrix, operator_data.cpp:74-147)
//
// W_R and W_I are orthogonal, symmetric involutions with entries |w| <= 1, so
// both the forward (Rf) and backward (Rt) swaps use the same W.  The diagonal
// scalings are folded into the edge factors (first and last rotation of each
// degree) and into the z-translation matrices H_m.
#pragma once

#include <cstddef>
#include <vector>

namespace sfmm {

struct HostTables {
    int P = 0;
    // W for degree n (d = n+1) at woff[n].  Only the checkerboard a swap
    // uses is stored: W_R(i, j) is nonzero only for j = jr(i) + 2t with
    // jr(i) = (i+n) & 1, W_I(i, j) only for j = ji(i) + 2t with
    // ji(i) = jr(i) ^ 1.  Slot t holds R = wrows(d,pad) rows of W_R (row i at
    // 2tR + i) followed by R rows of W_I (at 2tR + R + i).  Rows are padded
    // to a multiple of row_pad(P) and slots to wcols(d) = (d+3)/2 with zeros
    // (the swap loops prefetch one slot past the last column), so the
    // kernels load coefficients without bounds checks.
    int pad = 8;
    std::vector<double> W;
    std::vector<int> woff;
    // The kernels' swap loops step through a block with a compile-time row
    // count: 8-row padding for 4 or 8 threads per translation (order bounds up
    // to 32), 32-row padding for one warp per translation.  A context above
    // order 32 (pad 32) therefore also keeps the blocks of degrees below 32
    // padded to 8 rows, for its launches at order bounds up to 32; empty when
    // pad is 8.
    std::vector<double> W8;
    std::vector<int> woff8;
    // Edge factors indexed n(n+1)/2 + m:
    std::vector<double> e_in_M;   // E^(n)_m        forward of M2M/M2L inputs
    std::vector<double> e_in_L;   // 1 / F^(n)_m    forward of L2L inputs
    std::vector<double> e_out_L;  // F^(n)_m        backward of M2L/L2L outputs
    std::vector<double> e_out_M;  // 1 / E^(n)_m    backward of M2M outputs
    // z-translation matrices per op (0 M2M, 1 M2L, 2 L2L) and column m:
    // entry (output n', input k) at hoff[m] + (k-m)*hrows(P-m,pad) + (n'-m),
    // output rows padded with zeros to a multiple of row_pad(P).
    std::vector<double> H[3];
    std::vector<int> hoff;
};

// Dehnen's swap matrix B_n^{m,l} (swap_matrix.cpp:149-171), all n < P,
// stored per n as (2n+1)^2 with (m,l) at (m+n) + (l+n)(2n+1).
std::vector<std::vector<double>> swap_matrices(int P);

// Row padding of the coefficient blocks: 8 when the kernels run 4 threads
// per translation (orders up to 32), 32 when they run one warp per
// translation (larger orders).
inline int row_pad(int P) { return P <= 32 ? 8 : 32; }
inline int wrows(int d, int pad) { return (d + pad - 1) & ~(pad - 1); }
inline int wcols(int d) { return (d + 3) / 2; }
// W_R (part 0) or W_I (part 1) of degree n at (row i, column j), from the
// compact layout
double w_entry(const HostTables &t, int n, int part, int i, int j);
inline int hrows(int L, int pad) { return (L + pad - 1) & ~(pad - 1); }

HostTables build_tables(int P);

}  // namespace sfmm
