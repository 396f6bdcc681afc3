/*
 * CPU oracle for solidfmm's translation path (M2M, M2L, L2L).
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py as the checker.  The
 * product (libsfmm_gb300.so) never links, loads or calls it.
 *
 * Contents
 *   - solid harmonics R and S (restated from solidfmm/harmonics.cpp:32-224)
 *   - Dehnen's swap matrices B_n^{m,l} (solidfmm/swap_matrix.cpp:149-171)
 *   - naive O(P^4) translation formulas (doc/solidfmm.tex:1404-1432, with the
 *     M2M inner sum over l=-k..k)
 *   - a lane-batched restatement of the rotation-based O(P^3) driver
 *     (solidfmm/translations.cpp:37-630 over the generic microkernel
 *     semantics of solidfmm/microkernel_generic.cpp:37-380), multithreaded
 *     by target hash like solidfmm/multithreaded_translator.cpp:56-70,283.
 *
 * Layout: expansions in the reference's solid layout (solidfmm/solid.hpp:59-60):
 * re(n,m) at n(n+1)+m, im(n,m) at (n+1)^2+m, n<P, P(P+1) reals per expansion.
 * Batches: translation i reads source src + sidx[i]*sstride (order Pin[i])
 * and accumulates into dst + tidx[i]*dstride (order Pout[i]) with shift
 * (xyz[3i], xyz[3i+1], xyz[3i+2]) = new centre - old centre.
 * op: 0 = M2M, 1 = M2L, 2 = L2L.
 */
#ifndef SFMM_ORACLE_H
#define SFMM_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

void orc_R_d(size_t P, double x, double y, double z, double *out);
void orc_S_d(size_t P, double x, double y, double z, double *out);
double orc_swap_B(int n, int m, int l);

/* out[j] += sum_q charge[j*nq+q] * R(pos[j*nq+q] - centre[j]) : P2M (solid.cpp:70-104 fmadd of harmonics::R) */
void orc_p2m_d(size_t P, size_t nexp, size_t nq, const double *charge, const double *pos,
               const double *centre, double *out, size_t stride);
/* out[j] += sum_q charge * S(pos - centre) : P2L */
void orc_p2l_d(size_t P, size_t nexp, size_t nq, const double *charge, const double *pos,
               const double *centre, double *out, size_t stride);
/* potential sum_{n,m} conj-pairing of an expansion with a harmonic (solid.cpp:41-66 dot) */
double orc_dot_d(size_t PA, const double *A, size_t PB, const double *B);

int orc_naive_d(int op, size_t n, const double *src, size_t sstride, const uint32_t *Pin,
                double *dst, size_t dstride, const uint32_t *Pout, const uint32_t *sidx,
                const uint32_t *tidx, const double *xyz, int nthreads);

int orc_rot_d(int op, size_t n, const double *src, size_t sstride, const uint32_t *Pin,
              double *dst, size_t dstride, const uint32_t *Pout, const uint32_t *sidx,
              const uint32_t *tidx, const double *xyz, int nthreads, double *seconds);
int orc_rot_f(int op, size_t n, const float *src, size_t sstride, const uint32_t *Pin,
              float *dst, size_t dstride, const uint32_t *Pout, const uint32_t *sidx,
              const uint32_t *tidx, const float *xyz, int nthreads, double *seconds);

#ifdef __cplusplus
}
#endif
#endif
