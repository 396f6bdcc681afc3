/*
 * CPU oracle for solidfmm's translation path.  TEST INFRASTRUCTURE ONLY:
 * tests/, __graft_entry__.smoke() and bench.py's CPU legs use it as the
 * checker; the product never links or calls it.  See oracle.h for layout.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static double now_seconds(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* target ownership hash (same role as the NASAM mix of multithreaded_translator.cpp:56-70) */
static uint64_t target_hash(uint64_t v)
{
    v ^= v >> 31;
    v *= 0x7fb5d329728ea185ULL;
    v ^= v >> 27;
    v *= 0x81dadef4bc2dd44dULL;
    v ^= v >> 33;
    return v;
}

#define RE(n, m) ((size_t)(n) * ((n) + 1) + (m))
#define IM(n, m) ((size_t)((n) + 1) * ((n) + 1) + (m))

/* ---- solid harmonics (solidfmm/harmonics.cpp:32-80 R_impl, :177-224 S_impl) ---- */
void orc_R_d(size_t P, double x, double y, double z, double *o)
{
    if (P == 0) return;
    memset(o, 0, sizeof(double) * P * (P + 1));
    o[RE(0, 0)] = 1;
    if (P == 1) return;
    o[RE(1, 0)] = z;
    o[RE(1, 1)] = x / 2;
    o[IM(1, 1)] = y / 2;
    for (size_t m = 2; m < P; ++m) {
        double a = o[RE(m - 1, m - 1)], b = o[IM(m - 1, m - 1)], f = 1.0 / (double)(2 * m);
        o[RE(m, m)] = (a * x - b * y) * f;
        o[IM(m, m)] = (a * y + b * x) * f;
    }
    for (size_t m = 1; m + 1 < P; ++m) {
        o[RE(m + 1, m)] = z * o[RE(m, m)];
        o[IM(m + 1, m)] = z * o[IM(m, m)];
    }
    double r2 = x * x + y * y + z * z;
    for (size_t m = 0; m + 2 < P; ++m)
        for (size_t n = m + 2; n < P; ++n) {
            double f = 1.0 / ((double)(n + m) * (double)(n - m));
            o[RE(n, m)] = (o[RE(n - 1, m)] * z * (double)(2 * n - 1) - r2 * o[RE(n - 2, m)]) * f;
            o[IM(n, m)] = (o[IM(n - 1, m)] * z * (double)(2 * n - 1) - r2 * o[IM(n - 2, m)]) * f;
        }
}

void orc_S_d(size_t P, double x, double y, double z, double *o)
{
    if (P == 0) return;
    memset(o, 0, sizeof(double) * P * (P + 1));
    double r2inv = 1 / (x * x + y * y + z * z);
    o[RE(0, 0)] = sqrt(r2inv);
    if (P == 1) return;
    o[RE(1, 0)] = z * r2inv * o[RE(0, 0)];
    o[RE(1, 1)] = x * r2inv * o[RE(0, 0)];
    o[IM(1, 1)] = y * r2inv * o[RE(0, 0)];
    for (size_t m = 2; m < P; ++m) {
        double a = o[RE(m - 1, m - 1)], b = o[IM(m - 1, m - 1)], f = (double)(2 * m - 1) * r2inv;
        o[RE(m, m)] = (a * x - b * y) * f;
        o[IM(m, m)] = (a * y + b * x) * f;
    }
    for (size_t m = 1; m + 1 < P; ++m) {
        double f = (double)(2 * m + 1) * z * r2inv;
        o[RE(m + 1, m)] = f * o[RE(m, m)];
        o[IM(m + 1, m)] = f * o[IM(m, m)];
    }
    for (size_t m = 0; m + 2 < P; ++m)
        for (size_t n = m + 2; n < P; ++n) {
            double c = (double)(n + m - 1) * (double)(n - m - 1);
            o[RE(n, m)] = (o[RE(n - 1, m)] * z * (double)(2 * n - 1) - c * o[RE(n - 2, m)]) * r2inv;
            o[IM(n, m)] = (o[IM(n - 1, m)] * z * (double)(2 * n - 1) - c * o[IM(n - 2, m)]) * r2inv;
        }
}

/* ---- Dehnen's swap matrices (solidfmm/swap_matrix.cpp:149-171), stored per n as (2n+1)^2, [m+n + (l+n)(2n+1)] ---- */
#define SWAPB_MAX 128
static double *g_swapB[SWAPB_MAX];
static pthread_mutex_t g_swapB_lock = PTHREAD_MUTEX_INITIALIZER;

static double swapB_entry(int n, int m, int l)
{
    if (n < 0 || abs(l) > n || abs(m) > n) return 0;
    return g_swapB[n][(m + n) + (l + n) * (2 * n + 1)];
}

static const double *swapB_get(int n)
{
    pthread_mutex_lock(&g_swapB_lock);
    for (int k = 0; k <= n; ++k) {
        if (g_swapB[k]) continue;
        int w = 2 * k + 1;
        double *B = (double *)calloc((size_t)w * w, sizeof(double));
        if (k == 0) {
            B[0] = 1;
        } else {
            for (int l = -k; l <= k; ++l)
                B[(0 + k) + (l + k) * w] = 0.5 * (swapB_entry(k - 1, 0, l - 1) - swapB_entry(k - 1, 0, l + 1));
            for (int m = 0; m < k; ++m)
                for (int l = -k; l <= k; ++l) {
                    B[(m + 1 + k) + (l + k) * w] =
                        0.5 * (swapB_entry(k - 1, m, l - 1) + swapB_entry(k - 1, m, l + 1)) + swapB_entry(k - 1, m, l);
                    B[(-m - 1 + k) + (l + k) * w] =
                        0.5 * (swapB_entry(k - 1, -m, l - 1) + swapB_entry(k - 1, -m, l + 1)) - swapB_entry(k - 1, -m, l);
                }
        }
        g_swapB[k] = B;
    }
    pthread_mutex_unlock(&g_swapB_lock);
    return g_swapB[n];
}

double orc_swap_B(int n, int m, int l)
{
    if (n < 0 || n >= SWAPB_MAX) return 0;
    swapB_get(n);
    return swapB_entry(n, m, l);
}

/* ---- P2M / P2L / dot ---- */
static void p2x(int sing, size_t P, size_t nexp, size_t nq, const double *q, const double *pos,
                const double *c, double *out, size_t stride)
{
    double *h = (double *)malloc(sizeof(double) * (P * (P + 1) + 1));
    for (size_t j = 0; j < nexp; ++j)
        for (size_t k = 0; k < nq; ++k) {
            const double *p = pos + 3 * (j * nq + k);
            double x = p[0] - c[3 * j], y = p[1] - c[3 * j + 1], z = p[2] - c[3 * j + 2];
            if (sing) orc_S_d(P, x, y, z, h); else orc_R_d(P, x, y, z, h);
            double w = q[j * nq + k];
            for (size_t i = 0; i < P * (P + 1); ++i) out[j * stride + i] += w * h[i];
        }
    free(h);
}
void orc_p2m_d(size_t P, size_t nexp, size_t nq, const double *q, const double *pos, const double *c,
               double *out, size_t stride)
{
    p2x(0, P, nexp, nq, q, pos, c, out, stride);
}
void orc_p2l_d(size_t P, size_t nexp, size_t nq, const double *q, const double *pos, const double *c,
               double *out, size_t stride)
{
    p2x(1, P, nexp, nq, q, pos, c, out, stride);
}

/* solidfmm/solid.cpp:41-66: 2*sum(a*b) - sum over the m=0 column */
double orc_dot_d(size_t PA, const double *A, size_t PB, const double *B)
{
    size_t P = PA < PB ? PA : PB;
    double t = 0, t2 = 0;
    for (size_t n = 0; n < P; ++n)
        for (size_t m = 0; m <= n; ++m) {
            t += A[RE(n, m)] * B[RE(n, m)] + A[IM(n, m)] * B[IM(n, m)];
        }
    for (size_t n = 0; n < P; ++n) t2 += A[RE(n, 0)] * B[RE(n, 0)];
    return 2 * t - t2;
}

/* ---- naive O(P^4) formulas (doc/solidfmm.tex:1404-1432) ---- */
/* coefficient C_n^m of an expansion for any m, via C_n^{-m} = (-1)^m conj(C_n^m) (doc/solidfmm.tex:1097-1101) */
static void coef(const double *C, int P, int n, int m, double *re, double *im)
{
    if (n < 0 || n >= P || abs(m) > n) { *re = *im = 0; return; }
    int am = abs(m);
    double r = C[RE(n, am)], i = C[IM(n, am)];
    if (m < 0) {
        double s = (am & 1) ? -1 : 1;
        r *= s;
        i = -i * s;
    }
    *re = r;
    *im = i;
}

static void naive_one(int op, const double *src, int Pin, double *dst, int Pout, double x, double y, double z,
                      double *h)
{
    int PH = Pin + Pout + 1;
    if (op == 1) orc_S_d((size_t)PH, x, y, z, h);
    else if (op == 0) orc_R_d((size_t)PH, -x, -y, -z, h);
    else orc_R_d((size_t)PH, x, y, z, h);
    for (int n = 0; n < Pout; ++n)
        for (int m = 0; m <= n; ++m) {
            double ar = 0, ai = 0;
            if (op == 1) { /* L_n^m = (-1)^n sum_k sum_l conj(M_k^l) S_{n+k}^{m+l}(r) */
                for (int k = 0; k < Pin; ++k)
                    for (int l = -k; l <= k; ++l) {
                        double mr, mi, sr, si;
                        coef(src, Pin, k, l, &mr, &mi);
                        coef(h, PH, n + k, m + l, &sr, &si);
                        ar += mr * sr + mi * si;
                        ai += mr * si - mi * sr;
                    }
                if (n & 1) { ar = -ar; ai = -ai; }
            } else if (op == 0) { /* M_n^m = sum_{k<=n} sum_{l=-k..k} M_k^l R_{n-k}^{m-l}(-r) */
                for (int k = 0; k < Pin && k <= n; ++k)
                    for (int l = -k; l <= k; ++l) {
                        double mr, mi, rr, ri;
                        coef(src, Pin, k, l, &mr, &mi);
                        coef(h, PH, n - k, m - l, &rr, &ri);
                        ar += mr * rr - mi * ri;
                        ai += mr * ri + mi * rr;
                    }
            } else { /* L_n^m = sum_{k=n}^{Pin-1} sum_l L_k^l conj(R_{k-n}^{l-m}(r)) */
                for (int k = n; k < Pin; ++k)
                    for (int l = -k; l <= k; ++l) {
                        double lr, li, rr, ri;
                        coef(src, Pin, k, l, &lr, &li);
                        coef(h, PH, k - n, l - m, &rr, &ri);
                        ar += lr * rr + li * ri;
                        ai += li * rr - lr * ri;
                    }
            }
            dst[RE(n, m)] += ar;
            if (m) dst[IM(n, m)] += ai;
        }
}

typedef struct {
    int op, tid, nthr;
    size_t n;
    const double *src; size_t sstride; const uint32_t *Pin;
    double *dst; size_t dstride; const uint32_t *Pout;
    const uint32_t *sidx, *tidx;
    const double *xyz;
} naive_job;

static void *naive_worker(void *arg)
{
    naive_job *j = (naive_job *)arg;
    int pm = 0;
    for (size_t i = 0; i < j->n; ++i) {
        int s = (int)(j->Pin[i] + j->Pout[i] + 1);
        if (s > pm) pm = s;
    }
    double *h = (double *)malloc(sizeof(double) * ((size_t)pm * (pm + 1) + 1));
    for (size_t i = 0; i < j->n; ++i) {
        uint32_t t = j->tidx ? j->tidx[i] : (uint32_t)i;
        if (j->nthr > 1 && (int)(target_hash(t) % (uint64_t)j->nthr) != j->tid) continue;
        uint32_t s = j->sidx ? j->sidx[i] : (uint32_t)i;
        naive_one(j->op, j->src + (size_t)s * j->sstride, (int)j->Pin[i], j->dst + (size_t)t * j->dstride,
                  (int)j->Pout[i], j->xyz[3 * i], j->xyz[3 * i + 1], j->xyz[3 * i + 2], h);
    }
    free(h);
    return NULL;
}

int orc_naive_d(int op, size_t n, const double *src, size_t sstride, const uint32_t *Pin, double *dst,
                size_t dstride, const uint32_t *Pout, const uint32_t *sidx, const uint32_t *tidx,
                const double *xyz, int nthreads)
{
    if (op < 0 || op > 2) return 1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    naive_job jobs[256];
    pthread_t th[256];
    for (int t = 0; t < nthreads; ++t) {
        jobs[t] = (naive_job){op, t, nthreads, n, src, sstride, Pin, dst, dstride, Pout, sidx, tidx, xyz};
        if (nthreads > 1) pthread_create(&th[t], NULL, naive_worker, &jobs[t]);
        else naive_worker(&jobs[t]);
    }
    if (nthreads > 1)
        for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    return 0;
}

/* ---- rotation-based driver, double and float ---- */
#define LANES 8
#define REAL double
#define SUF _d
#define HYPOT hypot
#include "oracle_rot.inc"
#undef REAL
#undef SUF
#undef HYPOT

#define REAL float
#define SUF _f
#define HYPOT hypotf
#include "oracle_rot.inc"
#undef REAL
#undef SUF
#undef HYPOT
