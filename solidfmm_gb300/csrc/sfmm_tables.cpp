#include "sfmm_tables.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>

namespace sfmm {

std::vector<std::vector<double>> swap_matrices(int P)
{
    std::vector<std::vector<double>> B(P > 0 ? P : 0);
    auto b = [&](int n, int m, int l) -> double {
        if (n < 0 || std::abs(l) > n || std::abs(m) > n) return 0.0;
        return B[n][(m + n) + (l + n) * (2 * n + 1)];
    };
    for (int n = 0; n < P; ++n) {
        int w = 2 * n + 1;
        B[n].assign(size_t(w) * w, 0.0);
        auto at = [&](int m, int l) -> double & { return B[n][(m + n) + (l + n) * w]; };
        if (n == 0) {
            at(0, 0) = 1;
            continue;
        }
        // recursion in the degree (swap_matrix.cpp:155-170)
        for (int l = -n; l <= n; ++l) at(0, l) = 0.5 * (b(n - 1, 0, l - 1) - b(n - 1, 0, l + 1));
        for (int m = 0; m < n; ++m)
            for (int l = -n; l <= n; ++l) {
                at(m + 1, l) = 0.5 * (b(n - 1, m, l - 1) + b(n - 1, m, l + 1)) + b(n - 1, m, l);
                at(-m - 1, l) = 0.5 * (b(n - 1, -m, l - 1) + b(n - 1, -m, l + 1)) - b(n - 1, -m, l);
            }
    }
    return B;
}

namespace {

// sqrt(k!) in FP64 (k! itself is finite up to 170!, the largest the
// tables need for P <= 86).
struct SqrtFac {
    std::vector<double> v;
    explicit SqrtFac(int kmax) : v(kmax + 1)
    {
        double f = 1;
        for (int k = 0; k <= kmax; ++k) {
            if (k) f *= k;
            v[k] = std::sqrt(f);
        }
    }
    double operator()(int k) const { return v[k]; }
};

}  // namespace

double w_entry(const HostTables &t, int n, int part, int i, int j)
{
    const int d = n + 1, R = wrows(d, t.pad);
    if (i < 0 || j < 0 || i >= d || j >= d) return 0.0;
    const bool rnz = ((i + j + n) & 1) == 0;
    if (rnz != (part == 0)) return 0.0;
    return t.W[t.woff[n] + size_t(j >> 1) * 2 * R + (part ? R : 0) + i];
}

namespace {

// Swap blocks of degrees n < nmax with rows padded to a multiple of pad (the
// layout of HostTables::W).
void build_w(const std::vector<std::vector<double>> &B, const SqrtFac &sf, int nmax, int pad,
             std::vector<double> &W, std::vector<int> &woff)
{
    const double s2 = std::sqrt(2.0);
    woff.resize(nmax);
    size_t tot = 0;
    for (int n = 0; n < nmax; ++n) {
        woff[n] = (int)tot;
        tot += 2 * size_t(wcols(n + 1)) * wrows(n + 1, pad);
    }
    W.assign(tot, 0.0);
    for (int n = 0; n < nmax; ++n) {
        const int d = n + 1, w = 2 * n + 1;
        auto Bv = [&](int m, int l) { return B[n][(m + n) + (l + n) * w]; };
        auto D = [&](int m) { return sf(n - m) * sf(n + m); };
        auto E = [&](int m) { return m == 0 ? D(0) / s2 : D(m); };
        const int R = wrows(d, pad);
        double *WR = &W[woff[n]];  // slot t: W_R rows at 2tR, W_I rows at 2tR + R
        double *WI = WR + R;
        for (int i = 0; i < d; ++i)       // output row (coefficient m = i)
            for (int j = 0; j < d; ++j) { // input column (coefficient l = j)
                // the reference's real/imag combinations (operator_data.cpp:99-147)
                double rf, imf;
                if (j == 0) rf = Bv(0, i);
                else if (j & 1) rf = Bv(j, i) - Bv(-j, i);
                else rf = Bv(j, i) + Bv(-j, i);
                if (j & 1) imf = Bv(j, i) + Bv(-j, i);
                else imf = Bv(j, i) - Bv(-j, i);
                // keep only the checkerboard the reference stores
                const bool rnz = ((i + j + n) & 1) == 0;
                const size_t slot = size_t(j >> 1) * 2 * R + i;  // j = jr(i) + 2t or ji(i) + 2t
                if (rnz) WR[slot] = rf * (E(i) / E(j));
                else if (i > 0 && j > 0) WI[slot] = imf * (D(i) / D(j));
            }
    }
}

}  // namespace

HostTables build_tables(int P)
{
    HostTables t;
    t.P = P;
    const int pad = row_pad(P);
    t.pad = pad;
    auto B = swap_matrices(P);
    SqrtFac sf(2 * P + 2);
    std::vector<double> fac(2 * P + 2);
    fac[0] = 1;
    for (int k = 1; k < 2 * P + 2; ++k) fac[k] = fac[k - 1] * k;
    const double s2 = std::sqrt(2.0);

    build_w(B, sf, P, pad, t.W, t.woff);
    if (pad != 8) build_w(B, sf, std::min(P, 32), 8, t.W8, t.woff8);

    size_t ne = size_t(P) * (P + 1) / 2;
    t.e_in_M.resize(ne);
    t.e_in_L.resize(ne);
    t.e_out_L.resize(ne);
    t.e_out_M.resize(ne);
    for (int n = 0; n < P; ++n)
        for (int m = 0; m <= n; ++m) {
            double D = sf(n - m) * sf(n + m);
            double s = m == 0 ? s2 : 1.0;
            size_t k = size_t(n) * (n + 1) / 2 + m;
            t.e_in_M[k] = D / s;
            t.e_in_L[k] = 1.0 / (D * s);
            t.e_out_L[k] = D * s;
            t.e_out_M[k] = s / D;
        }

    t.hoff.resize(P);
    size_t th = 0;
    for (int m = 0; m < P; ++m) {
        t.hoff[m] = (int)th;
        th += size_t(P - m + 2) * hrows(P - m, pad);
    }
    for (int op = 0; op < 3; ++op) t.H[op].assign(th, 0.0);
    for (int m = 0; m < P; ++m) {
        const int HR = hrows(P - m, pad);
        for (int k = m; k < P; ++k)
            for (int np = m; np < P; ++np) {
                size_t idx = t.hoff[m] + size_t(k - m) * HR + (np - m);
                double Dk = sf(k - m) * sf(k + m);
                double Dn = sf(np - m) * sf(np + m);
                // M2L: (-1)^(n'+m) (n'+k)! / (D^(n') D^(k))   (zm2l, translations.cpp:283-296)
                double h1 = fac[np + k] / Dn / Dk;
                t.H[1][idx] = ((np + m) & 1) ? -h1 : h1;
                // M2M: D^(n') / ((n'-k)! D^(k)), k <= n'   (zm2m, translations.cpp:366-377)
                if (k <= np) t.H[0][idx] = Dn / (fac[np - k] * Dk);
                // L2L: D^(k) / (D^(n') (k-n')!), k >= n'   (zm2m, translations.cpp:440-451)
                if (k >= np) t.H[2][idx] = Dk / (Dn * fac[k - np]);
            }
    }
    return t;
}

}  // namespace sfmm
