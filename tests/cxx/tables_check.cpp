// Operator tables (sfmm_tables.cpp) on the host: for several context orders
// the swap blocks of every degree are orthogonal involutions (W W = I for the
// full matrix assembled from its W_R and W_I checkerboards), the 8-row padded
// copy that contexts above order 32 keep for their 4- and 8-thread launches
// holds the same entries as the 32-row original, every block's padding is
// zero, and the z-translation offsets stay inside their tables.  Prints "ok"
// and exits 0 on success.
#include <cmath>
#include <cstdio>
#include <vector>

#include "sfmm_tables.hpp"

using namespace sfmm;

static int failures = 0;
#define CHECK(c, ...)                                   \
    do {                                                \
        if (!(c)) {                                     \
            std::printf("FAIL %s: ", #c);               \
            std::printf(__VA_ARGS__);                   \
            std::printf("\n");                          \
            ++failures;                                 \
        }                                               \
    } while (0)

// the swap of degree n as a dense real (2d x 2d) map on (re, im) parts:
// re' = W_R re, im' = W_I im (W_I zero in row/column 0: im of m = 0 is 0)
static double involution_error(const HostTables &t, int n)
{
    const int d = n + 1;
    double worst = 0;
    for (int part = 0; part < 2; ++part)
        for (int i = 0; i < d; ++i)
            for (int j = 0; j < d; ++j) {
                double s = 0;
                for (int k = 0; k < d; ++k) s += w_entry(t, n, part, i, k) * w_entry(t, n, part, k, j);
                const double want = (i == j && !(part == 1 && i == 0)) ? 1.0 : 0.0;
                worst = std::fmax(worst, std::fabs(s - want));
            }
    return worst;
}

int main()
{
    for (int P : {1, 2, 16, 32, 33, 86}) {
        const HostTables t = build_tables(P);
        CHECK(t.pad == row_pad(P), "P=%d", P);
        CHECK((int)t.woff.size() == P, "P=%d", P);
        for (int n = 0; n < P; ++n) {
            const double err = involution_error(t, n);
            CHECK(err < 1e-12 * (n + 1), "P=%d n=%d error %g", P, n, err);
            // the block ends before the next one starts, padding zero
            const int d = n + 1, R = wrows(d, t.pad);
            const size_t end = t.woff[n] + 2 * size_t(wcols(d)) * R;
            CHECK(end == (n + 1 < P ? (size_t)t.woff[n + 1] : t.W.size()), "P=%d n=%d", P, n);
            for (int slot = 0; slot < wcols(d); ++slot)
                for (int part = 0; part < 2; ++part)
                    for (int i = d; i < R; ++i)
                        CHECK(t.W[t.woff[n] + size_t(slot) * 2 * R + part * R + i] == 0.0, "P=%d n=%d pad", P, n);
        }
        if (t.pad == 8) {
            CHECK(t.W8.empty() && t.woff8.empty(), "P=%d", P);
        } else {
            const int n8 = P < 32 ? P : 32;
            CHECK((int)t.woff8.size() == n8, "P=%d", P);
            HostTables v;  // the 8-row copy seen through the same accessor
            v.pad = 8;
            v.W = t.W8;
            v.woff = t.woff8;
            for (int n = 0; n < n8; ++n)
                for (int part = 0; part < 2; ++part)
                    for (int i = 0; i <= n; ++i)
                        for (int j = 0; j <= n; ++j)
                            CHECK(w_entry(v, n, part, i, j) == w_entry(t, n, part, i, j), "P=%d n=%d (%d,%d)", P, n,
                                  i, j);
            const size_t end8 = t.woff8[n8 - 1] + 2 * size_t(wcols(n8)) * wrows(n8, 8);
            CHECK(end8 == t.W8.size(), "P=%d", P);
        }
        // z-translation: column m's block ends inside the table
        for (int m = 0; m < P; ++m) {
            const size_t last = t.hoff[m] + size_t(P - m - 1) * hrows(P - m, t.pad) + (P - m - 1);
            for (int op = 0; op < 3; ++op) CHECK(last < t.H[op].size(), "P=%d m=%d", P, m);
        }
    }
    if (failures) return 1;
    std::printf("ok\n");
    return 0;
}
