// Host bookkeeping of the classic call (sfmm_hostbatch.cpp) against a
// sequential restatement: entries in translation-major order, one slot per
// distinct target address with the largest coefficient count named for it,
// the first invalid translation reported.  Addresses are synthetic (the
// bookkeeping never dereferences a solid).  Prints "ok" and exits 0 on success.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <random>
#include <set>
#include <vector>

#include "sfmm_hostbatch.hpp"

using namespace sfmm;

static int failures = 0;
#define CHECK(c)                                                                  \
    do {                                                                          \
        if (!(c)) {                                                               \
            std::printf("FAIL %s:%d: %s (case %s)\n", __FILE__, __LINE__, #c, name); \
            ++failures;                                                           \
            return;                                                               \
        }                                                                         \
    } while (0)

struct Batch {
    std::vector<const void *> src;
    std::vector<void *> dst;
    std::vector<size_t> pin, pout;
    std::vector<double> x, y, z;
    std::vector<float> xf, yf, zf;
};

static void *addr(unsigned long long a) { return reinterpret_cast<void *>(static_cast<uintptr_t>(a)); }

// Run the bookkeeping with nthr threads and compare with the restatement.
static void check(const char *name, const Batch &b, size_t dim, bool f64, size_t P, size_t nthr, int want_path,
                  bool want_repeat)
{
    ClassicInput in;
    in.n = b.src.size();
    in.src = b.src.data();
    in.p_in = b.pin.data();
    in.dst = b.dst.data();
    in.p_out = b.pout.data();
    in.dim = dim;
    in.x = f64 ? (const void *)b.x.data() : (const void *)b.xf.data();
    in.y = f64 ? (const void *)b.y.data() : (const void *)b.yf.data();
    in.z = f64 ? (const void *)b.z.data() : (const void *)b.zf.data();
    in.f64 = f64;
    in.P = P;
    const size_t es = f64 ? 8 : 4;
    // restatement: entries, and slots by address
    std::vector<unsigned long long> sp, dp;
    std::vector<uint32_t> pi, po;
    std::vector<double> sh;
    std::map<unsigned long long, uint32_t> maxcnt;
    size_t pmax = 1;
    for (size_t i = 0; i < in.n; ++i) {
        pmax = std::max(pmax, std::max(b.pin[i], b.pout[i]));
        if (!b.pin[i] || !b.pout[i]) continue;
        for (size_t d = 0; d < dim; ++d) {
            sp.push_back((uintptr_t)b.src[i] + d * b.pin[i] * (b.pin[i] + 1) * es);
            const unsigned long long t = (uintptr_t)b.dst[i] + d * b.pout[i] * (b.pout[i] + 1) * es;
            dp.push_back(t);
            pi.push_back((uint32_t)b.pin[i]);
            po.push_back((uint32_t)b.pout[i]);
            sh.push_back(f64 ? b.x[i] : (double)b.xf[i]);
            sh.push_back(f64 ? b.y[i] : (double)b.yf[i]);
            sh.push_back(f64 ? b.z[i] : (double)b.zf[i]);
            uint32_t &m = maxcnt[t];
            m = std::max<uint32_t>(m, (uint32_t)(b.pout[i] * (b.pout[i] + 1)));
        }
    }
    const ClassicScan sc = classic_scan(in, nthr);
    CHECK(sc.bad == SIZE_MAX);
    CHECK(sc.entries == sp.size());
    CHECK(sc.pmax == pmax);
    const size_t M = sc.entries;
    std::vector<unsigned long long> osp(M), odp(M), otp(M);
    std::vector<uint32_t> opi(M), opo(M), oti(M), otc(M);
    std::vector<double> osh(3 * M);
    ClassicEntries out;
    out.sptr = osp.data();
    out.dptr = odp.data();
    out.pin = opi.data();
    out.pout = opo.data();
    out.tidx = oti.data();
    out.shift = osh.data();
    out.tptr = otp.data();
    out.tcnt = otc.data();
    SlotScratch scratch;
    bool repeat = !want_repeat;
    SlotPath path;
    const size_t nt = classic_fill(in, sc, out, scratch, &repeat, &path);
    CHECK(osp == sp && odp == dp && opi == pi && opo == po && osh == sh);
    CHECK(repeat == want_repeat);
    CHECK((int)path == want_path);
    CHECK(nt == maxcnt.size());
    std::set<unsigned long long> seen;
    for (size_t s = 0; s < nt; ++s) {
        CHECK(seen.insert(otp[s]).second);  // slots are distinct
        CHECK(maxcnt.count(otp[s]) && otc[s] == maxcnt[otp[s]]);
    }
    for (size_t e = 0; e < M; ++e) CHECK(oti[e] < nt && otp[oti[e]] == dp[e]);
    if (!want_repeat)
        for (size_t e = 0; e < M; ++e) CHECK(oti[e] == e);
}

static Batch make(size_t n, std::mt19937_64 &rng)
{
    Batch b;
    b.src.resize(n);
    b.dst.resize(n);
    b.pin.resize(n);
    b.pout.resize(n);
    std::uniform_real_distribution<double> u(-3, 3);
    for (size_t i = 0; i < n; ++i) {
        b.x.push_back(u(rng));
        b.y.push_back(u(rng));
        b.z.push_back(u(rng));
        b.xf.push_back((float)b.x.back());
        b.yf.push_back((float)b.y.back());
        b.zf.push_back((float)b.z.back());
    }
    return b;
}

int main()
{
    std::mt19937_64 rng(7);
    const unsigned long long SB = 0x10000000000ull, DB = 0x20000000000ull, SLOT = 1 << 16;
    for (size_t nthr : {1, 3, 8}) {
        for (size_t dim : {1, 3}) {
            for (bool f64 : {true, false}) {
                const size_t n = 40000;
                // 1. distinct targets at rising addresses, some zero orders
                Batch b = make(n, rng);
                for (size_t i = 0; i < n; ++i) {
                    b.src[i] = addr(SB + (rng() % 1000) * SLOT);
                    b.dst[i] = addr(DB + i * SLOT);
                    b.pin[i] = 1 + rng() % 12;
                    b.pout[i] = (i % 97 == 5) ? 0 : 1 + rng() % 12;
                }
                check("ascending", b, dim, f64, 12, nthr, (int)SlotPath::ascending, false);
                // 2. sorted by target, runs of 1..30; with one component the
                //    orders named for a target vary (its slot takes the
                //    largest), with several they locate the components and
                //    stay the target's own
                size_t t = 0, left = 0, po = 1;
                for (size_t i = 0; i < n; ++i) {
                    if (!left) {
                        ++t;
                        left = 1 + rng() % 30;
                        po = 1 + rng() % 12;
                    }
                    --left;
                    b.dst[i] = addr(DB + t * SLOT);
                    b.pout[i] = dim == 1 ? 1 + rng() % 12 : po;
                }
                // (components of a repeated target interleave: the addresses
                // fall back at each repetition, so several components hash)
                check("runs", b, dim, f64, 12, nthr, (int)(dim == 1 ? SlotPath::runs : SlotPath::hashed), true);
                // 3. the same targets in random order
                for (size_t i = n - 1; i > 0; --i) {
                    const size_t j = rng() % (i + 1);
                    std::swap(b.dst[i], b.dst[j]);
                    std::swap(b.pout[i], b.pout[j]);
                }
                check("hashed", b, dim, f64, 12, nthr, (int)SlotPath::hashed, true);
                // 4. distinct targets at falling addresses: hashed, no repeat
                for (size_t i = 0; i < n; ++i) b.dst[i] = addr(DB + (n - i) * SLOT);
                check("descending", b, dim, f64, 12, nthr, (int)SlotPath::hashed, false);
            }
        }
        // 5. errors: the first invalid translation, order checked before pointers
        std::mt19937_64 r2(3);
        Batch b = make(50000, r2);
        for (size_t i = 0; i < b.src.size(); ++i) {
            b.src[i] = addr(SB + i * SLOT);
            b.dst[i] = addr(DB + i * SLOT);
            b.pin[i] = b.pout[i] = 8;
        }
        ClassicInput in;
        in.n = b.src.size();
        in.src = b.src.data();
        in.p_in = b.pin.data();
        in.dst = b.dst.data();
        in.p_out = b.pout.data();
        in.x = b.x.data();
        in.y = b.y.data();
        in.z = b.z.data();
        in.P = 8;
        b.dst[41000] = nullptr;
        b.pout[45000] = 9;
        const char *name = "errors";
        auto run = [&]() {
            ClassicScan sc = classic_scan(in, nthr);
            return std::make_pair(sc.bad, sc.bad_kind);
        };
        auto r = run();
        if (!(r.first == 41000 && r.second == 2)) {
            std::printf("FAIL errors: %zu %d\n", r.first, r.second);
            ++failures;
        }
        b.pin[30000] = 9;
        r = run();
        if (!(r.first == 30000 && r.second == 1)) {
            std::printf("FAIL errors: %zu %d\n", r.first, r.second);
            ++failures;
        }
        b.pin[30000] = 0;  // zero order with a valid target: no error, no entry
        b.src[30000] = nullptr;
        r = run();
        if (!(r.first == 41000 && r.second == 2)) {
            std::printf("FAIL errors: %zu %d\n", r.first, r.second);
            ++failures;
        }
        (void)name;
    }
    if (failures) return 1;
    std::printf("ok\n");
    return 0;
}
