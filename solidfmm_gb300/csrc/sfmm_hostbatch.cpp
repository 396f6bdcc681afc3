// Parallel host bookkeeping of the classic translation call (declarations and
// the reference interfaces it serves: sfmm_hostbatch.hpp).
#include "sfmm_hostbatch.hpp"

#include <algorithm>
#include <cstring>

namespace sfmm {

namespace {

inline size_t lo_of(size_t n, size_t t, size_t nthr) { return share_lo(n, t, nthr); }

// relaxed atomic max of a 32-bit counter
inline void atomic_max(uint32_t *p, uint32_t v)
{
    uint32_t old = __atomic_load_n(p, __ATOMIC_RELAXED);
    while (old < v && !__atomic_compare_exchange_n(p, &old, v, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
    }
}

inline size_t hash_slot(unsigned long long k, size_t mask)
{
    return (size_t)(((k >> 3) * 0x9E3779B97F4A7C15ull) >> 20) & mask;
}

inline double shift_of(const ClassicInput &in, const void *a, size_t i)
{
    return in.f64 ? static_cast<const double *>(a)[i] : (double)static_cast<const float *>(a)[i];
}

}  // namespace

size_t host_threads(size_t work)
{
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    return std::min<size_t>(std::min<size_t>(hw, 16), work / 32768 + 1);
}

ClassicScan classic_scan(const ClassicInput &in, size_t nthr)
{
    nthr = std::max<size_t>(nthr, 1);
    struct Part {
        size_t entries = 0, pmax = 1, bad = SIZE_MAX;
        int kind = 0;
    };
    std::vector<Part> part(nthr);
    fork_join(nthr, [&](size_t t) {
        Part r;
        const size_t hi = lo_of(in.n, t + 1, nthr);
        for (size_t i = lo_of(in.n, t, nthr); i < hi; ++i) {
            const size_t pi = in.p_in[i], po = in.p_out[i];
            if (pi > in.P || po > in.P) {
                r.bad = i;
                r.kind = 1;
                break;
            }
            if ((pi && !in.src[i]) || (po && !in.dst[i])) {
                r.bad = i;
                r.kind = 2;
                break;
            }
            r.pmax = std::max(r.pmax, std::max(pi, po));
            if (pi && po) r.entries += in.dim;
        }
        part[t] = r;
    });
    ClassicScan sc;
    sc.per_thread.resize(nthr);
    for (size_t t = 0; t < nthr; ++t) {
        if (part[t].bad != SIZE_MAX && sc.bad == SIZE_MAX) {  // the lowest share with an error holds the first
            sc.bad = part[t].bad;
            sc.bad_kind = part[t].kind;
        }
        sc.entries += part[t].entries;
        sc.pmax = std::max(sc.pmax, part[t].pmax);
        sc.per_thread[t] = part[t].entries;
    }
    return sc;
}

size_t classic_fill(const ClassicInput &in, const ClassicScan &sc, const ClassicEntries &out, SlotScratch &scratch,
                    bool *repeat, SlotPath *path)
{
    const size_t nthr = sc.per_thread.size();
    const size_t M = sc.entries;
    const size_t es = in.f64 ? 8 : 4;
    std::vector<size_t> base(nthr + 1, 0);
    for (size_t t = 0; t < nthr; ++t) base[t + 1] = base[t] + sc.per_thread[t];

    // 1. entries, and the order of the target addresses in each share
    struct Order {
        bool any = false, nondecr = true, strict = true;
        unsigned long long first = 0, last = 0;
    };
    std::vector<Order> ord(nthr);
    fork_join(nthr, [&](size_t t) {
        Order o;
        size_t e = base[t];
        const size_t hi = lo_of(in.n, t + 1, nthr);
        for (size_t i = lo_of(in.n, t, nthr); i < hi; ++i) {
            const size_t pi = in.p_in[i], po = in.p_out[i];
            if (!pi || !po) continue;
            const size_t cbi = pi * (pi + 1) * es, cbo = po * (po + 1) * es;  // bytes per component
            const double sx = shift_of(in, in.x, i), sy = shift_of(in, in.y, i), sz = shift_of(in, in.z, i);
            const unsigned long long s0 = (unsigned long long)(uintptr_t)in.src[i];
            const unsigned long long d0 = (unsigned long long)(uintptr_t)in.dst[i];
            for (size_t d = 0; d < in.dim; ++d, ++e) {
                const unsigned long long tp = d0 + d * cbo;
                out.sptr[e] = s0 + d * cbi;
                out.dptr[e] = tp;
                out.pin[e] = (uint32_t)pi;
                out.pout[e] = (uint32_t)po;
                out.shift[3 * e] = sx;
                out.shift[3 * e + 1] = sy;
                out.shift[3 * e + 2] = sz;
                if (o.any) {
                    o.nondecr = o.nondecr && tp >= o.last;
                    o.strict = o.strict && tp > o.last;
                } else {
                    o.first = tp;
                    o.any = true;
                }
                o.last = tp;
            }
        }
        ord[t] = o;
    });
    bool nondecr = true, strict = true, any = false;
    unsigned long long prev = 0;
    for (const Order &o : ord) {
        if (!o.any) continue;
        nondecr = nondecr && o.nondecr && (!any || o.first >= prev);
        strict = strict && o.strict && (!any || o.first > prev);
        prev = o.last;
        any = true;
    }

    // entry shares for the passes below
    auto elo = [&](size_t t) { return lo_of(M, t, nthr); };
    auto identity_slots = [&]() {
        fork_join(nthr, [&](size_t t) {
            for (size_t e = elo(t); e < elo(t + 1); ++e) {
                out.tidx[e] = (uint32_t)e;
                out.tptr[e] = out.dptr[e];
                out.tcnt[e] = out.pout[e] * (out.pout[e] + 1);
            }
        });
        *repeat = false;
        return M;
    };

    // 2a. rising addresses: every target is distinct, slot = entry
    if (strict) {
        if (path) *path = SlotPath::ascending;
        return identity_slots();
    }

    // 2b. non-decreasing addresses: a slot per run of equal addresses
    if (nondecr) {
        if (path) *path = SlotPath::runs;
        std::vector<size_t> starts(nthr, 0), sbase(nthr + 1, 0);
        fork_join(nthr, [&](size_t t) {
            size_t c = 0;
            for (size_t e = elo(t); e < elo(t + 1); ++e) c += (e == 0 || out.dptr[e] != out.dptr[e - 1]);
            starts[t] = c;
        });
        for (size_t t = 0; t < nthr; ++t) sbase[t + 1] = sbase[t] + starts[t];
        const size_t nt = sbase[nthr];
        fork_join(nthr, [&](size_t t) {
            const size_t lo = lo_of(nt, t, nthr), hi = lo_of(nt, t + 1, nthr);
            if (hi > lo) std::memset(out.tcnt + lo, 0, (hi - lo) * sizeof(uint32_t));
        });
        fork_join(nthr, [&](size_t t) {
            size_t s = sbase[t] - 1;  // slot of the entry before this share (wraps for t = 0, set at e = 0)
            for (size_t e = elo(t); e < elo(t + 1); ++e) {
                if (e == 0 || out.dptr[e] != out.dptr[e - 1]) {
                    ++s;
                    out.tptr[s] = out.dptr[e];
                }
                out.tidx[e] = (uint32_t)s;
                // a run may continue into the next share: counts merge by atomic maximum
                atomic_max(out.tcnt + s, out.pout[e] * (out.pout[e] + 1));
            }
        });
        *repeat = nt < M;
        return nt;
    }

    // 2c. any other order: concurrent open addressing (linear probing) over the
    //     target addresses, at most half full
    if (path) *path = SlotPath::hashed;
    size_t cap = 64;
    while (cap < 2 * M) cap <<= 1;
    if (scratch.cap < cap) {
        scratch.key.reset();
        scratch.cnt.reset();
        scratch.cap = 0;
        scratch.key.reset(new unsigned long long[cap]);
        scratch.cnt.reset(new uint32_t[cap]);
        scratch.cap = cap;
    }
    unsigned long long *key = scratch.key.get();
    uint32_t *cnt = scratch.cnt.get();
    const size_t mask = cap - 1;
    fork_join(nthr, [&](size_t t) {
        const size_t lo = lo_of(cap, t, nthr), hi = lo_of(cap, t + 1, nthr);
        std::memset(key + lo, 0, (hi - lo) * sizeof(unsigned long long));
        std::memset(cnt + lo, 0, (hi - lo) * sizeof(uint32_t));
    });
    std::vector<char> rep(nthr, 0);
    fork_join(nthr, [&](size_t t) {
        bool r = false;
        for (size_t e = elo(t); e < elo(t + 1); ++e) {
            const unsigned long long k = out.dptr[e];  // non-zero: entries have a target
            size_t h = hash_slot(k, mask);
            for (;;) {
                unsigned long long cur = __atomic_load_n(key + h, __ATOMIC_RELAXED);
                if (cur == 0) {
                    unsigned long long expect = 0;
                    if (__atomic_compare_exchange_n(key + h, &expect, k, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED))
                        break;
                    cur = expect;
                }
                if (cur == k) {
                    r = true;
                    break;
                }
                h = (h + 1) & mask;
            }
            out.tidx[e] = (uint32_t)h;  // table position for now
            atomic_max(cnt + h, out.pout[e] * (out.pout[e] + 1));
        }
        rep[t] = r;
    });
    if (std::find(rep.begin(), rep.end(), 1) == rep.end()) return identity_slots();
    // slots in table order: rank of each occupied position
    std::vector<size_t> occ(nthr, 0), obase(nthr + 1, 0);
    fork_join(nthr, [&](size_t t) {
        size_t c = 0;
        for (size_t h = lo_of(cap, t, nthr); h < lo_of(cap, t + 1, nthr); ++h) c += key[h] != 0;
        occ[t] = c;
    });
    for (size_t t = 0; t < nthr; ++t) obase[t + 1] = obase[t] + occ[t];
    fork_join(nthr, [&](size_t t) {
        size_t r = obase[t];
        for (size_t h = lo_of(cap, t, nthr); h < lo_of(cap, t + 1, nthr); ++h)
            if (key[h]) {
                out.tptr[r] = key[h];
                out.tcnt[r] = cnt[h];
                cnt[h] = (uint32_t)r;  // position -> slot
                ++r;
            }
    });
    fork_join(nthr, [&](size_t t) {
        for (size_t e = elo(t); e < elo(t + 1); ++e) out.tidx[e] = cnt[out.tidx[e]];
    });
    *repeat = true;
    return obase[nthr];
}

}  // namespace sfmm
