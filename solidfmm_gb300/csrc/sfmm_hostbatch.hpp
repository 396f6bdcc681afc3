// Host bookkeeping of the classic translation call: arrays of source and
// target solid addresses with per-translation orders and shifts, as the
// reference's m2l/m2m/l2l(op, buf, howmany, M**, L**, x, y, z) overloads and
// multithreaded_translator ranges pass them (translations.hpp:103-170,
// translations.cpp:743-755 for dim > 1).
//
// One entry per (translation, component) with work (a zero order adds
// nothing), in translation-major order, and one slot per distinct target
// address.  Built on the host cores in parallel, straight into caller
// storage (the pinned staging of the kernel's metadata).  Target addresses
// that rise strictly need no deduplication; non-decreasing ones (batches
// sorted by target) form runs; any other order goes through a concurrent
// open-addressing table.  No CUDA dependency: the CPU tests build this file
// on its own.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <thread>
#include <vector>

namespace sfmm {

// fn(t) for every share t in [0, nthr): share 0 on the calling thread, the
// others on new threads; shares whose thread cannot be created run on the
// calling thread, so this never throws on its own.
template <class F>
void fork_join(size_t nthr, F &&fn)
{
    std::vector<std::thread> th;
    size_t spawned = 1;
    if (nthr > 1) {
        try {
            th.reserve(nthr - 1);
            for (; spawned < nthr; ++spawned) th.emplace_back(fn, spawned);
        } catch (...) {
        }
    }
    fn(size_t(0));
    for (size_t t = spawned; t < nthr; ++t) fn(t);
    for (auto &x : th) x.join();
}

// first index of share t of n items split nthr ways
inline size_t share_lo(size_t n, size_t t, size_t nthr) { return n * t / nthr; }

struct ClassicInput {
    size_t n = 0;                      // translations
    const void *const *src = nullptr;  // source solid buffers
    const size_t *p_in = nullptr;      // source orders
    void *const *dst = nullptr;        // target solid buffers
    const size_t *p_out = nullptr;     // target orders
    size_t dim = 1;                    // components per solid
    const void *x = nullptr, *y = nullptr, *z = nullptr;  // shift, double (f64) or float
    bool f64 = true;                   // coefficient and shift type
    size_t P = 0;                      // operator order: larger orders are an error
};

struct ClassicScan {
    size_t entries = 0;               // (translation, component) pairs with work
    size_t pmax = 1;                  // largest order named
    size_t bad = SIZE_MAX;            // first invalid translation, SIZE_MAX if none
    int bad_kind = 0;                 // 1: order above P, 2: null solid pointer with work
    std::vector<size_t> per_thread;   // entries of each thread's share of translations
};

// Caller storage for the entries (capacity: entries) and slots (capacity:
// entries; the slot count is at most the entry count).
struct ClassicEntries {
    unsigned long long *sptr = nullptr, *dptr = nullptr;  // component addresses
    uint32_t *pin = nullptr, *pout = nullptr;             // orders
    uint32_t *tidx = nullptr;                             // slot of each entry
    double *shift = nullptr;                              // 3 per entry
    unsigned long long *tptr = nullptr;                   // target address of each slot
    uint32_t *tcnt = nullptr;                             // coefficients of each slot (largest order named)
};

// Target table kept between calls (grows to twice the largest batch).
struct SlotScratch {
    std::unique_ptr<unsigned long long[]> key;
    std::unique_ptr<uint32_t[]> cnt;
    size_t cap = 0;
};

// How the slots were found (for tests and diagnostics).
enum class SlotPath { ascending = 0, runs = 1, hashed = 2 };

// Threads for a batch of `work` entries: one for small batches, at most 16.
size_t host_threads(size_t work);

// Validate and count; the first invalid translation is reported the way a
// sequential scan finds it (order checked before pointers).
ClassicScan classic_scan(const ClassicInput &in, size_t nthr);

// Fill the entries and slots with the scan's threads; returns the slot
// count.  *repeat is whether a target address is named by more than one
// entry.  Throws std::bad_alloc (table growth).
size_t classic_fill(const ClassicInput &in, const ClassicScan &sc, const ClassicEntries &out, SlotScratch &scratch,
                    bool *repeat, SlotPath *path = nullptr);

}  // namespace sfmm
