// check_arena.cpp -- CPU property check of the serving output arena.
//
// Built by tests/test_arena.py with g++ against mrg8_gb300/csrc/mrg8g_arena.h.
// Random admissions and out-of-order releases (a FIFO window of live requests
// released in shuffled order, as completions and client releases interleave)
// against an independent model: every block lies in [0, cap) on a 256-byte
// boundary, no two live blocks overlap, used() is the sum of the live sizes,
// a request is refused only when no gap between the live blocks can hold it
// (so holding an old block never strands the space released after it), an
// empty arena takes a request of any size up to cap, and releasing everything
// returns the arena to empty.  Also the pattern of a client that keeps its
// oldest result while later ones are released.  Prints "ok <allocations>".
#include <algorithm>
#include <cstdio>
#include <cstdint>
#include <random>
#include <vector>

#include "mrg8g_arena.h"

struct Live {
    uint64_t seq, off, size;
};

static int fail(const char* what, unsigned long long a, unsigned long long b) {
    std::printf("FAIL %s %llu %llu\n", what, a, b);
    return 1;
}

// Largest gap between the live blocks (model side).
static uint64_t largest_gap(std::vector<Live> live, uint64_t cap) {
    std::sort(live.begin(), live.end(), [](const Live& x, const Live& y) { return x.off < y.off; });
    uint64_t at = 0, best = 0;
    for (const Live& l : live) {
        best = std::max(best, l.off - at);
        at = l.off + l.size;
    }
    return std::max(best, cap - at);
}

int main() {
    std::mt19937_64 rng(12345);
    unsigned long long allocations = 0;
    for (int round = 0; round < 40; ++round) {
        const uint64_t cap = (uint64_t)(1 + rng() % 64) << (12 + round % 12);
        mrg8g::Arena a(cap);
        std::vector<Live> live;
        uint64_t used = 0;
        const int window = 1 + (int)(rng() % 200);
        for (int step = 0; step < 20000; ++step) {
            const bool do_alloc = live.size() < (size_t)window && (rng() % 3 != 0);
            if (do_alloc) {
                const uint64_t want = rng() % 5 == 0 ? 0 : 1 + rng() % std::max<uint64_t>(1, cap / (1 + rng() % 16));
                uint64_t off = 0, seq = 0;
                if (!a.alloc(want, &off, &seq)) {
                    if (live.empty() && want <= cap) return fail("empty arena refused", want, cap);
                    const uint64_t need = want ? (want + 255) / 256 * 256 : 256;
                    if (need <= cap && largest_gap(live, cap) >= need) return fail("refused with a gap", need, largest_gap(live, cap));
                    continue;
                }
                ++allocations;
                const uint64_t size = want ? (want + 255) / 256 * 256 : 256;
                if (off % 256 || off + size > cap) return fail("block outside the arena", off, size);
                for (const Live& l : live)
                    if (off < l.off + l.size && l.off < off + size) return fail("overlap", off, l.off);
                live.push_back({seq, off, size});
                used += size;
            } else if (!live.empty()) {
                // release one of the oldest few, so releases come out of order
                const size_t k = rng() % std::min<size_t>(live.size(), 8);
                a.release(live[k].seq);
                a.release(live[k].seq);  // a second release is ignored
                used -= live[k].size;
                live.erase(live.begin() + (long)k);
            }
            if (a.used() != used) return fail("used", a.used(), used);
            if (a.largest_free() != largest_gap(live, cap)) return fail("largest free range", a.largest_free(), largest_gap(live, cap));
        }
        std::shuffle(live.begin(), live.end(), rng);
        for (const Live& l : live) a.release(l.seq);
        if (a.used() != 0) return fail("not empty after releasing all", a.used(), 0);
        uint64_t off = 1, seq = 0;
        if (!a.alloc(cap, &off, &seq) || off != 0) return fail("full-size request after emptying", off, cap);
    }
    {   // two results fit at a time; the client holds the older while the newer is released
        const uint64_t blk = 1398272, cap = 4u << 20;
        mrg8g::Arena a(cap);
        uint64_t o0, s0, o1, s1, o2, s2;
        if (!a.alloc(blk, &o0, &s0) || !a.alloc(blk, &o1, &s1)) return fail("two blocks", 0, 0);
        uint64_t ox, sx;
        if (a.alloc(blk, &ox, &sx)) return fail("third block fit", ox, cap);
        a.release(s1);  // the newer first
        if (!a.alloc(blk, &o2, &s2) || o2 != o1) return fail("released space not reused", o2, o1);
        ++allocations;
    }
    std::printf("ok %llu\n", allocations);
    return 0;
}
