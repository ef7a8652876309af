// check_tiles.cpp -- CPU property check of how batches cut instances into
// tiles (mrg8_gb300/csrc/mrg8g_tiles.h), the same functions the batch kernel
// (derive_tile) and the host planner use.
//
// Built by tests/test_tiles.py with g++.  Random instances (every kind,
// lengths 0 .. 2^22, buffers at every element offset within 16 bytes) and
// several tile sizes: the listed tiles of make_tiles cover every instance
// exactly once ([0, n), no gaps, no overlap), a head tile (flagged) holds
// exactly the outputs before the buffer's first 16-byte boundary, every body
// tile starts on a 16-byte boundary and is full but for the instance's last;
// the list is ordered by bytes, largest first; count_tiles agrees; and the
// derived tiling (instances longest first, tile_prefix counts, derive_tile of
// each local index) produces the same tiles per instance.  Prints "ok <tiles>".
#include <cstdio>
#include <map>
#include <random>
#include <tuple>
#include <vector>

#include "mrg8g_tiles.h"

using namespace mrg8g;

static int fail(const char* what, unsigned long long a, unsigned long long b) {
    std::printf("FAIL %s %llu %llu\n", what, a, b);
    return 1;
}

using TileKey = std::tuple<uint64_t, uint32_t, bool>;  // start, length, head flag

int main() {
    std::mt19937_64 rng(2024);
    unsigned long long checked = 0;
    for (int round = 0; round < 60; ++round) {
        const uint32_t count = 1 + (uint32_t)(rng() % 300);
        std::vector<BatchInst> insts(count);
        for (uint32_t i = 0; i < count; ++i) {
            BatchInst& in = insts[i];
            in.kind = (int32_t)(rng() % 5);
            const uint32_t elem = tile_elem_bytes(in.kind);
            const int r = (int)(rng() % 10);
            in.n = r == 0 ? 0 : r == 1 ? rng() % 8 : (uint64_t)(1ull << (rng() % 23)) + rng() % 1000;
            in.out = reinterpret_cast<void*>((uintptr_t)0x7f0000000000ull + 4096 * (rng() % 1000) + elem * (rng() % (16 / elem)));
            in.offset = 0;
            in.slot1 = 0;
        }
        const uint64_t rows[] = {16, 24, 512, 2048};
        const uint64_t T = rows[round % 4] * 32 * 2;
        std::vector<BatchTile> tiles;
        make_tiles(insts.data(), count, T, tiles);
        if (tiles.size() != count_tiles(insts.data(), count, T)) return fail("count_tiles", tiles.size(), count_tiles(insts.data(), count, T));
        std::vector<std::map<uint64_t, TileKey>> per(count);
        uint64_t prev_bytes = ~0ull;
        for (const BatchTile& t : tiles) {
            const BatchInst& in = insts[t.inst];
            const uint32_t elem = tile_elem_bytes(in.kind);
            const bool head = (t.len_flags & kTileHead) != 0;
            const uint32_t len = t.len_flags & ~kTileHead;
            const uint64_t bytes = (uint64_t)len * elem;
            if (bytes > prev_bytes) return fail("order", bytes, prev_bytes);
            prev_bytes = bytes;
            if (!len) return fail("empty tile", t.inst, t.start);
            if (!per[t.inst].emplace(t.start, TileKey{t.start, len, head}).second) return fail("duplicate start", t.inst, t.start);
        }
        for (uint32_t i = 0; i < count; ++i) {
            const BatchInst& in = insts[i];
            const uint32_t elem = tile_elem_bytes(in.kind);
            const uintptr_t addr = reinterpret_cast<uintptr_t>(in.out);
            const uint64_t head_want = std::min<uint64_t>(((16 - addr % 16) % 16) / elem, in.n);
            uint64_t at = 0;
            size_t k = 0;
            for (const auto& kv : per[i]) {
                const uint64_t start = std::get<0>(kv.second);
                const uint32_t len = std::get<1>(kv.second);
                const bool head = std::get<2>(kv.second);
                if (start != at) return fail("gap or overlap", i, start);
                if (k == 0 && head_want) {
                    if (!head || len != head_want) return fail("head tile", i, len);
                } else {
                    if (head) return fail("stray head flag", i, start);
                    if ((addr + start * elem) % 16) return fail("body tile not on a 16-byte boundary", i, start);
                    if (len != T && start + len != in.n) return fail("short body tile before the end", i, start);
                }
                at = start + len;
                ++k;
            }
            if (at != in.n) return fail("instance not covered", i, at);
            checked += k;
        }
        // The derived tiling: longest first, prefix counts, one tile per local index.
        std::vector<BatchInst> sorted(insts);
        sort_largest_first(sorted.data(), count);
        for (uint32_t i = 1; i < count; ++i)
            if (sorted[i].n * tile_elem_bytes(sorted[i].kind) > sorted[i - 1].n * tile_elem_bytes(sorted[i - 1].kind))
                return fail("longest first", i, 0);
        std::vector<uint32_t> base(count + 1);
        const uint64_t total = tile_prefix(sorted.data(), count, T, base.data());
        if (total != tiles.size() || base[count] != total) return fail("tile_prefix total", total, tiles.size());
        std::vector<BatchTile> mine;
        for (uint32_t i = 0; i < count; ++i) {
            std::vector<BatchTile> want;
            make_tiles(&sorted[i], 1, T, want);
            if (base[i + 1] - base[i] != want.size()) return fail("prefix count", i, want.size());
            std::map<uint64_t, TileKey> a, b;
            for (const BatchTile& t : want) a.emplace(t.start, TileKey{t.start, t.len_flags & ~kTileHead, (t.len_flags & kTileHead) != 0});
            for (uint32_t li = 0; li < base[i + 1] - base[i]; ++li) {
                const BatchTile t = derive_tile(li, sorted[i], i, (uint32_t)T);
                if (t.inst != i) return fail("derived tile owner", i, t.inst);
                b.emplace(t.start, TileKey{t.start, t.len_flags & ~kTileHead, (t.len_flags & kTileHead) != 0});
            }
            if (a != b) return fail("derived tiles differ", i, b.size());
        }
    }
    std::printf("ok %llu\n", checked);
    return 0;
}
