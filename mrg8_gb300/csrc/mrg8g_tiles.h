// mrg8g_tiles.h -- how a batch cuts its instances into tiles.
//
// Header-only, so that the batch kernel (derive_tile), the host planner
// (make_tiles, tile_prefix, ...) and the CPU tests
// (tests/native/check_tiles.cpp) share one definition.  Every instance is cut
// into an unaligned head (the outputs before the first 16-byte boundary of its
// buffer, fewer than one 16-byte vector, written by one lane) and body tiles
// of tile_elems outputs (the last one shorter); body tiles therefore start on
// 16-byte boundaries.
#pragma once
#include <stdint.h>

#include "mrg8g_internal.h"

#if !defined(__CUDA_ARCH__)
#include <algorithm>
#include <vector>
#endif

namespace mrg8g {

// Bytes per output of a kind (fp64 kinds 8, the others 4).
MRG8G_HDC inline uint32_t tile_elem_bytes(int32_t kind) { return (kind == 1 || kind == 2) ? 8u : 4u; }

// Outputs before the first 16-byte boundary of the instance's buffer.
MRG8G_HDC inline uint64_t head_outputs(const BatchInst& in) {
    const uint32_t elem = tile_elem_bytes(in.kind);
    const uint64_t head = ((16u - (uint32_t)((uintptr_t)in.out & 15u)) & 15u) / elem;
    return head < in.n ? head : in.n;
}

// Tiles of one instance with body tiles of tile_elems outputs.
MRG8G_HDC inline uint64_t instance_tiles(const BatchInst& in, uint64_t tile_elems) {
    if (!in.n) return 0;
    const uint64_t head = head_outputs(in);
    return (head ? 1 : 0) + (in.n - head + tile_elems - 1) / tile_elems;
}

// Tile li (0-based within instance i) of a device-tiled launch.
MRG8G_HDC inline BatchTile derive_tile(uint32_t li, const BatchInst& in, uint32_t i, uint32_t tile_elems) {
    const uint64_t head = head_outputs(in);
    BatchTile t;
    t.inst = i;
    if (head && li == 0) {
        t.start = 0;
        t.len_flags = (uint32_t)head | kTileHead;
    } else {
        t.start = head + (uint64_t)(li - (head ? 1u : 0u)) * tile_elems;
        const uint64_t left = in.n - t.start;
        t.len_flags = (uint32_t)(left < tile_elems ? left : tile_elems);
    }
    return t;
}

#if !defined(__CUDA_ARCH__)

// Host-listed tiles of every instance with body tiles of tile_elems outputs,
// ordered by bytes, largest first, so the dynamic queue ends with the
// smallest pieces.
inline void make_tiles(const BatchInst* insts, uint32_t count, uint64_t tile_elems, std::vector<BatchTile>& tiles) {
    tiles.clear();
    for (uint32_t i = 0; i < count; ++i) {
        const uint64_t k = instance_tiles(insts[i], tile_elems);
        for (uint64_t li = 0; li < k; ++li) tiles.push_back(derive_tile((uint32_t)li, insts[i], i, (uint32_t)tile_elems));
    }
    std::stable_sort(tiles.begin(), tiles.end(), [&](const BatchTile& x, const BatchTile& y) {
        const uint64_t bx = (uint64_t)(x.len_flags & ~kTileHead) * tile_elem_bytes(insts[x.inst].kind);
        const uint64_t by = (uint64_t)(y.len_flags & ~kTileHead) * tile_elem_bytes(insts[y.inst].kind);
        return bx > by;
    });
}

// Instances ordered by bytes, largest first (the derived tiling's order).
inline void sort_largest_first(BatchInst* insts, uint32_t count) {
    std::stable_sort(insts, insts + count, [](const BatchInst& x, const BatchInst& y) {
        return x.n * tile_elem_bytes(x.kind) > y.n * tile_elem_bytes(y.kind);
    });
}

// Tiles of a plan (both tilings cut the instances the same way), counted
// without building them.
inline uint64_t count_tiles(const BatchInst* insts, uint32_t count, uint64_t tile_elems) {
    uint64_t total = 0;
    for (uint32_t i = 0; i < count; ++i) total += instance_tiles(insts[i], tile_elems);
    return total;
}

// base[i] = first tile of instance i, base[count] = the total (the return
// value, in 64 bits so that callers can reject a total above 2^32 - 1).
inline uint64_t tile_prefix(const BatchInst* insts, uint32_t count, uint64_t tile_elems, uint32_t* base) {
    uint64_t total = 0;
    for (uint32_t i = 0; i < count; ++i) {
        base[i] = (uint32_t)total;
        total += instance_tiles(insts[i], tile_elems);
    }
    base[count] = (uint32_t)total;
    return total;
}

#endif

}  // namespace mrg8g
