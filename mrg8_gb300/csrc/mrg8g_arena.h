// mrg8g_arena.h -- the serving output arena (host-side bookkeeping only).
//
// Header-only so that the CPU tests can drive it without a GPU
// (tests/native/check_arena.cpp).
#pragma once
#include <cstdint>
#include <iterator>
#include <map>
#include <unordered_map>

namespace mrg8g {

// First-fit arena over [0, cap) at 256-byte granularity.  Free space is kept
// as address-ordered ranges that are merged with their neighbours on release,
// so a request fits whenever some free range is large enough, whatever order
// the results are released in.  (A first-in first-out ring cannot reuse the
// space of a released block while an older one is still held; a client that
// kept its oldest result while waiting for newer ones could then wait
// forever.)  Every block gets a fresh sequence number, its release handle, so
// a repeated or stale release is ignored.
class Arena {
public:
    explicit Arena(uint64_t cap) : cap_(cap) {
        if (cap_) free_[0] = cap_;
    }
    bool alloc(uint64_t bytes, uint64_t* off, uint64_t* seq) {
        bytes = bytes ? (bytes + 255) / 256 * 256 : 256;
        if (bytes > cap_) return false;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            const uint64_t at = it->first, rest = it->second - bytes;
            free_.erase(it);
            if (rest) free_[at + bytes] = rest;
            *off = at;
            *seq = next_seq_++;
            live_[*seq] = Block{at, bytes};
            used_ += bytes;
            return true;
        }
        return false;
    }
    void release(uint64_t seq) {
        auto it = live_.find(seq);
        if (it == live_.end()) return;
        uint64_t at = it->second.off, size = it->second.size;
        live_.erase(it);
        used_ -= size;
        auto next = free_.lower_bound(at);
        if (next != free_.end() && at + size == next->first) {
            size += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == at) {
                prev->second += size;
                return;
            }
        }
        free_[at] = size;
    }
    uint64_t used() const { return used_; }
    // Largest free range (merged ranges: equals the largest gap between live blocks).
    uint64_t largest_free() const {
        uint64_t m = 0;
        for (const auto& f : free_) m = f.second > m ? f.second : m;
        return m;
    }

private:
    struct Block {
        uint64_t off, size;
    };
    uint64_t cap_, used_ = 0, next_seq_ = 0;
    std::map<uint64_t, uint64_t> free_;           // offset -> length
    std::unordered_map<uint64_t, Block> live_;    // sequence number -> block
};

}  // namespace mrg8g
