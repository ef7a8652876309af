// mrg8g_arena.h -- the serving output arena (host-side bookkeeping only).
//
// Header-only so that the CPU tests can drive it without a GPU
// (tests/native/check_arena.cpp).
#pragma once
#include <cstdint>
#include <deque>

namespace mrg8g {

// First-in first-out arena over [0, cap): blocks are handed out in admission
// order and reclaimed from the oldest once released (out-of-order releases
// wait for the older ones).  256-byte granularity.  Every block (and every
// padding block left at the end when the ring wraps) gets the next sequence
// number, so a release finds its block in O(1).
class Arena {
public:
    explicit Arena(uint64_t cap) : cap_(cap) {}
    bool alloc(uint64_t bytes, uint64_t* off, uint64_t* seq) {
        bytes = bytes ? (bytes + 255) / 256 * 256 : 256;
        if (bytes > cap_) return false;
        if (blocks_.empty()) head_ = tail_ = 0;
        // Live blocks occupy [tail, head) or, once wrapped, [tail, cap) + [0, head).
        const bool wrapped = !blocks_.empty() && head_ <= tail_;
        uint64_t at;
        if (!wrapped) {
            if (cap_ - head_ >= bytes) {
                at = head_;
            } else if (tail_ >= bytes) {
                if (head_ < cap_) blocks_.push_back({head_, cap_ - head_, true});  // unused end
                at = 0;
            } else {
                return false;
            }
        } else if (tail_ - head_ >= bytes) {
            at = head_;
        } else {
            return false;
        }
        *seq = base_seq_ + blocks_.size();
        blocks_.push_back({at, bytes, false});
        head_ = at + bytes;
        used_ += bytes;
        *off = at;
        return true;
    }
    void release(uint64_t seq) {
        if (seq < base_seq_ || seq - base_seq_ >= blocks_.size()) return;
        Block& b = blocks_[seq - base_seq_];
        if (b.released) return;
        b.released = true;
        used_ -= b.size;
        while (!blocks_.empty() && blocks_.front().released) {
            blocks_.pop_front();
            ++base_seq_;
        }
        if (blocks_.empty()) head_ = tail_ = 0;
        else tail_ = blocks_.front().off;
    }
    uint64_t used() const { return used_; }

private:
    struct Block {
        uint64_t off, size;
        bool released;
    };
    uint64_t cap_, head_ = 0, tail_ = 0, used_ = 0, base_seq_ = 0;
    std::deque<Block> blocks_;
};

}  // namespace mrg8g
