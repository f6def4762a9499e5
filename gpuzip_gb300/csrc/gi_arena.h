// gi_arena.h - the request server's input arena: a first-fit allocator of byte ranges.
//
// Host-only bookkeeping over [0, capacity) of one device buffer. Ranges are whole units of
// `align` bytes (4 KiB by default, so every request's input starts 16-byte aligned for the
// copies into a pass); freed ranges merge with free neighbours, so the arena never fragments
// into more free ranges than there are live ones plus one. Not thread-safe: the server holds
// its lock around every call.
#pragma once

#include <algorithm>
#include <cstdint>
#include <iterator>
#include <map>

namespace gz {

class Arena {
  public:
    static constexpr uint64_t NONE = ~0ull;

    explicit Arena(uint64_t capacity = 0, uint64_t align = 4096) { reset(capacity, align); }

    void reset(uint64_t capacity, uint64_t align) {
        align_ = align ? align : 1;
        cap_ = capacity / align_ * align_;
        free_.clear();
        if (cap_) free_[0] = cap_;
        used_ = peak_ = 0;
    }

    // offset of a range of n bytes, or NONE when no free range is large enough
    uint64_t alloc(uint64_t n) {
        n = units(n);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            const uint64_t off = it->first, len = it->second;
            free_.erase(it);
            if (len > n) free_[off + n] = len - n;
            used_ += n;
            peak_ = std::max(peak_, used_);
            return off;
        }
        return NONE;
    }

    // gives back a range that alloc(n) returned at off
    void release(uint64_t off, uint64_t n) {
        n = units(n);
        used_ -= n;
        auto next = free_.lower_bound(off);
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {  // merge with the range before
                off = prev->first;
                n += prev->second;
                free_.erase(prev);
            }
        }
        if (next != free_.end() && off + n == next->first) {  // and with the range after
            n += next->second;
            free_.erase(next);
        }
        free_[off] = n;
    }

    bool fits(uint64_t n) const { return largest_free() >= units(n); }
    uint64_t largest_free() const {
        uint64_t m = 0;
        for (const auto& f : free_) m = std::max(m, f.second);
        return m;
    }
    uint64_t capacity() const { return cap_; }
    uint64_t used() const { return used_; }
    uint64_t peak() const { return peak_; }
    size_t free_ranges() const { return free_.size(); }

  private:
    uint64_t units(uint64_t n) const { return std::max<uint64_t>(1, (n + align_ - 1) / align_) * align_; }
    uint64_t cap_ = 0, align_ = 4096, used_ = 0, peak_ = 0;
    std::map<uint64_t, uint64_t> free_;  // offset -> length, disjoint, never adjacent
};

}  // namespace gz
