// First-fit range allocator over one contiguous block of bytes (host-side
// bookkeeping only). The serving engine carves each request's device region
// (mesh tables, field state and RK registers) out of one device allocation made
// when the server starts, so admitting and retiring requests never calls
// cudaMalloc/cudaFree (which would synchronise the device while other requests'
// kernels are running).
//
// Free ranges are kept sorted by offset and merged with their neighbours on
// release, so a retired region becomes available again as one piece.
#pragma once
#include <cstdint>
#include <iterator>
#include <map>
#include <stdexcept>

namespace dgtd {

class RangeAllocator {
public:
    RangeAllocator() = default;
    RangeAllocator(int64_t capacity, int64_t align) { reset(capacity, align); }

    void reset(int64_t capacity, int64_t align)
    {
        if (capacity < 0 || align <= 0 || (align & (align - 1)) != 0)
            throw std::invalid_argument("RangeAllocator: bad capacity or alignment");
        capacity_ = capacity;
        align_ = align;
        free_.clear();
        used_.clear();
        in_use_ = 0;
        if (capacity > 0) free_[0] = capacity;
    }

    int64_t round_up(int64_t bytes) const { return (bytes + align_ - 1) / align_ * align_; }

    // Offset of a new range of at least `bytes`, or -1 when no free range is large enough.
    int64_t alloc(int64_t bytes)
    {
        if (bytes <= 0) return -1;
        const int64_t need = round_up(bytes);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < need) continue;
            const int64_t off = it->first, len = it->second;
            free_.erase(it);
            if (len > need) free_[off + need] = len - need;
            used_[off] = need;
            in_use_ += need;
            return off;
        }
        return -1;
    }

    // Release a range returned by alloc(); false if `off` is not an allocated range.
    bool release(int64_t off)
    {
        auto u = used_.find(off);
        if (u == used_.end()) return false;
        int64_t start = off, len = u->second;
        in_use_ -= len;
        used_.erase(u);
        auto next = free_.lower_bound(start);
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == start) {
                start = prev->first;
                len += prev->second;
                free_.erase(prev);
            }
        }
        next = free_.lower_bound(start);
        if (next != free_.end() && start + len == next->first) {
            len += next->second;
            free_.erase(next);
        }
        free_[start] = len;
        return true;
    }

    int64_t capacity() const { return capacity_; }
    int64_t in_use() const { return in_use_; }
    int64_t largest_free() const
    {
        int64_t m = 0;
        for (const auto& f : free_) m = f.second > m ? f.second : m;
        return m;
    }
    int64_t n_free_ranges() const { return static_cast<int64_t>(free_.size()); }
    int64_t n_used_ranges() const { return static_cast<int64_t>(used_.size()); }

private:
    int64_t capacity_ = 0, align_ = 256, in_use_ = 0;
    std::map<int64_t, int64_t> free_;   // offset -> length
    std::map<int64_t, int64_t> used_;   // offset -> length
};

}  // namespace dgtd
