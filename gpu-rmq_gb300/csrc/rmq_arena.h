// rmq_arena.h — the server's device-memory arena bookkeeping (host only).
//
// One cudaMalloc of the HBM budget is carved into resident arrays by
// first-fit over a free list ordered by offset, in 256-byte granules; a
// released range merges with free neighbours on both sides.  No CUDA here:
// the offsets are byte offsets into the caller's allocation, so this file is
// also compiled into a CPU test.
#pragma once

#include <cstdint>
#include <iterator>
#include <map>

namespace rmq {

constexpr uint64_t kArenaGranule = 256;

inline uint64_t arena_round_up(uint64_t x) { return (x + kArenaGranule - 1) & ~(kArenaGranule - 1); }

class Arena {
public:
    void init(uint64_t size) {
        free_.clear();
        free_[0] = size;
    }
    // First free range (lowest offset) that holds `bytes` (rounded up to the
    // granule); false if none does.
    bool alloc(uint64_t bytes, uint64_t* off) {
        bytes = arena_round_up(bytes);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            const uint64_t o = it->first, rest = it->second - bytes;
            free_.erase(it);
            if (rest) free_[o + bytes] = rest;
            *off = o;
            return true;
        }
        return false;
    }
    // Returns [off, off + bytes) (the same bytes as its alloc) to the free list.
    void release(uint64_t off, uint64_t bytes) {
        bytes = arena_round_up(bytes);
        auto it = free_.emplace(off, bytes).first;
        auto next = std::next(it);
        if (next != free_.end() && off + bytes == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }
    // Free ranges (offset -> length), for inspection.
    const std::map<uint64_t, uint64_t>& free_ranges() const { return free_; }

private:
    std::map<uint64_t, uint64_t> free_;
};

// Eviction choice: the index of the least recently used array that may be
// evicted (resident, built, no batch in flight, and not `except`), or
// ~0 when none may.  Elements need `resident`, `ready`, `pins`, `last_use`.
template <typename Arrays>
uint64_t lru_victim(const Arrays& arrays, uint64_t except) {
    uint64_t victim = ~uint64_t(0), oldest = ~uint64_t(0);
    for (uint64_t i = 0; i < uint64_t(arrays.size()); ++i) {
        const auto& c = arrays[i];
        if (i != except && c.resident && c.ready && c.pins == 0 && c.last_use < oldest) {
            oldest = c.last_use;
            victim = i;
        }
    }
    return victim;
}

}  // namespace rmq
