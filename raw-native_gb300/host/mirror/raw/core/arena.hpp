#pragma once
// The fail-closed bump arena of raw-native's core layer (raw/core/arena.hpp): requests over
// the budget are refused (nullptr), never grown.
#include <cstddef>
namespace raw {
struct ArenaStats { std::size_t budget{0}, used{0}, high_water{0}, allocations{0}, refusals{0}; };
class Arena {
public:
    Arena(void* base, std::size_t budget);
    Arena(const Arena&) = delete;
    Arena& operator=(const Arena&) = delete;
    void* allocate(std::size_t n, std::size_t align = alignof(std::max_align_t));
    void reset();
    const ArenaStats& stats() const { return stats_; }
private:
    unsigned char* base_;
    ArenaStats stats_;
};
}  // namespace raw
