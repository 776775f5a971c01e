// A fail-closed bump arena with raw::Arena's contract (zero-size and over-budget requests
// are refused and counted; nothing grows), for the shim's stand-alone build.
#include "raw/core/arena.hpp"
namespace raw {
Arena::Arena(void* base, std::size_t budget) : base_(static_cast<unsigned char*>(base)) {
    stats_.budget = base_ ? budget : 0;
}
void* Arena::allocate(std::size_t n, std::size_t align) {
    const std::size_t start = align ? (stats_.used + align - 1) / align * align : stats_.used;
    if (n == 0 || start > stats_.budget || n > stats_.budget - start) { ++stats_.refusals; return nullptr; }
    stats_.used = start + n;
    if (stats_.used > stats_.high_water) stats_.high_water = stats_.used;
    ++stats_.allocations;
    return base_ + start;
}
void Arena::reset() { stats_.used = 0; }
}  // namespace raw
