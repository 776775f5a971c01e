#pragma once
// Row-major pixel buffer of raw-native's core layer (raw/core/image.hpp).
#include "raw/core/arena_allocator.hpp"
#include "raw/math/vec.hpp"
#include <cstddef>
#include <cstdint>
#include <vector>
namespace raw {
template <class T> struct Buffer {
    int w{0}, h{0};
    std::vector<T, ArenaAllocator<T>> px;
    Buffer() = default;
    explicit Buffer(Arena* a) : px(ArenaAllocator<T>(a)) {}
    void resize(int W, int H) { w = W; h = H; px.assign((std::size_t)W * H, T{}); }
    T& at(int x, int y) { return px[(std::size_t)y * w + x]; }
    const T& at(int x, int y) const { return px[(std::size_t)y * w + x]; }
};
}  // namespace raw
