#pragma once
// The occlusion accelerator's public face (raw/renderer/accel.hpp): the triangle list and
// the test mode the AO passes read.
#include "raw/core/arena_allocator.hpp"
#include "raw/math/primitives.hpp"
#include <vector>
namespace raw {
struct LinearAccel {
    std::vector<Tri, ArenaAllocator<Tri>> tris;
    enum class Mode : unsigned char { Bvh, Scan, Skew };
    Mode mode{Mode::Bvh};
};
}  // namespace raw
