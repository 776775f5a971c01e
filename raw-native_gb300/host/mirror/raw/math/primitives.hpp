#pragma once
// Ray and triangle records of raw-native's math layer (raw/math/primitives.hpp).
#include "raw/math/vec.hpp"
namespace raw {
struct Ray { Vec3 o, d; };
struct Tri { Vec3 a, b, c; };
}  // namespace raw
