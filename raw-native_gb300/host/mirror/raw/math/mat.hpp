#pragma once
// The 4x4 matrix of raw-native's math layer (raw/math/mat.hpp): row-major, element (r, c)
// at m[r * 4 + c]. Only the type and the projection helpers the camera declares.
#include "raw/math/vec.hpp"
namespace raw {
struct Mat4 { float m[16]{}; };
Mat4 perspective(float fovy, float aspect, float n, float f);
Mat4 lookAt(Vec3 eye, Vec3 center, Vec3 up);
}  // namespace raw
