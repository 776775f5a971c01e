#pragma once
// The ray-traced AO entry points (raw/renderer/ray_ao.hpp).
#include "raw/renderer/accel.hpp"
#include "raw/renderer/gbuffer.hpp"
namespace raw {
Buffer<float> computeRTAO(const GBuffer& g, const LinearAccel& accel, int samples, float radius,
                          Arena* arena = nullptr, int threads = 1);
void computeRTVisibility(const GBuffer& g, const LinearAccel& accel, int samples, float radius, Vec3 toLight,
                         Buffer<float>& ao, Buffer<float>& sky, Buffer<float>& sun, int threads = 1,
                         bool sunForced = false);
}  // namespace raw
