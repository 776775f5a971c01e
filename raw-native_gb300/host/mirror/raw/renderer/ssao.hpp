#pragma once
// The screen-space AO entry point (raw/renderer/ssao.hpp).
#include "raw/renderer/gbuffer.hpp"
namespace raw {
Buffer<float> computeSSAO(const GBuffer& g, int samples, float radius, Arena* arena = nullptr, int threads = 1);
}  // namespace raw
