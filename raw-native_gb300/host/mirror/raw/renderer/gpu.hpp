#pragma once
// The GPU renderer's entry points (raw/renderer/gpu.hpp:22-33).
#include "raw/renderer/gpu_reconcile.hpp"
#include "raw/renderer/render.hpp"
#include <string>
namespace raw {
bool gpuCompiled();
const char* gpuBackendName();
bool gpuInit(GpuAdapterInfo& info, std::string& err);
bool renderGpu(const Scene& scene, int w, int h, const Mat4& prevViewProj, const RenderOptions& opts,
               FrameResult& out, std::string& err, bool frameOnly = false);
}  // namespace raw
