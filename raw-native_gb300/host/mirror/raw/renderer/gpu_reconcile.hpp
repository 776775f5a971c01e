#pragma once
// The adapter record as the GPU certificate names it (raw/renderer/gpu_reconcile.hpp).
#include "raw/renderer/render.hpp"
#include "raw/rhi/rhi.hpp"
namespace raw {
using GpuAdapterInfo = rhi::AdapterInfo;
}  // namespace raw
