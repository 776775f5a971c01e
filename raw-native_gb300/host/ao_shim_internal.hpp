// ao_shim_internal.hpp -- what the shim's translation units share: the GPU accelerator of a
// raw::LinearAccel and the error path.
#pragma once
#include "raw/renderer/accel.hpp"
#include "rn_ao.h"

namespace raw::gpu_shim {

// The GPU accelerator built from `accel`'s triangle list. raw::LinearAccel is the
// reference's struct and has no room for a handle, so accelerators are cached by the
// triangle count and a 64-bit FNV-1a hash of the triangles' bytes (at most 8 live entries).
rn_accel* accelOf(const LinearAccel& accel);

// Throw std::runtime_error("<what>: <status message>"); the CLI's GPU path reports it as
// exit 4 / "unverifiable", the reference's answer when the device cannot do the work.
[[noreturn]] void fail(const char* what, const rn_status& st);

}  // namespace raw::gpu_shim
