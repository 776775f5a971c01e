#pragma once
// The adapter record of raw-native's hardware interface (raw/rhi/rhi.hpp): strings as the
// backend reports them, empty where it says nothing.
#include <string>
namespace raw::rhi {
struct AdapterInfo {
    std::string vendor, architecture, device, description, backend, driver;
};
}  // namespace raw::rhi
