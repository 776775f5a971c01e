// The lighting-model choice of raw/renderer/render.hpp for the stand-alone shim build (inside
// raw-native, src/renderer/render.cpp:57-67 defines these): without the ray-traced pass the
// frame is model 1; RAW_NATIVE_LIGHTING=v1 forces model 1, =v2 or =v2-nosun model 2, the
// latter with the sun's visibility forced to 1 (a test-only control); otherwise opts.lighting.
#include "raw/renderer/render.hpp"
#include <cstdlib>
#include <cstring>

namespace raw {

int lightingModel(const RenderOptions& o) {
    if (!o.rtao) return 1;
    const char* v = std::getenv("RAW_NATIVE_LIGHTING");
    if (v && std::strcmp(v, "v1") == 0) return 1;
    if (v && (std::strcmp(v, "v2") == 0 || std::strcmp(v, "v2-nosun") == 0)) return 2;
    return o.lighting == 1 ? 1 : 2;
}

bool lightingNoSun() {
    const char* v = std::getenv("RAW_NATIVE_LIGHTING");
    return v && std::strcmp(v, "v2-nosun") == 0;
}

}  // namespace raw
