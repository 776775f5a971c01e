// The link seam: raw-native's own scene, rasterizer and frame structure, with the AO passes
// resolved to the GPU shim (ao_shim.cpp, accel_shim.cpp) instead of ray_ao.cpp, ssao.cpp,
// reconcile.cpp and accel.cpp. Renders the built-in scene's AO passes as
// src/renderer/render.cpp:29-54 does and prints the reconcile; a GPU failure is reported as
// the reference reports one: "unverifiable" and exit 4.
#include "raw/renderer/ray_ao.hpp"
#include "raw/renderer/ssao.hpp"
#include "raw/renderer/raster.hpp"
#include "raw/renderer/render.hpp"
#include "raw/cert/reconcile.hpp"
#include "raw/scene/scene.hpp"
#include <cstdio>
#include <cstdlib>
#include <stdexcept>

int main(int argc, char** argv) {
    const int w = argc > 1 ? std::atoi(argv[1]) : 256, h = argc > 2 ? std::atoi(argv[2]) : 256;
    try {
        raw::Scene s = raw::buildTestScene(w, h);
        raw::GBuffer g = raw::rasterize(s, w, h);
        raw::LinearAccel accel;
        accel.build(s);
        const raw::Vec3 toLight = s.lights[0].dir * -1.0f;
        raw::Buffer<float> ao, sky, sun;
        raw::computeRTVisibility(g, accel, raw::kRtSamples, raw::kAoRadius, toLight, ao, sky, sun, 1, false);
        raw::Buffer<float> ss = raw::computeSSAO(g, raw::kSsSamples, raw::kAoRadius);
        raw::ReconcileResult r = raw::reconcile(ss, ao, g.mask, 0.12f);
        std::printf("reconcile: pixels=%d rmse=%.9g maxError=%.9g verdict=%s\n", r.pixels, r.rmse, r.maxError,
                    r.withinTolerance ? "verified" : "refuted");
        return 0;
    } catch (const std::exception& e) {
        std::printf("verdict=unverifiable (%s)\n", e.what());
        return 4;
    }
}
