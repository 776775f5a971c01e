#pragma once
// One rendered frame and the per-render options (raw/renderer/render.hpp): the G-buffer,
// both AO estimators, their reconcile, the clamped frame and its HDR view, the motion
// counts and the view-projection; the renderer's fixed AO sampling.
#include "raw/cert/reconcile.hpp"
#include "raw/math/mat.hpp"
#include "raw/renderer/gbuffer.hpp"
#include "raw/scene/scene.hpp"
namespace raw {
struct FrameResult {
    GBuffer g;
    Buffer<float> aoRT, aoSS;
    ReconcileResult rec;
    Buffer<Vec3> frame;
    Buffer<Vec3> hdr;
    int motionValid{0};
    int motionTotal{0};
    Mat4 viewProj{};
};
inline constexpr int kRtSamples = 64;
inline constexpr int kSsSamples = 24;
inline constexpr float kAoRadius = 2.0f;
struct RenderOptions {
    float tolerance{0.12f};
    bool rtao{true};
    int threads{1};
    int lighting{2};
};
int lightingModel(const RenderOptions& o);
bool lightingNoSun();
}  // namespace raw
