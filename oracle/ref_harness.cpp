// ref_harness.cpp -- extern "C" entry points over the reference's OWN sources.
//
// TEST INFRASTRUCTURE ONLY. oracle/Makefile compiles this file together with the few
// raw-native source files of the AO path (read in place, never copied) into
// oracle/_ref/libref_ao.so. Tests use it to pin the C restatement in rn_oracle.c and to
// make golden fixtures; nothing in the product links it.
//
// The frame follows src/renderer/render.cpp:29-54 (rtao, ssao, reconcile passes) with the
// scene of src/scene/scene.cpp:18-32 and the camera of src/tools/cli_params.cpp:12-18.
#include "raw/renderer/ray_ao.hpp"
#include "raw/renderer/ssao.hpp"
#include "raw/renderer/raster.hpp"
#include "raw/renderer/accel.hpp"
#include "raw/renderer/rt_bvh.hpp"
#include "raw/cert/reconcile.hpp"
#include "raw/scene/scene.hpp"
#include "raw/renderer/post.hpp"
#include "raw/renderer/motion.hpp"
#include <cstdint>
#include <cstring>
#include <vector>

using namespace raw;

namespace {
Scene sceneFromTris(const float* tris9, int ntri) {
    Scene s;
    Mesh m;
    for (int i = 0; i < ntri; ++i)
        for (int k = 0; k < 3; ++k) {
            const float* p = tris9 + (std::size_t)i * 9 + 3 * k;
            m.positions.push_back(Vec3{p[0], p[1], p[2]});
            m.normals.push_back(Vec3{0, 1, 0});
            m.indices.push_back(i * 3 + k);
        }
    s.meshes.push_back(std::move(m));
    return s;
}
GBuffer gbufferFrom(int w, int h, const float* pos, const float* nrm, const uint8_t* mask) {
    GBuffer g;
    g.resize(w, h);
    for (std::size_t i = 0; i < (std::size_t)w * h; ++i) {
        g.position.px[i] = Vec3{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        g.normal.px[i] = Vec3{nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]};
        g.mask.px[i] = mask[i];
    }
    return g;
}
}  // namespace

extern "C" {

// The built-in scene rendered as the CLI does: rasterize, accel, computeRTVisibility
// (lighting model 2), computeSSAO, reconcile. cam10 = eye, target, up, fovy.
__attribute__((visibility("default")))
void ref_render_default(int w, int h, const float* cam10, int spp, float radius, int ssSamples,
                        float tolerance, int threads, float* pos, float* nrm, uint8_t* mask,
                        float* ao, float* sky, float* sun, float* ss, float* err, float* stats4) {
    Scene s = buildTestScene(w, h);
    s.camera.eye = {cam10[0], cam10[1], cam10[2]};
    s.camera.center = {cam10[3], cam10[4], cam10[5]};
    s.camera.up = {cam10[6], cam10[7], cam10[8]};
    s.camera.fovy = cam10[9];
    s.camera.aspect = h > 0 ? (float)w / (float)h : 1.0f;
    GBuffer g = rasterize(s, w, h);
    LinearAccel accel;
    accel.build(s);
    const Vec3 toLight = s.lights[0].dir * -1.0f;
    Buffer<float> a, sk, su;
    computeRTVisibility(g, accel, spp, radius, toLight, a, sk, su, threads, false);
    Buffer<float> sa = computeSSAO(g, ssSamples, radius, nullptr, threads);
    ReconcileResult r = reconcile(sa, a, g.mask, tolerance);
    for (std::size_t i = 0; i < (std::size_t)w * h; ++i) {
        pos[3 * i] = g.position.px[i].x; pos[3 * i + 1] = g.position.px[i].y; pos[3 * i + 2] = g.position.px[i].z;
        nrm[3 * i] = g.normal.px[i].x; nrm[3 * i + 1] = g.normal.px[i].y; nrm[3 * i + 2] = g.normal.px[i].z;
        mask[i] = g.mask.px[i];
        ao[i] = a.px[i]; sky[i] = sk.px[i]; sun[i] = su.px[i]; ss[i] = sa.px[i]; err[i] = r.errorMap.px[i];
    }
    stats4[0] = r.rmse; stats4[1] = r.maxError; stats4[2] = (float)r.pixels; stats4[3] = r.withinTolerance ? 1.0f : 0.0f;
}

// computeRTVisibility (toLight3 != NULL) or computeRTAO over an arbitrary triangle list
// and G-buffer, with the reference's LinearAccel (SAH BVH).
__attribute__((visibility("default")))
void ref_trace(int w, int h, const float* pos, const float* nrm, const uint8_t* mask,
               const float* tris9, int ntri, int spp, float radius, const float* toLight3,
               float* ao, float* sky, float* sun, int threads) {
    const Scene s = sceneFromTris(tris9, ntri);
    LinearAccel accel;
    accel.build(s);
    const GBuffer g = gbufferFrom(w, h, pos, nrm, mask);
    if (toLight3) {
        Buffer<float> a, sk, su;
        computeRTVisibility(g, accel, spp, radius, Vec3{toLight3[0], toLight3[1], toLight3[2]}, a, sk, su, threads, false);
        std::memcpy(ao, a.px.data(), a.px.size() * 4);
        std::memcpy(sky, sk.px.data(), sk.px.size() * 4);
        std::memcpy(sun, su.px.data(), su.px.size() * 4);
    } else {
        Buffer<float> a = computeRTAO(g, accel, spp, radius, nullptr, threads);
        std::memcpy(ao, a.px.data(), a.px.size() * 4);
    }
}

__attribute__((visibility("default")))
void ref_ssao(int w, int h, const float* pos, const float* nrm, const uint8_t* mask, int samples,
              float radius, float* out, int threads) {
    const GBuffer g = gbufferFrom(w, h, pos, nrm, mask);
    Buffer<float> a = computeSSAO(g, samples, radius, nullptr, threads);
    std::memcpy(out, a.px.data(), a.px.size() * 4);
}

__attribute__((visibility("default")))
void ref_reconcile(int w, int h, const float* approx, const float* truth, const uint8_t* mask,
                   float tolerance, float* err, float* stats4) {
    Buffer<float> a, b; Buffer<uint8_t> m;
    a.resize(w, h); b.resize(w, h); m.resize(w, h);
    std::memcpy(a.px.data(), approx, (std::size_t)w * h * 4);
    std::memcpy(b.px.data(), truth, (std::size_t)w * h * 4);
    std::memcpy(m.px.data(), mask, (std::size_t)w * h);
    ReconcileResult r = reconcile(a, b, m, tolerance);
    std::memcpy(err, r.errorMap.px.data(), (std::size_t)w * h * 4);
    stats4[0] = r.rmse; stats4[1] = r.maxError; stats4[2] = (float)r.pixels; stats4[3] = r.withinTolerance ? 1.0f : 0.0f;
}

// rt::buildPloc; nodes as 9 int32 each {left, right, tri, lo0, hi0, lo1, hi1, lo2, hi2}.
__attribute__((visibility("default")))
int ref_ploc(const float* tris9, int n, int radius, int32_t* out9, uint32_t* rounds) {
    std::vector<Tri> t((std::size_t)n);
    std::memcpy(t.data(), tris9, (std::size_t)n * 36);
    const rt::Tree T = rt::buildPloc(t, radius);
    for (std::size_t i = 0; i < T.nodes.size(); ++i) {
        const rt::Node& x = T.nodes[i];
        int32_t* o = out9 + i * 9;
        o[0] = x.left; o[1] = x.right; o[2] = x.tri;
        for (int k = 0; k < 3; ++k) { std::memcpy(&o[3 + 2 * k], &x.lo[k], 4); std::memcpy(&o[4 + 2 * k], &x.hi[k], 4); }
    }
    *rounds = T.rounds;
    return T.root;
}

// rt::closest (src/renderer/rt_bvh.cpp:125-152) on rt::buildPloc's tree (default radius) for
// rays (n, 6): the triangle index (-1: none) and t (-1: none).
void ref_closest(const float* tris9, int ntri, const float* rays6, const float* tmax, int n, int32_t* tri, float* t) {
    std::vector<Tri> tv((std::size_t)ntri);
    std::memcpy(tv.data(), tris9, (std::size_t)ntri * 36);
    const rt::Tree T = rt::buildPloc(tv);
    for (int i = 0; i < n; ++i) {
        const float* r = rays6 + (std::size_t)i * 6;
        Hit h;
        if (rt::closest(T, tv, Ray{Vec3{r[0], r[1], r[2]}, Vec3{r[3], r[4], r[5]}}, tmax[i], h)) {
            tri[i] = h.tri;
            t[i] = h.t;
        } else {
            tri[i] = -1;
            t[i] = -1.0f;
        }
    }
}

}  // extern "C"


// raw::post::viewGBuffer (src/renderer/post_gtao.cpp:36-53) of a G-buffer and a camera
// (cam10: eye, center, up, fovy; aspect w / h; nearZ 0.1).
extern "C" void ref_view_gbuffer(int w, int h, const float* pos, const float* nrm, const uint8_t* mask,
                                 const float* cam10, float* vpos, float* vnrm, float* vdepth) {
    GBuffer g = gbufferFrom(w, h, pos, nrm, mask);
    g.depth.resize(w, h);
    Camera cam;
    cam.eye = Vec3{cam10[0], cam10[1], cam10[2]};
    cam.center = Vec3{cam10[3], cam10[4], cam10[5]};
    cam.up = Vec3{cam10[6], cam10[7], cam10[8]};
    cam.fovy = cam10[9];
    cam.aspect = (float)w / (float)h;
    const post::ViewGBuffer v = post::viewGBuffer(g, cam);
    std::memcpy(vpos, v.pos.data(), v.pos.size() * sizeof(float));
    std::memcpy(vnrm, v.nrm.data(), v.nrm.size() * sizeof(float));
    std::memcpy(vdepth, v.depth.data(), v.depth.size() * sizeof(float));
}

// raw::post::gtao (src/renderer/post_gtao.cpp:64-135) on a view-space G-buffer.
extern "C" void ref_gtao(int w, int h, const float* vpos, const float* vnrm, const float* vdepth, double tanHalf,
                         double aspect, double radius, int slices, int steps, double* out) {
    post::ViewGBuffer v;
    v.w = w; v.h = h; v.tanHalf = tanHalf; v.aspect = aspect;
    const std::size_t n = (std::size_t)w * h;
    v.pos.assign(vpos, vpos + 3 * n);
    v.nrm.assign(vnrm, vnrm + 3 * n);
    v.depth.assign(vdepth, vdepth + n);
    post::GtaoParams p;
    p.radius = radius; p.slices = slices; p.steps = steps;
    const std::vector<double> r = post::gtao(v, p);
    std::memcpy(out, r.data(), n * sizeof(double));
}

// raw::computeMotion (src/renderer/motion.cpp:17-32) of a G-buffer's positions and mask between
// two view-projections (16 floats each, row-major); returns the valid count.
extern "C" int ref_motion(int w, int h, const float* pos, const uint8_t* mask, const float* vp16, const float* prev16,
                          float* motion2) {
    std::vector<float> nrm((std::size_t)w * h * 3, 0.0f);
    GBuffer g = gbufferFrom(w, h, pos, nrm.data(), mask);
    g.motion.resize(w, h);
    Mat4 a, b;
    std::memcpy(a.m, vp16, sizeof a.m);
    std::memcpy(b.m, prev16, sizeof b.m);
    const int valid = computeMotion(g, a, b);
    for (std::size_t i = 0; i < (std::size_t)w * h; ++i) {
        motion2[2 * i] = g.motion.px[i].x;
        motion2[2 * i + 1] = g.motion.px[i].y;
    }
    return valid;
}
