// C entry points over the shim for tests: they build raw:: objects from plain arrays, call
// the reference's symbols as the renderer would, and copy the results out. Each returns 0,
// or -1 with the exception's message in `msg`.
#include "raw/renderer/ray_ao.hpp"
#include "raw/renderer/ssao.hpp"
#include "raw/renderer/gpu.hpp"
#include "raw/cert/reconcile.hpp"
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <string>
#include <vector>

using namespace raw;

namespace {
GBuffer gbuffer(int w, int h, const float* pos, const float* nrm, const uint8_t* mask) {
    GBuffer g;
    g.resize(w, h);
    for (std::size_t i = 0; i < (std::size_t)w * h; ++i) {
        g.position.px[i] = Vec3{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        g.normal.px[i] = Vec3{nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]};
        g.mask.px[i] = mask[i];
    }
    return g;
}
int report(const std::exception& e, char* msg, int len) {
    if (msg && len > 0) std::snprintf(msg, (std::size_t)len, "%s", e.what());
    return -1;
}
}  // namespace

extern "C" {

__attribute__((visibility("default")))
int shim_rt_visibility(int w, int h, const float* pos, const float* nrm, const uint8_t* mask, const float* tris,
                       int ntri, int spp, float radius, const float* toLight, int sunForced, int skew, float* ao,
                       float* sky, float* sun, char* msg, int msglen) {
    try {
        const GBuffer g = gbuffer(w, h, pos, nrm, mask);
        LinearAccel acc;
        acc.tris.resize((std::size_t)ntri);
        if (ntri) std::memcpy(acc.tris.data(), tris, (std::size_t)ntri * sizeof(Tri));
        if (skew) acc.mode = LinearAccel::Mode::Skew;
        if (toLight) {
            Buffer<float> a, s, u;
            computeRTVisibility(g, acc, spp, radius, Vec3{toLight[0], toLight[1], toLight[2]}, a, s, u, 8,
                                sunForced != 0);
            std::memcpy(ao, a.px.data(), a.px.size() * 4);
            std::memcpy(sky, s.px.data(), s.px.size() * 4);
            std::memcpy(sun, u.px.data(), u.px.size() * 4);
        } else {
            const Buffer<float> a = computeRTAO(g, acc, spp, radius);
            std::memcpy(ao, a.px.data(), a.px.size() * 4);
        }
        return 0;
    } catch (const std::exception& e) {
        return report(e, msg, msglen);
    }
}

__attribute__((visibility("default")))
int shim_ssao(int w, int h, const float* pos, const float* nrm, const uint8_t* mask, int samples, float radius,
              float* out, char* msg, int msglen) {
    try {
        const Buffer<float> a = computeSSAO(gbuffer(w, h, pos, nrm, mask), samples, radius);
        std::memcpy(out, a.px.data(), a.px.size() * 4);
        return 0;
    } catch (const std::exception& e) {
        return report(e, msg, msglen);
    }
}

// stats4: rmse, maxError, pixels, within. arena_used: bytes the caller's arena handed out.
__attribute__((visibility("default")))
int shim_reconcile(int w, int h, const float* approx, const float* truth, const uint8_t* mask, float tolerance,
                   float* err, float* stats4, uint64_t* arena_used, char* msg, int msglen) {
    try {
        Buffer<float> a, t;
        Buffer<uint8_t> m;
        a.resize(w, h); t.resize(w, h); m.resize(w, h);
        const std::size_t n = (std::size_t)w * h;
        if (n) {
            std::memcpy(a.px.data(), approx, n * 4);
            std::memcpy(t.px.data(), truth, n * 4);
            std::memcpy(m.px.data(), mask, n);
        }
        std::vector<unsigned char> backing(n * 4 + 64);
        Arena arena(backing.data(), backing.size());
        const ReconcileResult r = reconcile(a, t, m, tolerance, &arena);
        if (n) std::memcpy(err, r.errorMap.px.data(), n * 4);
        stats4[0] = r.rmse; stats4[1] = r.maxError; stats4[2] = (float)r.pixels; stats4[3] = r.withinTolerance ? 1.f : 0.f;
        *arena_used = arena.stats().used;
        return 0;
    } catch (const std::exception& e) {
        return report(e, msg, msglen);
    }
}

// raw::renderGpu (gpu_shim.cpp) on a scene of `ntri` triangles, one mesh each with its own
// albedo, seen from cam10 (eye, target, up, fovy; aspect w / h); light4 = direction and
// intensity of the one light, or NULL for none. FrameResult's planes are copied out (any
// pointer may be NULL); stats4 = rmse, maxError, pixels, within; motion2 = valid, total;
// vp16 = FrameResult::viewProj; adapter gets gpuInit's "vendor|architecture|device|backend|driver".
__attribute__((visibility("default")))
int shim_render_gpu(int w, int h, const float* cam10, const float* prev_vp16, const float* tris9, const float* nrm9,
                    const float* alb3, int ntri, const float* light4, int rtao, int lighting, float tolerance,
                    int frame_only, float* depth, float* pos, float* nrm, float* alb, uint8_t* mask, float* motion,
                    float* ao_rt, float* ao_ss, float* err, float* frame, float* hdr, float* stats4, int* motion2,
                    float* vp16, char* adapter, int adapter_len, char* msg, int msglen) {
    try {
        std::string e;
        GpuAdapterInfo info;
        if (!gpuInit(info, e)) throw std::runtime_error("gpuInit: " + e);
        if (adapter && adapter_len > 0)
            std::snprintf(adapter, (std::size_t)adapter_len, "%s|%s|%s|%s|%s", info.vendor.c_str(),
                          info.architecture.c_str(), info.device.c_str(), info.backend.c_str(), info.driver.c_str());
        Scene s;
        for (int t = 0; t < ntri; ++t) {
            Mesh m;
            for (int k = 0; k < 3; ++k) {
                m.positions.push_back(Vec3{tris9[9 * t + 3 * k], tris9[9 * t + 3 * k + 1], tris9[9 * t + 3 * k + 2]});
                m.normals.push_back(Vec3{nrm9[9 * t + 3 * k], nrm9[9 * t + 3 * k + 1], nrm9[9 * t + 3 * k + 2]});
                m.indices.push_back(k);
            }
            m.material.albedo = Vec3{alb3[3 * t], alb3[3 * t + 1], alb3[3 * t + 2]};
            s.meshes.push_back(m);
        }
        if (light4) s.lights.push_back(Light{Vec3{light4[0], light4[1], light4[2]}, light4[3]});
        s.camera.eye = Vec3{cam10[0], cam10[1], cam10[2]};
        s.camera.center = Vec3{cam10[3], cam10[4], cam10[5]};
        s.camera.up = Vec3{cam10[6], cam10[7], cam10[8]};
        s.camera.fovy = cam10[9];
        s.camera.aspect = (float)w / (float)h;
        Mat4 prev;
        std::memcpy(prev.m, prev_vp16, sizeof prev.m);
        RenderOptions o;
        o.tolerance = tolerance;
        o.rtao = rtao != 0;
        o.lighting = lighting;
        FrameResult r;
        if (!renderGpu(s, w, h, prev, o, r, e, frame_only != 0)) throw std::runtime_error("renderGpu: " + e);
        const std::size_t n = (std::size_t)w * h;
        auto put3 = [n](float* dst, const Buffer<Vec3>& b) {
            if (!dst || b.px.size() != n) return;
            for (std::size_t i = 0; i < n; ++i) { dst[3 * i] = b.px[i].x; dst[3 * i + 1] = b.px[i].y; dst[3 * i + 2] = b.px[i].z; }
        };
        auto put1 = [n](float* dst, const Buffer<float>& b) {
            if (dst && b.px.size() == n) std::memcpy(dst, b.px.data(), n * 4);
        };
        put3(frame, r.frame);
        if (!frame_only) {
            put1(depth, r.g.depth); put3(pos, r.g.position); put3(nrm, r.g.normal); put3(alb, r.g.albedo);
            if (mask) std::memcpy(mask, r.g.mask.px.data(), n);
            if (motion)
                for (std::size_t i = 0; i < n; ++i) { motion[2 * i] = r.g.motion.px[i].x; motion[2 * i + 1] = r.g.motion.px[i].y; }
            put1(ao_rt, r.aoRT); put1(ao_ss, r.aoSS); put1(err, r.rec.errorMap); put3(hdr, r.hdr);
        }
        if (stats4) {
            stats4[0] = r.rec.rmse; stats4[1] = r.rec.maxError; stats4[2] = (float)r.rec.pixels;
            stats4[3] = r.rec.withinTolerance ? 1.f : 0.f;
        }
        if (motion2) { motion2[0] = r.motionValid; motion2[1] = r.motionTotal; }
        if (vp16) std::memcpy(vp16, r.viewProj.m, 64);
        // frame-only: every plane but the frame is left empty, as the reference leaves it
        if (frame_only && (r.g.w != 0 || !r.aoSS.px.empty() || !r.hdr.px.empty())) throw std::runtime_error("frame-only filled more than the frame");
        return 0;
    } catch (const std::exception& e) {
        return report(e, msg, msglen);
    }
}

}  // extern "C"
