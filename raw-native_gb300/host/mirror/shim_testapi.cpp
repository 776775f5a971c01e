// C entry points over the shim for tests: they build raw:: objects from plain arrays, call
// the reference's symbols as the renderer would, and copy the results out. Each returns 0,
// or -1 with the exception's message in `msg`.
#include "raw/renderer/ray_ao.hpp"
#include "raw/renderer/ssao.hpp"
#include "raw/cert/reconcile.hpp"
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <exception>
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

}  // extern "C"
