// ao_shim.cpp -- raw-native's AO passes on the GPU behind the reference's own symbols.
//
// A build of raw-native that lists this file in place of src/renderer/ray_ao.cpp,
// src/renderer/ssao.cpp and src/cert/reconcile.cpp (and links librn_ao.so) sends
// computeRTAO, computeRTVisibility, computeSSAO and reconcile to one GB300 with no other
// source change: the frame graph (src/renderer/render.cpp:29-54), `verify`
// (src/tools/verify.cpp:77) and the tests call these symbols as before.
//
// Outputs are allocated exactly as the reference allocates them (same Buffer constructors,
// same order, from the caller's arena), so the arena certificate does not change; the
// library's device and staging memory stay outside the arena. The `threads` argument is
// accepted and ignored: the GPU path is one call from one host thread.
#include "raw/renderer/ray_ao.hpp"
#include "raw/renderer/ssao.hpp"
#include "raw/cert/reconcile.hpp"
#include "ao_shim_internal.hpp"
#include "rn_ao.h"

#include <cstdint>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

namespace raw::gpu_shim {

[[noreturn]] void fail(const char* what, const rn_status& st) {
    throw std::runtime_error(std::string(what) + ": " + st.message);
}

namespace {
struct Entry { std::size_t count; rn_accel* handle; };
struct Cache {
    std::mutex m;
    std::unordered_map<std::uint64_t, Entry> map;
    std::vector<std::uint64_t> order;   // insertion order, for eviction
    ~Cache() { for (auto& kv : map) rn_accel_free(kv.second.handle); }
};
Cache& cache() { static Cache c; return c; }

std::uint64_t fnv1a(const void* data, std::size_t bytes) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    std::uint64_t h = 1469598103934665603ull;
    for (std::size_t i = 0; i < bytes; ++i) { h ^= p[i]; h *= 1099511628211ull; }
    return h;
}
}  // namespace

rn_accel* accelOf(const LinearAccel& accel) {
    const std::size_t n = accel.tris.size();
    static_assert(sizeof(Tri) == 9 * sizeof(float), "raw::Tri is three Vec3");
    const std::uint64_t key = fnv1a(accel.tris.data(), n * sizeof(Tri)) ^ (std::uint64_t)n * 0x9E3779B97F4A7C15ull;
    Cache& c = cache();
    std::lock_guard<std::mutex> lock(c.m);
    auto it = c.map.find(key);
    if (it != c.map.end() && it->second.count == n) return it->second.handle;
    rn_accel* h = nullptr;
    rn_status st{};
    const float* tris = n ? &accel.tris.data()[0].a.x : nullptr;
    if (rn_accel_build(tris, (std::uint32_t)n, 0, &h, &st) != RN_OK) fail("LinearAccel (GPU build)", st);
    if (c.order.size() >= 8) {
        const std::uint64_t old = c.order.front();
        c.order.erase(c.order.begin());
        auto o = c.map.find(old);
        if (o != c.map.end()) { rn_accel_free(o->second.handle); c.map.erase(o); }
    }
    c.map[key] = Entry{n, h};
    c.order.push_back(key);
    return h;
}

namespace {
rn_gbuf gbufOf(const GBuffer& g) {
    return rn_gbuf{g.w, g.h, &g.position.px.data()[0].x, &g.normal.px.data()[0].x, g.mask.px.data()};
}
// RAW_NATIVE_AO_ORACLE=skew shortens the query distance by 1% (src/renderer/accel.cpp:6-11,28),
// the reference's false-success control; scan and the BVH give the same answers on the GPU.
float queryRadius(const LinearAccel& accel, float radius) {
    return accel.mode == LinearAccel::Mode::Skew ? radius * 0.99f : radius;
}
}  // namespace
}  // namespace raw::gpu_shim

namespace raw {

Buffer<float> computeRTAO(const GBuffer& g, const LinearAccel& accel, int samples, float radius, Arena* arena,
                          int threads) {
    (void)threads;
    Buffer<float> ao(arena);
    ao.resize(g.w, g.h);
    if ((std::size_t)g.w * (std::size_t)g.h == 0) return ao;
    const rn_gbuf gb = gpu_shim::gbufOf(g);
    rn_status st{};
    if (rn_ao_visibility(&gb, gpu_shim::accelOf(accel), samples, gpu_shim::queryRadius(accel, radius), nullptr, 0,
                         ao.px.data(), nullptr, nullptr, &st) != RN_OK)
        gpu_shim::fail("computeRTAO", st);
    return ao;
}

void computeRTVisibility(const GBuffer& g, const LinearAccel& accel, int samples, float radius, Vec3 toLight,
                         Buffer<float>& ao, Buffer<float>& sky, Buffer<float>& sun, int threads, bool sunForced) {
    (void)threads;
    ao.resize(g.w, g.h);
    sky.resize(g.w, g.h);
    sun.resize(g.w, g.h);
    if ((std::size_t)g.w * (std::size_t)g.h == 0) return;
    const rn_gbuf gb = gpu_shim::gbufOf(g);
    const float tl[3] = {toLight.x, toLight.y, toLight.z};     // normalized on the device, as the reference does
    rn_status st{};
    if (rn_ao_visibility(&gb, gpu_shim::accelOf(accel), samples, gpu_shim::queryRadius(accel, radius), tl,
                         RN_SKY | (sunForced ? RN_SUN_FORCED : 0), ao.px.data(), sky.px.data(), sun.px.data(),
                         &st) != RN_OK)
        gpu_shim::fail("computeRTVisibility", st);
}

Buffer<float> computeSSAO(const GBuffer& g, int samples, float radius, Arena* arena, int threads) {
    (void)threads;
    Buffer<float> ao(arena);
    ao.resize(g.w, g.h);
    if ((std::size_t)g.w * (std::size_t)g.h == 0) return ao;
    const rn_gbuf gb = gpu_shim::gbufOf(g);
    rn_status st{};
    if (rn_ssao(&gb, samples, radius, 0, ao.px.data(), &st) != RN_OK) gpu_shim::fail("computeSSAO", st);
    return ao;
}

ReconcileResult reconcile(const Buffer<float>& approx, const Buffer<float>& truth, const Buffer<uint8_t>& mask,
                          float tolerance, Arena* arena) {
    ReconcileResult r;
    r.errorMap = Buffer<float>(arena);
    r.errorMap.resize(approx.w, approx.h);
    const std::size_t np = (std::size_t)approx.w * (std::size_t)approx.h;
    if (truth.px.size() < np || mask.px.size() < np)
        throw std::invalid_argument("reconcile: truth or mask smaller than the approximation");
    if (np == 0) {
        r.withinTolerance = r.rmse <= tolerance;
        return r;
    }
    rn_reconcile_result out{};
    rn_status st{};
    if (rn_reconcile(approx.px.data(), truth.px.data(), mask.px.data(), approx.w, approx.h, tolerance, 0,
                     r.errorMap.px.data(), &out, &st) != RN_OK)
        gpu_shim::fail("reconcile", st);
    r.rmse = out.rmse;
    r.maxError = out.max_error;
    r.pixels = out.pixels;
    r.withinTolerance = out.within_tolerance != 0;
    return r;
}

}  // namespace raw
