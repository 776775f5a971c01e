// gpu_shim.cpp -- raw-native's `--gpu` frame on CUDA, behind the reference's own symbols.
//
// A build of raw-native that lists this file in place of src/renderer/gpu/gpu_renderer.cpp
// (and links librn_ao.so) gives raw::gpuCompiled, raw::gpuBackendName, raw::gpuInit and
// raw::renderGpu (raw/renderer/gpu.hpp:22-33) to the callers that use them unchanged:
// `raw_native_cli --gpu` (src/tools/gpu_run.cpp:66-96) renders the frame here, renders the
// CPU reference beside it and writes raw-gpu-cert/1 from reconcileGpuCpu as before. With no
// usable device gpuInit returns false with the library's reason, so gpu_run.cpp writes its
// "unverifiable" certificate and exits 4, the reference's answer on the null backend.
//
// The frame is rn_render_frame: the G-buffer with albedo, motion, SSAO, the ray-traced AO
// (with lighting model 2's sky and sun), shading and the HDR view, every plane equal to the
// CPU path's bit for bit, at the renderer's fixed sampling (raw/renderer/render.hpp:25-27).
// The AO reconcile comes back with the frame (computed on the GPU, the same numbers as
// reconcile()); FrameResult is filled as src/renderer/gpu/frame_pack.cpp:48-77 fills it.
#include "raw/renderer/gpu.hpp"
#include "rn_ao.h"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

namespace raw {

bool gpuCompiled() { return true; }

const char* gpuBackendName() { return "cuda"; }

bool gpuInit(GpuAdapterInfo& info, std::string& err) {
    rn_status st{};
    rn_device_desc d{};
    if (rn_device_info(&d, &st) != RN_OK) {
        err = st.message;
        return false;
    }
    char buf[64];
    info.vendor = "NVIDIA";
    std::snprintf(buf, sizeof buf, "sm_%d%d", d.cc_major, d.cc_minor);
    info.architecture = buf;
    info.device = d.name;
    std::snprintf(buf, sizeof buf, " (%d SMs, %.0f GiB)", d.sm_count, (double)d.total_bytes / (1024.0 * 1024 * 1024));
    info.description = std::string(d.name) + buf;
    info.backend = "cuda";
    std::snprintf(buf, sizeof buf, "CUDA driver %d.%d, runtime %d.%d", d.driver_version / 1000,
                  (d.driver_version % 1000) / 10, d.runtime_version / 1000, (d.runtime_version % 1000) / 10);
    info.driver = buf;
    return true;
}

bool renderGpu(const Scene& scene, int w, int h, const Mat4& prevViewProj, const RenderOptions& opts,
               FrameResult& r, std::string& err, bool frameOnly) {
    r = FrameResult();
    if (w <= 0 || h <= 0) {
        err = "frame size " + std::to_string(w) + "x" + std::to_string(h);
        return false;
    }
    // rn_render_frame projects with aspect w / h and near/far 0.1/100, the CLI's camera
    // (src/tools/cli_params.cpp:12-18); any other projection would not be the CPU frame's.
    const Camera& c = scene.camera;
    if (c.aspect != (float)w / (float)h || c.nearZ != 0.1f || c.farZ != 100.0f) {
        err = "the CUDA frame takes the CLI's projection (aspect w/h, near 0.1, far 100)";
        return false;
    }
    if (lightingNoSun()) {
        err = "RAW_NATIVE_LIGHTING=v2-nosun (the test-only control) is not built on the CUDA backend";
        return false;
    }
    // triangles in scene order, as packTriangles lays them out (frame_pack.cpp:7-20)
    std::vector<float> tris, nrms, alb;
    for (const Mesh& m : scene.meshes)
        for (std::size_t i = 0; i + 2 < m.indices.size(); i += 3) {
            for (int k = 0; k < 3; ++k) {
                const Vec3 p = m.positions[m.indices[i + k]], n = m.normals[m.indices[i + k]];
                tris.insert(tris.end(), {p.x, p.y, p.z});
                nrms.insert(nrms.end(), {n.x, n.y, n.z});
            }
            alb.insert(alb.end(), {m.material.albedo.x, m.material.albedo.y, m.material.albedo.z});
        }
    rn_frame_scene sc{};
    sc.tris = tris.data();
    sc.normals = nrms.data();
    sc.albedo = alb.data();
    sc.ntri = (uint32_t)(alb.size() / 3);
    sc.has_light = scene.lights.empty() ? 0 : 1;
    if (sc.has_light) {
        sc.light_dir[0] = scene.lights[0].dir.x;
        sc.light_dir[1] = scene.lights[0].dir.y;
        sc.light_dir[2] = scene.lights[0].dir.z;
        sc.light_intensity = scene.lights[0].intensity;
    }
    const float cam[10] = {c.eye.x, c.eye.y, c.eye.z, c.center.x, c.center.y, c.center.z, c.up.x, c.up.y, c.up.z,
                           c.fovy};
    const rn_frame_options o{opts.tolerance, opts.rtao ? 1 : 0, lightingModel(opts), kRtSamples, kAoRadius,
                             kSsSamples};
    const std::size_t n = (std::size_t)w * (std::size_t)h;
    std::vector<float> frame(n * 3), hdr, depth, pos, nrm, albedo, motion, ao_rt, ao_ss, errmap;
    std::vector<uint8_t> mask;
    rn_frame_out out{};
    out.frame = frame.data();
    if (!frameOnly) {
        hdr.resize(n * 3); depth.resize(n); pos.resize(n * 3); nrm.resize(n * 3); albedo.resize(n * 3);
        motion.resize(n * 2); ao_ss.resize(n); errmap.resize(n); mask.resize(n);
        if (opts.rtao) ao_rt.resize(n);
        out.hdr = hdr.data(); out.depth = depth.data(); out.position = pos.data(); out.normal = nrm.data();
        out.albedo = albedo.data(); out.motion = motion.data(); out.ao_ss = ao_ss.data();
        out.error_map = errmap.data(); out.mask = mask.data();
        out.ao_rt = opts.rtao ? ao_rt.data() : nullptr;
    }
    rn_status st{};
    if (rn_render_frame(&sc, cam, prevViewProj.m, w, h, &o, 0, &out, &st) != RN_OK) {
        err = st.message;
        return false;
    }
    r.frame.resize(w, h);
    for (std::size_t i = 0; i < n; ++i) r.frame.px[i] = {frame[3 * i], frame[3 * i + 1], frame[3 * i + 2]};
    if (frameOnly) return true;
    r.g.resize(w, h);
    r.aoSS.resize(w, h);
    r.hdr.resize(w, h);
    if (opts.rtao) r.aoRT.resize(w, h);
    for (std::size_t i = 0; i < n; ++i) {
        const bool cov = mask[i] != 0;
        r.g.depth.px[i] = cov ? depth[i] : std::numeric_limits<float>::infinity();
        r.g.position.px[i] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        r.g.normal.px[i] = {nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]};
        r.g.albedo.px[i] = {albedo[3 * i], albedo[3 * i + 1], albedo[3 * i + 2]};
        r.g.mask.px[i] = cov ? 1 : 0;
        r.g.motion.px[i] = {motion[2 * i], motion[2 * i + 1]};
        r.aoSS.px[i] = ao_ss[i];
        if (opts.rtao) r.aoRT.px[i] = ao_rt[i];
        r.hdr.px[i] = {hdr[3 * i], hdr[3 * i + 1], hdr[3 * i + 2]};
    }
    r.motionValid = out.motion_valid;
    r.motionTotal = out.motion_total;
    r.rec.errorMap.resize(w, h);
    if (opts.rtao) {
        std::memcpy(r.rec.errorMap.px.data(), errmap.data(), n * sizeof(float));
        r.rec.rmse = out.rec.rmse;
        r.rec.maxError = out.rec.max_error;
        r.rec.pixels = out.rec.pixels;
        r.rec.withinTolerance = out.rec.within_tolerance != 0;
    }
    std::memcpy(r.viewProj.m, out.view_proj, sizeof r.viewProj.m);
    return true;
}

}  // namespace raw
