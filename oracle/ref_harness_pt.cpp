// ref_harness_pt.cpp -- extern "C" entry points over the reference's OWN path tracer.
//
// TEST INFRASTRUCTURE ONLY, compiled by oracle/Makefile into oracle/_ref/libref_ao.so with
// the reference's path-tracer sources read in place: raw::rt::pathTraceCpu
// (src/renderer/rt_pt_cpu.cpp), finishPtScene and the lit scenes (src/renderer/rt_pt_scene.cpp),
// and the lobe's energy table (src/renderer/rt_pt_energy.cpp). Tests use it to pin the C
// restatement (rn_oracle.c's rno_pathtrace) and to make the golden fixtures of
// tests/golden/ (the reference's own scenes and its outputs on them).
//
// The two pbr::Tables symbols defined at the end come from a file the reference's CMake
// generates (the anisotropic albedo table, embedded); that file is not built here. Only the
// v3 material model (raw::pbr::Tables) reads them, which a v2 scene never constructs: the
// stand-ins abort if ever called.
#include "raw/renderer/rt_pathtrace.hpp"
#include "raw/renderer/rt_scenes.hpp"
#include "raw/renderer/swr_scenes.hpp"
#include "raw/renderer/pbr.hpp"
#include "rt_pt_math.hpp"
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace raw;

namespace {

// The counterparts of rn_oracle.c's rno_pt_scene / rno_pt_desc (plain arrays, one layout).
struct PtSceneIn {
    const float* pos; const float* nrm; const float* uv; uint32_t nvert;
    const uint32_t* idx; const uint32_t* triTex; uint32_t ntri;
    const uint32_t* texEntries; uint32_t ntex;
    const uint32_t* texels; uint32_t ntexels;
    const float* materials;   // 7 floats each: baseFactor, roughness, metallic, specular, emission
    float sunDir[3], sunIrr[3], sky[3];
};
struct PtDescIn {
    uint64_t seed;
    uint32_t spp, sppBegin, maxBounces;
    int32_t width, height;
    float camera[10], previous[10];
    int32_t jitter, rr;
    uint32_t controls;   // bit 0 dropLambertCosine, 1 misWeightOne, 2 aovDropSpecularIndirect,
                         // 3 aovEmissionToDiffuse, 4 legacyLobeV2
};
struct PtOut {
    float *radiance, *albedo, *normal, *depth, *variance;
    int32_t* triangle;
    float* motion;
    float *diffuse, *specular, *emission, *diffuseAlbedo, *specularAlbedo, *diffuseVariance, *specularVariance;
};

rt::PtCamera cam(const float* c) {
    return {{c[0], c[1], c[2]}, {c[3], c[4], c[5]}, {c[6], c[7], c[8]}, c[9]};
}

rt::PtScene build(const PtSceneIn& in) {
    rt::PtScene s;
    s.name = "harness";
    for (uint32_t i = 0; i < in.nvert; ++i) {
        s.geo.pos.push_back({in.pos[3 * i], in.pos[3 * i + 1], in.pos[3 * i + 2]});
        s.geo.nrm.push_back({in.nrm[3 * i], in.nrm[3 * i + 1], in.nrm[3 * i + 2]});
        s.geo.uv.push_back({in.uv[2 * i], in.uv[2 * i + 1]});
    }
    s.geo.idx.assign(in.idx, in.idx + 3 * (std::size_t)in.ntri);
    s.geo.triTexture.assign(in.triTex, in.triTex + in.ntri);
    for (uint32_t t = 0; t < in.ntex; ++t)
        s.tex.entries.push_back({in.texEntries[3 * t], in.texEntries[3 * t + 1], in.texEntries[3 * t + 2]});
    s.tex.texels.assign(in.texels, in.texels + in.ntexels);
    for (uint32_t t = 0; t < in.ntex; ++t) {
        const float* m = in.materials + 7 * (std::size_t)t;
        s.materials.push_back({m[0], m[1], m[2], m[3], {m[4], m[5], m[6]}});
    }
    s.sunDir = {in.sunDir[0], in.sunDir[1], in.sunDir[2]};
    s.sunIrradiance = {in.sunIrr[0], in.sunIrr[1], in.sunIrr[2]};
    s.sky = {in.sky[0], in.sky[1], in.sky[2]};
    rt::finishPtScene(s);
    return s;
}

void copy(float* dst, const std::vector<float>& v) { if (dst) std::memcpy(dst, v.data(), v.size() * sizeof(float)); }

}  // namespace

extern "C" {

// The lobe's energy table, interface v4 (EnergyTable::kFloats floats: the (A, B) nodes, then
// each roughness row's cosine-weighted means).
__attribute__((visibility("default")))
int ref_pt_energy_table(float* out) {
    const rt::pt::EnergyTable& t = rt::pt::energyTable();
    if (out) std::memcpy(out, t.v.data(), t.v.size() * sizeof(float));
    return (int)t.v.size();
}

// The reference's lit scenes as plain arrays. name: retro_room, iso_street, dense_block,
// furnace (emission e, albedo a), white_plane (material 7 floats in `mat7`, sky `sky3`).
// counts[5] = nvert, ntri, ntex, ntexels, nemitters; call once with the arrays NULL for the
// sizes. light9 = sunDir, sunIrradiance, sky; cam10 = the scene's camera.
__attribute__((visibility("default")))
int ref_pt_scene(const char* name, float e, float a, const float* mat7, const float* sky3, uint32_t* counts,
                 float* pos, float* nrm, float* uv, uint32_t* idx, uint32_t* triTex, uint32_t* texEntries,
                 uint32_t* texels, float* materials, float* light9, float* cam10) {
    const std::string n(name);
    rt::PtScene s;
    rt::PtCamera c;
    if (n == "retro_room") { s = rt::ptRetroRoom(); c = rt::cameraOf(swr::retroRoom()); }
    else if (n == "iso_street") { s = rt::ptIsoStreet(); c = rt::cameraOf(swr::isoStreet()); }
    else if (n == "dense_block") { s = rt::ptDenseBlock(); c = rt::cameraOf(rt::denseBlock()); }
    else if (n == "furnace") { s = rt::ptFurnace(e, a); c = rt::cameraOf(rt::furnaceBox()); }
    else if (n == "white_plane") {
        s = rt::ptWhitePlane({mat7[0], mat7[1], mat7[2], mat7[3], {mat7[4], mat7[5], mat7[6]}}, {sky3[0], sky3[1], sky3[2]});
        c = rt::whitePlaneCamera();
    } else return -1;
    counts[0] = (uint32_t)s.geo.pos.size(); counts[1] = (uint32_t)s.geo.triangles();
    counts[2] = (uint32_t)s.tex.entries.size(); counts[3] = (uint32_t)s.tex.texels.size();
    counts[4] = (uint32_t)s.emitters.size();
    if (!pos) return 0;
    for (std::size_t i = 0; i < s.geo.pos.size(); ++i) {
        pos[3 * i] = s.geo.pos[i].x; pos[3 * i + 1] = s.geo.pos[i].y; pos[3 * i + 2] = s.geo.pos[i].z;
        nrm[3 * i] = s.geo.nrm[i].x; nrm[3 * i + 1] = s.geo.nrm[i].y; nrm[3 * i + 2] = s.geo.nrm[i].z;
        uv[2 * i] = s.geo.uv[i].x; uv[2 * i + 1] = s.geo.uv[i].y;
    }
    std::memcpy(idx, s.geo.idx.data(), s.geo.idx.size() * 4);
    std::memcpy(triTex, s.geo.triTexture.data(), s.geo.triTexture.size() * 4);
    for (std::size_t t = 0; t < s.tex.entries.size(); ++t) {
        texEntries[3 * t] = s.tex.entries[t].offset;
        texEntries[3 * t + 1] = s.tex.entries[t].width;
        texEntries[3 * t + 2] = s.tex.entries[t].height;
    }
    std::memcpy(texels, s.tex.texels.data(), s.tex.texels.size() * 4);
    for (std::size_t t = 0; t < s.tex.entries.size(); ++t) {
        const rt::PtMaterial& m = s.materials[t];
        const float v[7] = {m.baseFactor, m.roughness, m.metallic, m.specular, m.emission.x, m.emission.y, m.emission.z};
        std::memcpy(materials + 7 * t, v, sizeof v);
    }
    const float l[9] = {s.sunDir.x, s.sunDir.y, s.sunDir.z, s.sunIrradiance.x, s.sunIrradiance.y, s.sunIrradiance.z,
                        s.sky.x, s.sky.y, s.sky.z};
    std::memcpy(light9, l, sizeof l);
    const float cc[10] = {c.eye.x, c.eye.y, c.eye.z, c.target.x, c.target.y, c.target.z, c.up.x, c.up.y, c.up.z, c.fovy};
    std::memcpy(cam10, cc, sizeof cc);
    return 0;
}

// raw::rt::pathTraceCpu of a scene given as arrays (finishPtScene builds its tree, emitter list
// and CDF); every AOV is copied out (any pointer may be NULL). Returns the emitter count.
__attribute__((visibility("default")))
int ref_pathtrace(const PtSceneIn* in, const PtDescIn* di, int threads, PtOut* out) {
    const rt::PtScene s = build(*in);
    rt::PathTraceDesc d;
    d.seed = di->seed; d.spp = di->spp; d.sppBegin = di->sppBegin; d.maxBounces = di->maxBounces;
    d.width = di->width; d.height = di->height;
    d.camera = cam(di->camera); d.previous = cam(di->previous);
    d.jitter = di->jitter != 0; d.russianRoulette = di->rr != 0;
    d.controls.dropLambertCosine = (di->controls & 1u) != 0;
    d.controls.misWeightOne = (di->controls & 2u) != 0;
    d.controls.aovDropSpecularIndirect = (di->controls & 4u) != 0;
    d.controls.aovEmissionToDiffuse = (di->controls & 8u) != 0;
    d.controls.legacyLobeV2 = (di->controls & 16u) != 0;
    const rt::PathTraceOutput o = rt::pathTraceCpu(s, d, threads);
    copy(out->radiance, o.radiance); copy(out->albedo, o.albedo); copy(out->normal, o.normal);
    copy(out->depth, o.depth); copy(out->variance, o.variance); copy(out->motion, o.motion);
    if (out->triangle) std::memcpy(out->triangle, o.triangle.data(), o.triangle.size() * 4);
    copy(out->diffuse, o.diffuse); copy(out->specular, o.specular); copy(out->emission, o.emission);
    copy(out->diffuseAlbedo, o.diffuseAlbedo); copy(out->specularAlbedo, o.specularAlbedo);
    copy(out->diffuseVariance, o.diffuseVariance); copy(out->specularVariance, o.specularVariance);
    return (int)s.emitters.size();
}

}  // extern "C"

namespace raw::pbr {
const unsigned char* Tables::anisoBytes() { std::abort(); }
std::size_t Tables::anisoByteCount() { std::abort(); }
}  // namespace raw::pbr
