// accel_shim.cpp -- optional replacement of src/renderer/accel.cpp for the GPU build.
//
// LinearAccel::build keeps the triangle list in the arena exactly as the reference does
// (so the arena certificate is unchanged) but builds no CPU BVH: the AO passes trace the
// GPU accelerator (ao_shim.cpp). occluded() answers through the GPU too; occludedScan() is
// the reference's scan of every triangle, its test oracle, unchanged in meaning.
#include "raw/renderer/accel.hpp"
#include "ao_shim_internal.hpp"
#include "rn_ao.h"

#include <cstdlib>
#include <cstring>

namespace raw {
namespace {
// RAW_NATIVE_AO_ORACLE selects the test modes (src/renderer/accel.cpp:6-11).
LinearAccel::Mode modeFromEnvironment() {
    const char* v = std::getenv("RAW_NATIVE_AO_ORACLE");
    if (v && std::strcmp(v, "scan") == 0) return LinearAccel::Mode::Scan;
    if (v && std::strcmp(v, "skew") == 0) return LinearAccel::Mode::Skew;
    return LinearAccel::Mode::Bvh;
}
}  // namespace

void LinearAccel::build(const Scene& s, Arena* arena) {
    tris = std::vector<Tri, ArenaAllocator<Tri>>(ArenaAllocator<Tri>(arena));
    std::size_t count = 0;
    for (const Mesh& m : s.meshes) count += m.indices.size() / 3;
    tris.reserve(count);
    for (const Mesh& m : s.meshes)
        for (std::size_t i = 0; i + 2 < m.indices.size(); i += 3)
            tris.push_back(Tri{m.positions[m.indices[i]], m.positions[m.indices[i + 1]], m.positions[m.indices[i + 2]]});
    mode = modeFromEnvironment();
}

bool LinearAccel::occluded(const Ray& r, float maxDist) const {
    const float ray[6] = {r.o.x, r.o.y, r.o.z, r.d.x, r.d.y, r.d.z};
    const float tmax = mode == Mode::Skew ? maxDist * 0.99f : maxDist;
    std::uint8_t hit = 0;
    rn_status st{};
    if (rn_occluded(gpu_shim::accelOf(*this), ray, &tmax, 1, 0, &hit, &st) != RN_OK)
        gpu_shim::fail("LinearAccel::occluded", st);
    return hit != 0;
}

bool LinearAccel::occludedScan(const Ray& r, float maxDist) const {
    float t, u, v;
    for (const Tri& tri : tris)
        if (intersectTri(r, tri, t, u, v) && t < maxDist) return true;
    return false;
}

}  // namespace raw
