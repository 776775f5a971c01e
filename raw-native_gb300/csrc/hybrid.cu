// hybrid.cu -- closest-hit consumers of the AO path's BVH: the nearest-hit query of
// raw::rt::closest (src/renderer/rt_bvh.cpp:125-152) on the 4-wide tree, and the hybrid pass
// of raw::gpu_check::hybridGpu / cpuReference (src/renderer/gpu/rt_hybrid.cpp:43-83,
// src/renderer/gpu/rt_hybrid_parity.cpp:14-82): per covered G-buffer pixel a sun shadow ray
// (any hit) and a mirror reflection ray (closest hit, about the shading normal), both from
// an origin pushed off the surface along the geometric normal.
//
// Nearest hit: the smallest t > 1e-4 below t_max of the reference's watertight triangle test
// over all triangles, ties to the lowest triangle index, exactly as the reference's ordered
// walk defines it. The 4-wide walk visits children nearest first and culls a box only when
// its slab entry exceeds the best t found so far (with the same conservative padding and
// widened exit as the AO walk), so no triangle that could hold the answer is skipped, and
// the hit test is the AO path's: the answer is the scan's bit for bit.
#include "rn_internal.h"
#include "rn_device.cuh"
#include "trace_device.cuh"

namespace rn {
namespace {

using namespace trace_dev;

__global__ void closest_kernel(const Node4* __restrict__ nodes, const LeafTri* __restrict__ tris, int has_geometry,
                               const float* __restrict__ rays, const float* __restrict__ tmax, uint32_t n,
                               int32_t* __restrict__ tri, float* __restrict__ t_out, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const v3 o = load3(rays + (size_t)i * 6), d = load3(rays + (size_t)i * 6 + 3);
    float t = tmax[i];
    const int id = has_geometry ? walk_closest(nodes, tris, o, d, tmax[i], t, err) : -1;
    tri[i] = id;
    t_out[i] = id >= 0 ? t : -1.0f;
}

// rt_hybrid_parity.cpp:38-41: the origin pushed off the surface along the normal, toward the
// ray's side, by 2e-4 (1 + the position's largest magnitude).
__device__ __forceinline__ v3 offset_of(const v3& pos, const v3& ng, const v3& dir) {
    const float e = fmul(2e-4f, fadd(1.0f, fmaxf(fabsf(pos.x), fmaxf(fabsf(pos.y), fabsf(pos.z)))));
    return add(pos, scale(ng, dot(ng, dir) > 0.0f ? e : -e));
}

struct HybridArgs {
    int w, h;
    const float* pos;
    const float* nrm;
    const float* geo;     // geometric normals, or null: the G-buffer normals
    const uint8_t* mask;
    const Node4* nodes;
    const LeafTri* tris;
    int has_geometry;
    float ex, ey, ez;     // the eye
    float lx, ly, lz;     // toward the sun (normalized on the device)
    float* lit;           // 1 lit, 0 in shadow, -1 uncovered
    int32_t* refl_tri;    // the reflected triangle, -1 none
    float* refl_t;        // its t, -1 none
    uint32_t* err;
};

// rt_hybrid_parity.cpp:35-37, 57-80 over the library's G-buffer: d = normalize(pos - eye);
// the geometric normal faces the viewer and the shading normal lies on its side; lit = no
// hit toward the sun below 1e30; the reflection r = d - 2 (d.n) n and its nearest hit below
// 1e30; both origins pushed off along the geometric normal.
// A block covers 16 x 8 pixels, each warp an 8 x 4 packet: neighbouring rays share more of
// their walks than a 32-pixel row does.
// kMinBlocks: resident 128-thread blocks per SM asked of the register allocator (the
// walk's latency is hidden by more warps where the cap costs no spills).
template <int kMinBlocks>
__global__ void __launch_bounds__(128, kMinBlocks) hybrid_kernel(const HybridArgs a) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int x = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
    const int y = blockIdx.y * 8 + (warp >> 1) * 4 + (lane >> 3);
    if (x >= a.w || y >= a.h) return;
    const size_t i = (size_t)y * a.w + x;
    if (!a.mask[i]) {
        a.lit[i] = -1.0f;
        a.refl_tri[i] = -1;
        a.refl_t[i] = -1.0f;
        return;
    }
    const v3 pos = load3(a.pos + 3 * i);
    v3 n = load3(a.nrm + 3 * i);
    v3 ng = a.geo ? load3(a.geo + 3 * i) : n;
    const v3 d = normalize(sub(pos, mk(a.ex, a.ey, a.ez)));
    if (dot(ng, d) > 0.0f) ng = scale(ng, -1.0f);
    if (dot(n, ng) < 0.0f) n = scale(n, -1.0f);
    const v3 l = normalize(mk(a.lx, a.ly, a.lz));
    Counts cn;
    const bool shadow =
        a.has_geometry && walk<false>(a.nodes, a.tris, offset_of(pos, ng, l), l, 1e30f, 1e30f, a.err, cn) != 0;
    a.lit[i] = shadow ? 0.0f : 1.0f;
    const v3 r = sub(d, scale(n, fmul(2.0f, dot(d, n))));
    float t = 1e30f;
    const int id = a.has_geometry ? walk_closest(a.nodes, a.tris, offset_of(pos, ng, r), r, 1e30f, t, a.err) : -1;
    a.refl_tri[i] = id;
    a.refl_t[i] = id >= 0 ? t : -1.0f;
}

}  // namespace

int launch_closest(const Node4* nodes, const LeafTri* tris, int has_geometry, const float* rays, const float* tmax,
                   uint32_t n, int32_t* tri, float* t, uint32_t* err, cudaStream_t s) {
    if (n == 0) return RN_OK;
    closest_kernel<<<(n + 127) / 128, 128, 0, s>>>(nodes, tris, has_geometry, rays, tmax, n, tri, t, err);
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}

int launch_hybrid(int w, int h, const float* pos, const float* nrm, const float* geo_nrm, const uint8_t* mask,
                  const rn_accel* accel,
                  const float eye[3], const float to_sun[3], float* lit, int32_t* refl_tri, float* refl_t,
                  uint32_t* err, cudaStream_t s) {
    HybridArgs a{};
    a.w = w; a.h = h;
    a.pos = pos; a.nrm = nrm; a.geo = geo_nrm; a.mask = mask;
    a.nodes = accel->d_nodes; a.tris = accel->d_tris;
    a.has_geometry = accel->ntri > 0;
    a.ex = eye[0]; a.ey = eye[1]; a.ez = eye[2];
    a.lx = to_sun[0]; a.ly = to_sun[1]; a.lz = to_sun[2];
    a.lit = lit; a.refl_tri = refl_tri; a.refl_t = refl_t;
    a.err = err;
    const dim3 grid((w + 15) / 16, (h + 7) / 8);
    switch (ctx().tune.hybrid_min_blocks) {
        case 5: hybrid_kernel<5><<<grid, 128, 0, s>>>(a); break;
        case 8: hybrid_kernel<8><<<grid, 128, 0, s>>>(a); break;
        default: hybrid_kernel<6><<<grid, 128, 0, s>>>(a); break;
    }
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}

}  // namespace rn
