// trace.cu -- ray-traced AO and lighting model 2's visibility on the GPU: the hot loop of
// raw-native's CPU oracle (src/renderer/ray_ao.cpp:20-51) as one persistent kernel.
//
// Work: the frame is cut into 8 x 4 pixel tiles; each warp takes the next tile from a global
// counter, one pixel per lane, and walks its `spp` hemisphere rays, then the sun ray,
// through the 4-wide BVH. Neighbouring lanes trace neighbouring pixels, so the warp's rays
// start close together and visit similar nodes.
//
// One walk per hemisphere ray answers both of the reference's questions about it: a hit
// with t < radius (AO, ray_ao.cpp:39) and, for an open ray, a hit at any distance (sky,
// :41). The walk starts with the far limit and, once it has found a hit beyond the radius,
// keeps looking only for hits nearer than the radius; every box either query could need is
// visited, so both answers are the reference's. The sun ray is the last slot of the same
// loop, so the kernel holds one copy of the walk.
//
// Exactness: ray generation (basis, origin, cosine-weighted direction) and the triangle test
// use one IEEE rounding per operation in the reference's order; the sample angle's cos/sin
// carry the host libm's bits (rn_device.cuh). The box test is only required to be
// conservative, and is: padded boxes, the robust slab exit of Ize (2013) widened by
// 1.0000008, and NaN-safe min/max, so the any-hit answers are exactly the
// scan-every-triangle answers the reference's own BVH reproduces.
#include "rn_internal.h"
#include "rn_device.cuh"

namespace rn {
namespace {

constexpr int kStack = 96;
constexpr uint32_t kGuard = 1u << 24;       // node visits per ray before giving up
constexpr int kTileW = 8, kTileH = 4;

__device__ __forceinline__ float min_nan(float a, float b) {
    float r;
    asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float max_nan(float a, float b) {
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
// inverse(d) of src/renderer/bvh.cpp:29-33: 1/x, or a signed infinity for a zero component.
__device__ __forceinline__ float safe_inv(float x) { return x != 0.0f ? __frcp_rn(x) : copysignf(__int_as_float(0x7f800000), x); }

struct Inv { float x, y, z; };
__device__ __forceinline__ Inv make_inv(const v3& d) { return Inv{safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)}; }

// Slab entry of one child box. An axis whose distances are NaN (origin on the plane, zero
// direction component) constrains nothing, as in the reference's entry().
__device__ __forceinline__ bool slab(float lox, float hix, float loy, float hiy, float loz, float hiz,
                                     const v3& o, const Inv& iv, float tmax, float& tnear) {
    const float ax = (lox - o.x) * iv.x, bx = (hix - o.x) * iv.x;
    const float ay = (loy - o.y) * iv.y, by = (hiy - o.y) * iv.y;
    const float az = (loz - o.z) * iv.z, bz = (hiz - o.z) * iv.z;
    const float t0 = fmaxf(fmaxf(fmaxf(0.0f, min_nan(ax, bx)), min_nan(ay, by)), min_nan(az, bz));
    const float t1 = fminf(fminf(fminf(tmax, max_nan(ax, bx)), max_nan(ay, by)), max_nan(az, bz));
    tnear = t0;
    return t0 <= t1 * 1.0000008f;
}

// Per-thread traversal counters (the measurement build; compiled out otherwise).
struct Counts { unsigned long long rays = 0, nodes = 0, tris = 0, sky = 0; };

enum : int { HIT_NEAR = 1, HIT_FAR = 2 };

// One walk, two limits (tnear <= tfar): HIT_NEAR | HIT_FAR when some triangle is hit at
// 1e-4 < t < tnear; HIT_FAR alone when the nearest hit it needed to find lies in
// [tnear, tfar); 0 when nothing is hit before tfar. The any-hit query of raw::Bvh::occluded
// (src/renderer/bvh.cpp:119-138) is tnear == tfar.
template <bool kCount>
__device__ int walk(const Node4* __restrict__ nodes, const LeafTri* __restrict__ tris, const v3& o, const v3& d,
                    float tnear, float tfar, uint32_t* err, Counts& cn) {
    const Inv iv = make_inv(d);
    WRay wr;                             // the watertight set-up: formed at the first leaf
    bool wr_ready = false;
    float tmax = tfar;
    int far_hit = 0;
    int32_t stack[kStack];
    int sp = 0;
    int32_t cur = 0;                     // the root is always node 0
    for (uint32_t guard = 0; guard < kGuard; ++guard) {
        if (kCount) ++cn.nodes;
        const float4* q = reinterpret_cast<const float4*>(nodes + cur);
        const float4 lx = __ldg(q + 0), hx = __ldg(q + 1), ly = __ldg(q + 2), hy = __ldg(q + 3);
        const float4 lz = __ldg(q + 4), hz = __ldg(q + 5);
        const int4 ch = __ldg(reinterpret_cast<const int4*>(q + 6));
        const int cnt = __ldg(reinterpret_cast<const int*>(q + 7));
        const float LX[4] = {lx.x, lx.y, lx.z, lx.w}, HX[4] = {hx.x, hx.y, hx.z, hx.w};
        const float LY[4] = {ly.x, ly.y, ly.z, ly.w}, HY[4] = {hy.x, hy.y, hy.z, hy.w};
        const float LZ[4] = {lz.x, lz.y, lz.z, lz.w}, HZ[4] = {hz.x, hz.y, hz.z, hz.w};
        const int32_t CH[4] = {ch.x, ch.y, ch.z, ch.w};
        int32_t nearest = -1;
        float tbest = 3.0e38f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            float tn;
            if (k >= cnt || !slab(LX[k], HX[k], LY[k], HY[k], LZ[k], HZ[k], o, iv, tmax, tn)) continue;
            const int32_t c = CH[k];
            if (c < 0) {
                // a leaf: test its triangles now (a near hit ends the walk)
                if (!wr_ready) { wr = make_wray(o, d); wr_ready = true; }
                const uint32_t w = (uint32_t)~c;
                const uint32_t first = w >> 3, count = (w & 7u) + 1u;
                for (uint32_t i = 0; i < count; ++i) {
                    if (kCount) ++cn.tris;
                    const float4* tq = reinterpret_cast<const float4*>(tris + first + i);
                    const float4 A = __ldg(tq), B = __ldg(tq + 1), C = __ldg(tq + 2);
                    float t;
                    if (!hit_tri(wr, mk(A.x, A.y, A.z), mk(B.x, B.y, B.z), mk(C.x, C.y, C.z), t)) continue;
                    if (t < tnear) return HIT_NEAR | HIT_FAR;
                    if (t < tmax) { far_hit = HIT_FAR; tmax = tnear; }
                }
                continue;
            }
            if (nearest < 0) { nearest = c; tbest = tn; continue; }
            // keep the nearer child to descend into, stack the other
            int32_t push = c;
            if (tn < tbest) { push = nearest; nearest = c; tbest = tn; }
            if (sp >= kStack) { atomicOr(err, DEV_STACK_OVERFLOW); return far_hit; }
            stack[sp++] = push;
        }
        if (nearest >= 0) { cur = nearest; continue; }
        if (sp == 0) return far_hit;
        cur = stack[--sp];
    }
    atomicOr(err, DEV_GUARD);
    return far_hit;
}

// One pixel: its spp cosine-weighted rays (AO and, when asked, the sky), then the sun ray.
template <bool kCount>
__device__ __forceinline__ void trace_pixel(const TraceParams& p, int x, int y, const v3& toLight, Counts& cn) {
    const float kFar = 1e30f;
    const size_t i = (size_t)y * p.w + x;
    if (!p.mask[i]) {
        p.ao[i] = 1.0f;
        if (p.want_sky) { p.sky[i] = 1.0f; p.sun[i] = 1.0f; }
        return;
    }
    const v3 P = load3(p.pos + 3 * i), n = load3(p.nrm + 3 * i);
    // basis (ray_ao.cpp:14-17)
    const v3 a = fabsf(n.x) > 0.9f ? mk(0.0f, 1.0f, 0.0f) : mk(1.0f, 0.0f, 0.0f);
    const v3 t = normalize(cross(a, n)), b = cross(n, t);
    const v3 origin = add(P, scale(n, 1e-3f));
    const uint32_t ux = (uint32_t)x, uy = (uint32_t)y;
    const float tfar_h = p.want_sky ? kFar : p.radius;
    const int slots = p.spp + ((p.want_sky && !p.sun_forced) ? 1 : 0);
    int open = 0, freec = 0;
    bool lit = true;
    // the correction byte of the next sample is fetched one iteration ahead
    uint32_t k2n = hash24(ux, uy, 1u);
    int cbn = p.corr ? __ldg(p.corr + k2n) : 0;
    for (int s = 0; s < slots; ++s) {
        v3 dir;
        float tn, tf;
        if (s < p.spp) {
            const uint32_t k2 = k2n;
            const int cb = cbn;
            if (s + 1 < p.spp) {
                k2n = hash24(ux, uy, (uint32_t)(2 * s + 3));
                cbn = p.corr ? __ldg(p.corr + k2n) : 0;
            }
            const float u1 = unit24(hash24(ux, uy, (uint32_t)(2 * s)));
            float c, sn;
            angle_sincos(sample_angle(k2), sn, c);
            if (p.corr) apply_corr(cb, c, sn);
            const float r = fsqrt(u1);
            const float lx = fmul(r, c), ly = fmul(r, sn);
            const float lz = fsqrt(smax(0.0f, fsub(1.0f, u1)));
            dir = normalize(add(add(scale(t, lx), scale(b, ly)), scale(n, lz)));
            tn = p.radius;
            tf = tfar_h;
        } else {
            dir = toLight;
            tn = tf = kFar;
        }
        const int h = p.has_geometry ? walk<kCount>(p.nodes, p.tris, origin, dir, tn, tf, p.err_word, cn) : 0;
        if (s < p.spp) {
            if (kCount) { ++cn.rays; if (p.want_sky && !(h & HIT_NEAR)) ++cn.sky; }
            if (!(h & HIT_NEAR)) {
                ++open;
                if (!(h & HIT_FAR)) ++freec;
            }
        } else {
            lit = h == 0;
        }
    }
    p.ao[i] = fdiv((float)open, (float)p.spp);
    if (p.want_sky) {
        p.sky[i] = fdiv((float)freec, (float)p.spp);
        p.sun[i] = lit ? 1.0f : 0.0f;
    }
}

// kCount: trace only every `stride`-th tile and add the rays, node fetches and triangle
// fetches to counts[0..3] (hemisphere rays, nodes, tris, sky continuations); the outputs of
// the other tiles are left unwritten. "Sky continuations" are the open hemisphere rays whose
// walk went on past the radius: the same walk serves both queries.
template <bool kCount, int kMinBlocks>
__global__ void __launch_bounds__(256, kMinBlocks) trace_kernel(const __grid_constant__ TraceParams p, uint32_t* tile_ctr,
                                                                unsigned long long* counts, uint32_t stride) {
    const int tiles_x = (p.w + kTileW - 1) / kTileW, tiles_y = (p.h + kTileH - 1) / kTileH;
    const uint32_t ntiles = (uint32_t)tiles_x * tiles_y;
    const unsigned lane = threadIdx.x & 31u;
    Counts cn;
    // lighting model 2's sun direction, normalized on the device as computeRTVisibility does
    const v3 toLight = normalize(mk(p.lx, p.ly, p.lz));
    while (true) {
        uint32_t tile = 0;
        if (lane == 0) tile = atomicAdd(tile_ctr, 1u);
        tile = __shfl_sync(0xffffffffu, tile, 0);
        if (tile >= ntiles) break;
        const int x = (int)(tile % tiles_x) * kTileW + (int)(lane % kTileW);
        const int y = (int)(tile / tiles_x) * kTileH + (int)(lane / kTileW);
        // no lane leaves the loop body early: the next tile fetch is a full-warp shuffle
        if (kCount && tile % stride != 0) continue;
        if (x < p.w && y < p.h) trace_pixel<kCount>(p, x, y, toLight, cn);
    }
    if (kCount) {
        atomicAdd(counts, cn.rays);
        atomicAdd(counts + 1, cn.nodes);
        atomicAdd(counts + 2, cn.tris);
        atomicAdd(counts + 3, cn.sky);
    }
}

__global__ void occluded_kernel(const Node4* __restrict__ nodes, const LeafTri* __restrict__ tris, int has_geometry,
                                const float* __restrict__ rays, const float* __restrict__ tmax, uint32_t n,
                                uint8_t* __restrict__ hit, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const v3 o = load3(rays + (size_t)i * 6), d = load3(rays + (size_t)i * 6 + 3);
    Counts cn;
    const float tm = tmax[i];
    hit[i] = (has_geometry && walk<false>(nodes, tris, o, d, tm, tm, err, cn) != 0) ? 1 : 0;
}

}  // namespace

// Residency variants: the register budget decides how many 256-thread blocks share an SM
// (2: up to 128 registers, 3: 80, 4: 64, with spills to L1). The launch uses enough
// blocks to fill every SM at that residency; ctx().tune.trace_min_blocks picks the variant.
template <int kMB>
void launch_variant(const TraceParams& p, int sm_count, cudaStream_t s, uint32_t* tile_ctr, unsigned long long* counts,
                    uint32_t stride) {
    const int blocks = sm_count * kMB;
    if (counts)
        trace_kernel<true, kMB><<<blocks, 256, 0, s>>>(p, tile_ctr, counts, stride < 1 ? 1 : stride);
    else
        trace_kernel<false, kMB><<<blocks, 256, 0, s>>>(p, tile_ctr, nullptr, 1);
}

int launch_trace(const TraceParams& p, int sm_count, cudaStream_t s, unsigned long long* counts, uint32_t stride) {
    // the tile counter sits in the word after the error word
    uint32_t* tile_ctr = p.err_word + 1;
    cudaMemsetAsync(tile_ctr, 0, 4, s);
    switch (ctx().tune.trace_min_blocks) {
        case 2: launch_variant<2>(p, sm_count, s, tile_ctr, counts, stride); break;
        case 4: launch_variant<4>(p, sm_count, s, tile_ctr, counts, stride); break;
        default: launch_variant<3>(p, sm_count, s, tile_ctr, counts, stride); break;
    }
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}

int launch_occluded(const Node4* nodes, const LeafTri* tris, int has_geometry, const float* rays, const float* tmax,
                    uint32_t n, uint8_t* hit, uint32_t* err_word, cudaStream_t s) {
    if (n == 0) return RN_OK;
    occluded_kernel<<<(n + 255) / 256, 256, 0, s>>>(nodes, tris, has_geometry, rays, tmax, n, hit, err_word);
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}

}  // namespace rn
