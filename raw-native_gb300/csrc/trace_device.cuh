// trace_device.cuh -- the AO walk and the per-pixel loop of the ray-traced pass, shared by
// the single-frame kernel (trace.cu) and the batched multi-view kernel (batch.cu). See
// trace.cu for the design and the exactness argument.
#pragma once
#include "rn_internal.h"
#include "rn_device.cuh"

namespace rn {
namespace trace_dev {


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
// The slab tests only prune, so 1/x need not be correctly rounded: the hardware reciprocal
// (rcp.approx, at most 1 ulp off) scales each axis's plane distances by at most 1 +- 2^-23,
// and a box the ray truly enters then still passes t0 <= t1 x (1 + 2^-22 or so), inside the
// test's exit widening of 1.0000008 (about 1 + 2^-20.2).
__device__ __forceinline__ float rcp_fast(float x) {
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float safe_inv(float x) { return x != 0.0f ? rcp_fast(x) : copysignf(__int_as_float(0x7f800000), x); }

// The ray's inverse direction and origin x inverse direction, formed once per walk.
struct Inv { float x, y, z, ox, oy, oz; };
__device__ __forceinline__ Inv make_inv(const v3& o, const v3& d) {
    Inv r;
    r.x = safe_inv(d.x); r.y = safe_inv(d.y); r.z = safe_inv(d.z);
    r.ox = o.x * r.x; r.oy = o.y * r.y; r.oz = o.z * r.z;
    return r;
}

// Slab entry of one child box, each plane distance as one fused multiply-add,
// lo * inv - o * inv. The BVH only prunes, so the test has to be conservative, not exact:
// against (lo - o) * inv the fused form is off by at most about 2^-24 |o| in position, far
// inside the child boxes' outward padding (2^-19 of the coordinate plus 1e-6 of the
// extent), so no box a triangle hit lies in is culled. An axis whose distances are NaN
// (origin on the plane, zero or vanishing direction component) constrains nothing, as in
// the reference's entry(); that only keeps more boxes.
__device__ __forceinline__ bool slab(float lox, float hix, float loy, float hiy, float loz, float hiz,
                                     const v3& o, const Inv& iv, float tmax, float& tnear) {
    (void)o;
    const float ax = __fmaf_rn(lox, iv.x, -iv.ox), bx = __fmaf_rn(hix, iv.x, -iv.ox);
    const float ay = __fmaf_rn(loy, iv.y, -iv.oy), by = __fmaf_rn(hiy, iv.y, -iv.oy);
    const float az = __fmaf_rn(loz, iv.z, -iv.oz), bz = __fmaf_rn(hiz, iv.z, -iv.oz);
    const float t0 = fmaxf(fmaxf(fmaxf(0.0f, min_nan(ax, bx)), min_nan(ay, by)), min_nan(az, bz));
    const float t1 = fminf(fminf(fminf(tmax, max_nan(ax, bx)), max_nan(ay, by)), max_nan(az, bz));
    tnear = t0;
    return t0 <= t1 * 1.0000008f;
}

// Per-thread traversal counters (the measurement build; compiled out otherwise).
struct Counts { unsigned long long rays = 0, nodes = 0, tris = 0, sky = 0; };

enum : int { HIT_NEAR = 1, HIT_FAR = 2 };

// A warp's frontier: BVH entries (a child word and its padded box) that together hold every
// triangle a short ray of the warp's tile can reach. A triangle hit at t < radius lies within
// radius of its ray's origin, so its leaf box, and every ancestor's, overlaps the box Q of
// the tile's origins grown by the radius; the frontier is the set of Q-overlapping nodes
// reached by expanding Q-overlapping nodes from the root, level by level, while at most
// kFrontier entries result. AO walks start from it instead of re-descending from the root.
constexpr int kFrontier = 16;
struct FrontierEntry {
    float lo[3], hi[3];
    int32_t word;
    int32_t pad;
};

__device__ __forceinline__ bool box_overlaps(float lx, float ly, float lz, float hx, float hy, float hz,
                                             const float* qlo, const float* qhi) {
    return lx <= qhi[0] && hx >= qlo[0] && ly <= qhi[1] && hy >= qlo[1] && lz <= qhi[2] && hz >= qlo[2];
}

// The warp builds the frontier of box [qlo, qhi] into F (all 32 lanes call it); returns its
// size (0: start at the root). Breadth first: each round every entry that is an interior
// node is replaced by its Q-overlapping children, the lanes expanding their entries in
// parallel (one node fetch per lane, a prefix sum over the lanes for the output slots),
// while the result stays within kFrontier entries. A round costs one dependent node fetch,
// so the build takes about the tree's depth in fetch latencies. Up to `tail` greedy steps
// follow, each replacing the largest interior entry by its children while the frontier fits.
__device__ inline int build_frontier(const Node4* __restrict__ nodes, const float* qlo, const float* qhi,
                                     FrontierEntry* F, int tail) {
    const int lane = (int)(threadIdx.x & 31u);
    int32_t word = 0;                       // lane 0 starts with the root node
    float lo[3] = {0.0f, 0.0f, 0.0f}, hi[3] = {0.0f, 0.0f, 0.0f};
    int n = 1, built = 0;
    for (int round = 0; round < 64; ++round) {
        const bool mine = lane < n;
        const bool inner = mine && word >= 0;
        const Node4* N = nodes + (inner ? word : 0);
        unsigned hit = 0;
        if (inner)
            for (int k = 0; k < N->meta[0]; ++k)
                if (box_overlaps(N->lox[k], N->loy[k], N->loz[k], N->hix[k], N->hiy[k], N->hiz[k], qlo, qhi))
                    hit |= 1u << k;
        const int c = inner ? __popc(hit) : (mine ? 1 : 0);
        int incl = c;
        for (int off = 1; off < 32; off <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        if (!__any_sync(0xffffffffu, inner) || total > kFrontier) break;
        __syncwarp();                       // every lane has read its entry of the last round
        int pos = incl - c;
        if (inner) {
            for (int k = 0; k < 4; ++k)
                if (hit & (1u << k)) {
                    FrontierEntry e;
                    e.lo[0] = N->lox[k]; e.lo[1] = N->loy[k]; e.lo[2] = N->loz[k];
                    e.hi[0] = N->hix[k]; e.hi[1] = N->hiy[k]; e.hi[2] = N->hiz[k];
                    e.word = N->child[k];
                    e.pad = 0;
                    F[pos++] = e;
                }
        } else if (mine) {
            FrontierEntry e;
            e.lo[0] = lo[0]; e.lo[1] = lo[1]; e.lo[2] = lo[2];
            e.hi[0] = hi[0]; e.hi[1] = hi[1]; e.hi[2] = hi[2];
            e.word = word;
            e.pad = 0;
            F[pos] = e;
        }
        __syncwarp();
        n = total;
        built = 1;
        if (lane < n) {
            const FrontierEntry& e = F[lane];
            lo[0] = e.lo[0]; lo[1] = e.lo[1]; lo[2] = e.lo[2];
            hi[0] = e.hi[0]; hi[1] = e.hi[1]; hi[2] = e.hi[2];
            word = e.word;
        }
    }
    // then up to `tail` single steps, largest interior entry first, while the result fits
    for (int step = 0; built && step < tail; ++step) {
        const bool inner = lane < n && word >= 0;
        float best = inner ? fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]) : -1.0f;
        int bl = lane;
        for (int off = 16; off > 0; off >>= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best, off);
            const int ol = __shfl_xor_sync(0xffffffffu, bl, off);
            if (ob > best || (ob == best && ol < bl)) { best = ob; bl = ol; }
        }
        if (best < 0.0f) break;
        unsigned hit = 0;
        const Node4* N = nodes + (lane == bl ? word : 0);
        if (lane == bl)
            for (int k = 0; k < N->meta[0]; ++k)
                if (box_overlaps(N->lox[k], N->loy[k], N->loz[k], N->hix[k], N->hiy[k], N->hiz[k], qlo, qhi))
                    hit |= 1u << k;
        const int c = __popc(__shfl_sync(0xffffffffu, hit, bl));
        if (n - 1 + c > kFrontier) break;
        __syncwarp();
        if (lane == bl) {
            // the children replace entry bl and append after the last entry; none: the last
            // entry moves into slot bl
            int pos = bl;
            if (c == 0 && bl != n - 1) F[bl] = F[n - 1];
            for (int k = 0; k < 4; ++k)
                if (hit & (1u << k)) {
                    FrontierEntry e;
                    e.lo[0] = N->lox[k]; e.lo[1] = N->loy[k]; e.lo[2] = N->loz[k];
                    e.hi[0] = N->hix[k]; e.hi[1] = N->hiy[k]; e.hi[2] = N->hiz[k];
                    e.word = N->child[k];
                    e.pad = 0;
                    F[pos] = e;
                    pos = pos == bl ? n : pos + 1;
                }
        }
        __syncwarp();
        n = n - 1 + c;
        if (lane < n) {
            const FrontierEntry& e = F[lane];
            lo[0] = e.lo[0]; lo[1] = e.lo[1]; lo[2] = e.lo[2];
            hi[0] = e.hi[0]; hi[1] = e.hi[1]; hi[2] = e.hi[2];
            word = e.word;
        }
    }
    return built ? n : 0;
}

// One walk, two limits (tnear <= tfar): HIT_NEAR | HIT_FAR when some triangle is hit at
// 1e-4 < t < tnear; HIT_FAR alone when the nearest hit it needed to find lies in
// [tnear, tfar); 0 when nothing is hit before tfar. The any-hit query of raw::Bvh::occluded
// (src/renderer/bvh.cpp:119-138) is tnear == tfar.
// kLeafPass: a node's leaf children are tested after all four slab tests, in one loop over
// the leaves that passed (lanes whose leaves sit at different child positions test them
// together, and the triangle test exists once in the code instead of once per position).
// Either order finds the same answers: boxes are only culled against tmax >= tnear, and a
// far hit only lowers tmax to tnear.
template <bool kCount, int kStackN = kStack, bool kLeafPass = false>
__device__ int walk(const Node4* __restrict__ nodes, const LeafTri* __restrict__ tris, const v3& o, const v3& d,
                    float tnear, float tfar, uint32_t* err, Counts& cn, const FrontierEntry* F = nullptr,
                    int fn = 0) {
    const Inv iv = make_inv(o, d);
    WRay wr;                             // the watertight set-up: formed at the first leaf
    bool wr_ready = false;
    float tmax = tfar;
    int far_hit = 0;
    int32_t stack[kStackN];
    int sp = 0;
    int32_t cur = 0;                     // the root is always node 0
    if (fn > 0) {
        // start from the frontier: its entries are the root's stand-ins
        int32_t nearest = -1;
        float tbest = 3.0e38f;
        for (int e = 0; e < fn; ++e) {
            float tn;
            if (!slab(F[e].lo[0], F[e].hi[0], F[e].lo[1], F[e].hi[1], F[e].lo[2], F[e].hi[2], o, iv, tmax, tn)) continue;
            const int32_t c = F[e].word;
            if (c < 0) {
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
            int32_t push = c;
            if (tn < tbest) { push = nearest; nearest = c; tbest = tn; }
            stack[sp++] = push;                  // fn <= kFrontier < kStackN
        }
        if (nearest >= 0) cur = nearest;
        else if (sp > 0) cur = stack[--sp];
        else return far_hit;
    }
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
        unsigned leaves = 0;                  // kLeafPass: child positions of leaves to test
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            float tn;
            if (k >= cnt || !slab(LX[k], HX[k], LY[k], HY[k], LZ[k], HZ[k], o, iv, tmax, tn)) continue;
            const int32_t c = CH[k];
            if (kLeafPass && c < 0) { leaves |= 1u << k; continue; }
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
            if (sp >= kStackN) { atomicOr(err, DEV_STACK_OVERFLOW); return far_hit; }
            stack[sp++] = push;
        }
        if (kLeafPass)
            while (leaves) {
                const int k = __ffs(leaves) - 1;
                leaves &= leaves - 1u;
                const int32_t c = k == 0 ? ch.x : k == 1 ? ch.y : k == 2 ? ch.z : ch.w;
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
            }
        if (nearest >= 0) { cur = nearest; continue; }
        if (sp == 0) return far_hit;
        cur = stack[--sp];
    }
    atomicOr(err, DEV_GUARD);
    return far_hit;
}

// The nearest hit of raw::rt::closest (src/renderer/rt_bvh.cpp:125-152): the smallest t of the
// watertight test with 1e-4 < t < tmax, ties to the lowest triangle index (leaf triangles carry
// their input index). Children are visited nearest entry first; a box is culled only when its
// (padded, exit-widened) slab entry passes the best t so far, so the answer is the scan's.
__device__ inline int walk_closest(const Node4* __restrict__ nodes, const LeafTri* __restrict__ tris, const v3& o,
                            const v3& d, float tmax, float& t_hit, uint32_t* err) {
    const Inv iv = make_inv(o, d);
    const WRay wr = make_wray(o, d);
    float best = tmax;
    int best_tri = -1;
    int32_t stack[kStack];
    int sp = 0;
    int32_t cur = 0;
    for (uint32_t guard = 0; guard < kGuard; ++guard) {
        const float4* q = reinterpret_cast<const float4*>(nodes + cur);
        const float4 lx = __ldg(q + 0), hx = __ldg(q + 1), ly = __ldg(q + 2), hy = __ldg(q + 3);
        const float4 lz = __ldg(q + 4), hz = __ldg(q + 5);
        const int4 ch = __ldg(reinterpret_cast<const int4*>(q + 6));
        const int cnt = __ldg(reinterpret_cast<const int*>(q + 7));
        const float LX[4] = {lx.x, lx.y, lx.z, lx.w}, HX[4] = {hx.x, hx.y, hx.z, hx.w};
        const float LY[4] = {ly.x, ly.y, ly.z, ly.w}, HY[4] = {hy.x, hy.y, hy.z, hy.w};
        const float LZ[4] = {lz.x, lz.y, lz.z, lz.w}, HZ[4] = {hz.x, hz.y, hz.z, hz.w};
        const int32_t CH[4] = {ch.x, ch.y, ch.z, ch.w};
        // interior children that the ray enters before `best`, nearest first
        int32_t kid[4];
        float kt[4];
        int nk = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            float tn;
            if (k >= cnt || !slab(LX[k], HX[k], LY[k], HY[k], LZ[k], HZ[k], o, iv, best, tn)) continue;
            const int32_t c = CH[k];
            if (c < 0) {
                const uint32_t u = (uint32_t)~c;
                const uint32_t first = u >> 3, count = (u & 7u) + 1u;
                for (uint32_t i = 0; i < count; ++i) {
                    const float4* tq = reinterpret_cast<const float4*>(tris + first + i);
                    const float4 A = __ldg(tq), B = __ldg(tq + 1), C = __ldg(tq + 2);
                    float t;
                    if (!hit_tri(wr, mk(A.x, A.y, A.z), mk(B.x, B.y, B.z), mk(C.x, C.y, C.z), t)) continue;
                    const int id = __float_as_int(A.w);
                    if (t < best || (best_tri >= 0 && t == best && id < best_tri)) {
                        best = t;
                        best_tri = id;
                    }
                }
                continue;
            }
            int j = nk++;
            while (j > 0 && kt[j - 1] < tn) { kt[j] = kt[j - 1]; kid[j] = kid[j - 1]; --j; }
            kt[j] = tn;
            kid[j] = c;
        }
        // push the farther children, descend into the nearest
        for (int j = 0; j + 1 < nk; ++j) {
            if (sp >= kStack) { atomicOr(err, DEV_STACK_OVERFLOW); t_hit = best; return best_tri; }
            stack[sp++] = kid[j];
        }
        if (nk > 0) { cur = kid[nk - 1]; continue; }
        // pop the next pushed node: its children meet the best hit found since
        if (sp == 0) { t_hit = best; return best_tri; }
        cur = stack[--sp];
    }
    atomicOr(err, DEV_GUARD);
    t_hit = best;
    return best_tri;
}

// The frontier of the warp's tile for AO walks of `radius` (all 32 lanes call it and build
// it together). Returns its size, 0 when the tile has no covered pixel.
__device__ __forceinline__ int tile_frontier(const TraceParams& p, int x, int y, bool valid, FrontierEntry* F) {
    float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f}, mag = 0.0f;
    if (valid) {
        const size_t i = (size_t)y * p.w + x;
        if (p.mask[i]) {
            const v3 P = load3(p.pos + 3 * i), n = load3(p.nrm + 3 * i);
            const v3 o = add(P, scale(n, 1e-3f));
            lo[0] = hi[0] = o.x; lo[1] = hi[1] = o.y; lo[2] = hi[2] = o.z;
            mag = fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fabsf(o.z));
        }
    }
    for (int off = 16; off > 0; off >>= 1)
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], off));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], off));
        }
    for (int off = 16; off > 0; off >>= 1) mag = fmaxf(mag, __shfl_xor_sync(0xffffffffu, mag, off));
    if (lo[0] > hi[0]) return 0;
    // grow by the radius with margin for the rounding of t, |d| and the hit point
    const float g = p.radius * 1.0001f + 1e-5f * (mag + 1.0f);
    for (int a = 0; a < 3; ++a) { lo[a] -= g; hi[a] += g; }
    const int n = build_frontier(p.nodes, lo, hi, F, p.frontier_tail);
    __syncwarp();
    return n;
}

// Hemisphere direction of sample s of pixel (ux, uy) with frame (t, b, n): the arithmetic of
// trace_pixel's loop below (src/renderer/ray_ao.cpp:30-37), for callers that trace one
// sample per thread.
__device__ __forceinline__ v3 sample_direction(const v3& t, const v3& b, const v3& n, uint32_t ux, uint32_t uy,
                                               uint32_t s, const uint8_t* __restrict__ corr) {
    const uint32_t k2 = hash24(ux, uy, 2u * s + 1u);
    const float u1 = unit24(hash24(ux, uy, 2u * s));
    float c, sn;
    angle_sincos(sample_angle(k2), sn, c);
    if (corr) apply_corr(__ldg(corr + k2), c, sn);
    const float r = fsqrt(u1);
    const float lx = fmul(r, c), ly = fmul(r, sn);
    const float lz = fsqrt(smax(0.0f, fsub(1.0f, u1)));
    return normalize(add(add(scale(t, lx), scale(b, ly)), scale(n, lz)));
}

// One pixel: its spp cosine-weighted rays (AO and, when asked, the sky), then the sun ray.
template <bool kCount, int kStackN = kStack, bool kLeafPass = false>
__device__ __forceinline__ void trace_pixel(const TraceParams& p, int x, int y, const v3& toLight, Counts& cn,
                                            const FrontierEntry* F = nullptr, int fn = 0) {
    const float kFar = 1e30f;
    const size_t i = (size_t)y * p.w + x;
    const uint8_t m = p.mask[i];
    const v3 P = load3(p.pos + 3 * i), n = load3(p.nrm + 3 * i);
    if (p.mirror) {
        const size_t np = (size_t)p.w * p.h;
        store3(mirror_pos(p.mirror, np) + 3 * i, P);
        store3(mirror_nrm(p.mirror, np) + 3 * i, n);
        mirror_mask(p.mirror, np)[i] = m;
        if (!m) mirror_ao(p.mirror, np)[i] = 1.0f;
    }
    if (!m) {
        p.ao[i] = 1.0f;
        if (p.want_sky) { p.sky[i] = 1.0f; p.sun[i] = 1.0f; }
        return;
    }
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
        // AO-only walks may start from the warp's frontier; the sky and the sun need the root
        const bool local = s < p.spp && tf == p.radius;
        const int h = p.has_geometry ? walk<kCount, kStackN, kLeafPass>(p.nodes, p.tris, origin, dir, tn, tf, p.err_word,
                                                               cn, local ? F : nullptr, local ? fn : 0)
                                     : 0;
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
    if (p.mirror) mirror_ao(p.mirror, (size_t)p.w * p.h)[i] = p.ao[i];
    if (p.want_sky) {
        p.sky[i] = fdiv((float)freec, (float)p.spp);
        p.sun[i] = lit ? 1.0f : 0.0f;
    }
}


}  // namespace trace_dev
}  // namespace rn
