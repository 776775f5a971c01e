// trace.cu -- ray-traced AO and lighting model 2's visibility on the GPU: the hot loop of
// raw-native's CPU oracle (src/renderer/ray_ao.cpp:20-51) as one persistent kernel.
//
// Work: the frame is cut into packets of 32 pixels (8 x 4 by default; 4 x 8 and 16 x 2 are
// the autotuner's alternatives); each warp takes the next packet from a global counter, one
// pixel per lane, and walks its `spp` hemisphere rays, then the sun ray,
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
#include "trace_device.cuh"

namespace rn {
namespace {

using namespace trace_dev;

// kCount: trace only every `stride`-th tile and add the rays, node fetches and triangle
// fetches to counts[0..3] (hemisphere rays, nodes, tris, sky continuations); the outputs of
// the other tiles are left unwritten. "Sky continuations" are the open hemisphere rays whose
// walk went on past the radius: the same walk serves both queries.
template <bool kCount, int kMinBlocks, int kStackN, bool kLeafPass = false>
__global__ void __launch_bounds__(256, kMinBlocks) trace_kernel(const __grid_constant__ TraceParams p, uint32_t* tile_ctr,
                                                                unsigned long long* counts, uint32_t stride) {
    const int pl = p.packet_log2, tw = 1 << pl, th = 32 >> pl;
    const int tiles_x = (p.w + tw - 1) >> pl, tiles_y = (p.h + th - 1) / th;
    const uint32_t ntiles = (uint32_t)tiles_x * tiles_y;
    const unsigned lane = threadIdx.x & 31u;
    __shared__ FrontierEntry frontier[8][kFrontier];
    FrontierEntry* F = frontier[threadIdx.x >> 5];
    Counts cn;
    // lighting model 2's sun direction, normalized on the device as computeRTVisibility does
    const v3 toLight = normalize(mk(p.lx, p.ly, p.lz));
    while (true) {
        uint32_t tile = 0;
        if (lane == 0) tile = atomicAdd(tile_ctr, 1u);
        tile = __shfl_sync(0xffffffffu, tile, 0);
        if (tile >= ntiles) break;
        const int x = ((int)(tile % tiles_x) << pl) + (int)(lane & (tw - 1));
        const int y = (int)(tile / tiles_x) * th + (int)(lane >> pl);
        // no lane leaves the loop body early: the next tile fetch is a full-warp shuffle
        if (kCount && tile % stride != 0) continue;
        const int fn = (!p.want_sky && p.has_geometry && p.frontier) ? tile_frontier(p, x, y, x < p.w && y < p.h, F) : 0;
        if (x < p.w && y < p.h) trace_pixel<kCount, kStackN, kLeafPass>(p, x, y, toLight, cn, F, fn);
        __syncwarp();                              // the frontier is rebuilt for the next tile
    }
    if (kCount) {
        atomicAdd(counts, cn.rays);
        atomicAdd(counts + 1, cn.nodes);
        atomicAdd(counts + 2, cn.tris);
        atomicAdd(counts + 3, cn.sky);
    }
}

// AO-only walks with warp-level compaction. A warp takes a packet of 32 pixels and puts all
// of its walks (every covered pixel's spp samples) in one queue: each lane runs one walk
// (pixel, sample) at a time, a node per loop step, and whenever fewer than `refill` lanes are
// still walking, the idle lanes take the next walks of the queue, whichever pixel they
// belong to. A lane is therefore not held by the slowest walk of its own pixel's sample
// round, as in trace_kernel's one-pixel-per-lane loop; only the queue's last walks leave
// lanes idle. A walk's rays, box tests and hit test are trace_pixel's (sample_direction,
// slab, hit_tri, the frontier start), and a pixel's AO is its count of open walks over spp:
// an integer count, so the order the walks finish in changes no bit.
// With `sort` (at most kSortSpp samples a pixel) the queue is ordered by the walks' direction
// octant first (a counting sort of the packet's walks in shared memory), so the lanes that
// walk together point into one or two octants: nearby origins, the same signs of the
// direction, similar child orders and node sequences.
constexpr int kSortSpp = 16;
template <int kMinBlocks, int kStackN>
__global__ void __launch_bounds__(256, kMinBlocks) trace_ao_pool_kernel(const __grid_constant__ TraceParams p,
                                                                        uint32_t* tile_ctr, int refill, int sort) {
    const int pl = p.packet_log2, tw = 1 << pl, th = 32 >> pl;
    const int tiles_x = (p.w + tw - 1) >> pl, tiles_y = (p.h + th - 1) / th;
    const uint32_t ntiles = (uint32_t)tiles_x * tiles_y;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned below = (1u << lane) - 1u;
    __shared__ FrontierEntry frontier[8][kFrontier];
    __shared__ int open_sh[8][32];
    __shared__ uint8_t lane_sh[8][32];
    __shared__ uint16_t perm_sh[8][32 * kSortSpp];
    __shared__ uint32_t oct_sh[8][8];
    uint16_t* perm = perm_sh[threadIdx.x >> 5];
    uint32_t* octs = oct_sh[threadIdx.x >> 5];
    FrontierEntry* F = frontier[threadIdx.x >> 5];
    int* opens = open_sh[threadIdx.x >> 5];
    uint8_t* lane_of = lane_sh[threadIdx.x >> 5];   // the covered lanes in lane order
    const size_t np = (size_t)p.w * p.h;
    int32_t stack[kStackN];
    while (true) {
        uint32_t tile = 0;
        if (lane == 0) tile = atomicAdd(tile_ctr, 1u);
        tile = __shfl_sync(0xffffffffu, tile, 0);
        if (tile >= ntiles) break;
        const int x = ((int)(tile % tiles_x) << pl) + (int)(lane & (tw - 1));
        const int y = (int)(tile / tiles_x) * th + (int)(lane >> pl);
        const bool valid = x < p.w && y < p.h;
        const size_t i = valid ? (size_t)y * p.w + x : 0;
        uint8_t m = 0;
        v3 P = mk(0.0f, 0.0f, 0.0f), n = P;
        if (valid) {
            m = p.mask[i];
            P = load3(p.pos + 3 * i);
            n = load3(p.nrm + 3 * i);
            if (p.mirror) {
                store3(mirror_pos(p.mirror, np) + 3 * i, P);
                store3(mirror_nrm(p.mirror, np) + 3 * i, n);
                mirror_mask(p.mirror, np)[i] = m;
            }
            if (!m) {
                p.ao[i] = 1.0f;
                if (p.mirror) mirror_ao(p.mirror, np)[i] = 1.0f;
            }
        }
        const bool covered = valid && m;
        // basis (ray_ao.cpp:14-17) of the lane's own pixel; other lanes read it by shuffle
        const v3 a = fabsf(n.x) > 0.9f ? mk(0.0f, 1.0f, 0.0f) : mk(1.0f, 0.0f, 0.0f);
        v3 T = mk(0.0f, 0.0f, 0.0f), B = T, O = T;
        if (covered) {
            T = normalize(cross(a, n));
            B = cross(n, T);
            O = add(P, scale(n, 1e-3f));
        }
        const int fn = (p.has_geometry && p.frontier) ? tile_frontier(p, x, y, valid, F) : 0;
        const unsigned cov = __ballot_sync(0xffffffffu, covered);
        const int nc = __popc(cov);
        opens[lane] = 0;
        if (covered) lane_of[__popc(cov & below)] = (uint8_t)lane;
        __syncwarp();
        const uint32_t total = (uint32_t)nc * (uint32_t)p.spp;
        const bool sorted = sort && p.spp <= kSortSpp && total > 0;
        if (sorted) {
            // the octant of every walk (wi: pixel lane_of[wi % nc], sample wi / nc), counted,
            // then placed: perm[] lists the walks octant by octant
            if (lane < 8) octs[lane] = 0;
            __syncwarp();
            uint64_t mine = 0;                       // 4 bits a walk of this lane's share
            for (uint32_t k = 0; k < (uint32_t)kSortSpp; ++k) {
                const uint32_t wi = lane + 32u * k;
                const bool has = wi < total;
                const int src = (int)lane_of[has ? wi % (uint32_t)nc : 0u];
                const v3 pt = mk(__shfl_sync(0xffffffffu, T.x, src), __shfl_sync(0xffffffffu, T.y, src),
                                 __shfl_sync(0xffffffffu, T.z, src));
                const v3 pb = mk(__shfl_sync(0xffffffffu, B.x, src), __shfl_sync(0xffffffffu, B.y, src),
                                 __shfl_sync(0xffffffffu, B.z, src));
                const v3 pn = mk(__shfl_sync(0xffffffffu, n.x, src), __shfl_sync(0xffffffffu, n.y, src),
                                 __shfl_sync(0xffffffffu, n.z, src));
                const int qx = __shfl_sync(0xffffffffu, x, src), qy = __shfl_sync(0xffffffffu, y, src);
                if (has) {
                    const v3 dd = sample_direction(pt, pb, pn, (uint32_t)qx, (uint32_t)qy, wi / (uint32_t)nc, p.corr);
                    const uint32_t o8 = (dd.x < 0.0f ? 1u : 0u) | (dd.y < 0.0f ? 2u : 0u) | (dd.z < 0.0f ? 4u : 0u);
                    mine |= (uint64_t)o8 << (4 * k);
                    atomicAdd(&octs[o8], 1u);
                }
            }
            __syncwarp();
            if (lane == 0) {
                uint32_t run = 0;
                for (int o8 = 0; o8 < 8; ++o8) { const uint32_t c = octs[o8]; octs[o8] = run; run += c; }
            }
            __syncwarp();
            for (uint32_t k = 0; k < (uint32_t)kSortSpp; ++k) {
                const uint32_t wi = lane + 32u * k;
                if (wi < total) perm[atomicAdd(&octs[(mine >> (4 * k)) & 7u], 1u)] = (uint16_t)wi;
            }
            __syncwarp();
        }
        uint32_t next = 0;
        bool active = false;
        int q = 0;                    // the lane whose pixel the current walk belongs to
        v3 o = O, d = O;
        Inv iv;
        WRay wr;
        bool wr_ready = false;
        int32_t cur = 0;
        int sp = 0;
        uint32_t guard = 0;
        const float tmax = p.radius;
        while (p.has_geometry && total > 0) {
            const unsigned busy = __ballot_sync(0xffffffffu, active);
            if (__popc(busy) < refill && next < total) {
                // the idle lanes take the next walks of the queue, in lane order
                const unsigned idle = ~busy;
                const uint32_t my = next + (uint32_t)__popc(idle & below);
                next = min(total, next + (uint32_t)__popc(idle));
                const bool take = !active && my < total;
                const uint32_t wi = take ? (sorted ? (uint32_t)perm[my] : my) : 0u;
                const int src = (int)lane_of[wi % (uint32_t)nc];
                const v3 pt = mk(__shfl_sync(0xffffffffu, T.x, src), __shfl_sync(0xffffffffu, T.y, src),
                                 __shfl_sync(0xffffffffu, T.z, src));
                const v3 pb = mk(__shfl_sync(0xffffffffu, B.x, src), __shfl_sync(0xffffffffu, B.y, src),
                                 __shfl_sync(0xffffffffu, B.z, src));
                const v3 pn = mk(__shfl_sync(0xffffffffu, n.x, src), __shfl_sync(0xffffffffu, n.y, src),
                                 __shfl_sync(0xffffffffu, n.z, src));
                const v3 po = mk(__shfl_sync(0xffffffffu, O.x, src), __shfl_sync(0xffffffffu, O.y, src),
                                 __shfl_sync(0xffffffffu, O.z, src));
                const int qx = __shfl_sync(0xffffffffu, x, src), qy = __shfl_sync(0xffffffffu, y, src);
                if (take) {
                    q = src;
                    o = po;
                    d = sample_direction(pt, pb, pn, (uint32_t)qx, (uint32_t)qy, wi / (uint32_t)nc, p.corr);
                    iv = make_inv(o, d);
                    wr_ready = false;
                    sp = 0;
                    guard = 0;
                    active = true;
                    // start: the frontier's entries stand in for the root (walk(), trace_device.cuh)
                    cur = 0;
                    if (fn > 0) {
                        int32_t nearest = -1;
                        float tbest = 3.0e38f;
                        bool hit = false;
                        for (int e = 0; e < fn && !hit; ++e) {
                            float tn;
                            if (!slab(F[e].lo[0], F[e].hi[0], F[e].lo[1], F[e].hi[1], F[e].lo[2], F[e].hi[2], o, iv,
                                      tmax, tn))
                                continue;
                            const int32_t c = F[e].word;
                            if (c < 0) {
                                if (!wr_ready) { wr = make_wray(o, d); wr_ready = true; }
                                const uint32_t w = (uint32_t)~c;
                                const uint32_t first = w >> 3, count = (w & 7u) + 1u;
                                for (uint32_t k = 0; k < count && !hit; ++k) {
                                    const float4* tq = reinterpret_cast<const float4*>(p.tris + first + k);
                                    const float4 A = __ldg(tq), Bq = __ldg(tq + 1), C = __ldg(tq + 2);
                                    float t;
                                    if (hit_tri(wr, mk(A.x, A.y, A.z), mk(Bq.x, Bq.y, Bq.z), mk(C.x, C.y, C.z), t) &&
                                        t < tmax)
                                        hit = true;
                                }
                                continue;
                            }
                            if (nearest < 0) { nearest = c; tbest = tn; continue; }
                            int32_t push = c;
                            if (tn < tbest) { push = nearest; nearest = c; tbest = tn; }
                            stack[sp++] = push;                  // fn <= kFrontier < kStackN
                        }
                        if (hit) active = false;                 // occluded: not open
                        else if (nearest >= 0) cur = nearest;
                        else if (sp > 0) cur = stack[--sp];
                        else { active = false; atomicAdd(&opens[q], 1); }
                    }
                }
            }
            if (!__any_sync(0xffffffffu, active)) {
                if (next >= total) break;
                continue;
            }
            if (!active) continue;
            // one node of the lane's walk
            const float4* nq = reinterpret_cast<const float4*>(p.nodes + cur);
            const float4 lx = __ldg(nq + 0), hx = __ldg(nq + 1), ly = __ldg(nq + 2), hy = __ldg(nq + 3);
            const float4 lz = __ldg(nq + 4), hz = __ldg(nq + 5);
            const int4 ch = __ldg(reinterpret_cast<const int4*>(nq + 6));
            const int cnt = __ldg(reinterpret_cast<const int*>(nq + 7));
            const float LX[4] = {lx.x, lx.y, lx.z, lx.w}, HX[4] = {hx.x, hx.y, hx.z, hx.w};
            const float LY[4] = {ly.x, ly.y, ly.z, ly.w}, HY[4] = {hy.x, hy.y, hy.z, hy.w};
            const float LZ[4] = {lz.x, lz.y, lz.z, lz.w}, HZ[4] = {hz.x, hz.y, hz.z, hz.w};
            const int32_t CH[4] = {ch.x, ch.y, ch.z, ch.w};
            int32_t nearest = -1;
            float tbest = 3.0e38f;
            bool hit = false, overflow = false;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float tn;
                if (hit || k >= cnt || !slab(LX[k], HX[k], LY[k], HY[k], LZ[k], HZ[k], o, iv, tmax, tn)) continue;
                const int32_t c = CH[k];
                if (c < 0) {
                    if (!wr_ready) { wr = make_wray(o, d); wr_ready = true; }
                    const uint32_t w = (uint32_t)~c;
                    const uint32_t first = w >> 3, count = (w & 7u) + 1u;
                    for (uint32_t j = 0; j < count; ++j) {
                        const float4* tq = reinterpret_cast<const float4*>(p.tris + first + j);
                        const float4 A = __ldg(tq), Bq = __ldg(tq + 1), C = __ldg(tq + 2);
                        float t;
                        if (hit_tri(wr, mk(A.x, A.y, A.z), mk(Bq.x, Bq.y, Bq.z), mk(C.x, C.y, C.z), t) && t < tmax) {
                            hit = true;
                            break;
                        }
                    }
                    continue;
                }
                if (nearest < 0) { nearest = c; tbest = tn; continue; }
                int32_t push = c;
                if (tn < tbest) { push = nearest; nearest = c; tbest = tn; }
                if (sp >= kStackN) { overflow = true; continue; }
                stack[sp++] = push;
            }
            if (overflow) { atomicOr(p.err_word, DEV_STACK_OVERFLOW); active = false; continue; }
            if (hit) { active = false; continue; }
            if (++guard >= kGuard) { atomicOr(p.err_word, DEV_GUARD); active = false; continue; }
            if (nearest >= 0) { cur = nearest; continue; }
            if (sp > 0) { cur = stack[--sp]; continue; }
            active = false;                              // nothing within the radius: open
            atomicAdd(&opens[q], 1);
        }
        __syncwarp();
        if (covered) {
            // no geometry: every ray is open
            const int open = p.has_geometry ? opens[lane] : p.spp;
            p.ao[i] = fdiv((float)open, (float)p.spp);
            if (p.mirror) mirror_ao(p.mirror, np)[i] = p.ao[i];
        }
        __syncwarp();                              // the frontier and counts are reused by the next packet
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

// AO of listed pixels with one thread per (pixel, sample): the same rays and hit rule as
// trace_pixel (AO only), for pixel sets too small or too uneven to keep packets of pixels
// busy (the surrogate's fallback tiles). open[list[i]] receives pixel list[i]'s open rays,
// added by one atomic per warp and pixel.
__global__ void __launch_bounds__(256) ao_samples_kernel(const __grid_constant__ TraceParams p,
                                                         const uint32_t* __restrict__ list,
                                                         const uint32_t* __restrict__ count,
                                                         uint32_t* __restrict__ open) {
    const uint64_t total = (uint64_t)(*count) * (uint32_t)p.spp;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t base = (uint64_t)blockIdx.x * blockDim.x;
    Counts cn;
    // whole warps step together, so the per-warp vote below sees every lane
    for (uint64_t w0 = base; w0 < total; w0 += stride) {
        const uint64_t w = w0 + threadIdx.x;
        const bool valid = w < total;
        uint32_t px = 0xFFFFFFFFu;
        int o = 0;
        if (valid) {
            px = list[w / (uint32_t)p.spp];
            const uint32_t s = (uint32_t)(w % (uint32_t)p.spp);
            const uint32_t x = px % (uint32_t)p.w, y = px / (uint32_t)p.w;
            const v3 P = load3(p.pos + 3 * (size_t)px), n = load3(p.nrm + 3 * (size_t)px);
            const v3 a = fabsf(n.x) > 0.9f ? mk(0.0f, 1.0f, 0.0f) : mk(1.0f, 0.0f, 0.0f);
            const v3 t = normalize(cross(a, n)), b = cross(n, t);
            const v3 origin = add(P, scale(n, 1e-3f));
            const v3 dir = sample_direction(t, b, n, x, y, s, p.corr);
            const int h = p.has_geometry ? walk<false>(p.nodes, p.tris, origin, dir, p.radius, p.radius, p.err_word, cn) : 0;
            o = (h & HIT_NEAR) ? 0 : 1;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, px);
        const int sum = __popc(__ballot_sync(0xffffffffu, o) & peers);
        if (valid && (__ffs(peers) - 1) == (int)(threadIdx.x & 31u) && sum) atomicAdd(open + px, (uint32_t)sum);
    }
}

}  // namespace

int launch_ao_samples(const TraceParams& p, const uint32_t* list, const uint32_t* count, uint32_t* open,
                      int sm_count, cudaStream_t s) {
    ao_samples_kernel<<<sm_count * 8, 256, 0, s>>>(p, list, count, open);
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}

// Residency variants: the register budget decides how many 256-thread blocks share an SM
// (2: up to 128 registers, 3: 80, 4: 64, with spills to L1). The launch uses enough
// blocks to fill every SM at that residency; ctx().tune.trace_min_blocks picks the variant.
// Stack variants: 48 entries where the tree's bound (16 + 3 x wide depth) fits, else 96.
// The counting build (traversal statistics) always uses the 96-entry stack.
template <int kMB, int kStackN>
void launch_variant(const TraceParams& p, int sm_count, cudaStream_t s, uint32_t* tile_ctr, unsigned long long* counts,
                    uint32_t stride) {
    const int blocks = sm_count * kMB;
    const int pool = ctx().tune.trace_pool;
    if (counts)
        trace_kernel<true, kMB, kStack><<<blocks, 256, 0, s>>>(p, tile_ctr, counts, stride < 1 ? 1 : stride);
    else if (pool > 0 && !p.want_sky)
        trace_ao_pool_kernel<kMB, kStackN><<<blocks, 256, 0, s>>>(p, tile_ctr, pool, ctx().tune.trace_pool_sort);
    else if (ctx().tune.trace_leaf_pass)
        trace_kernel<false, kMB, kStackN, true><<<blocks, 256, 0, s>>>(p, tile_ctr, nullptr, 1);
    else
        trace_kernel<false, kMB, kStackN><<<blocks, 256, 0, s>>>(p, tile_ctr, nullptr, 1);
}

template <int kStackN>
void launch_stack(const TraceParams& p, int sm_count, cudaStream_t s, uint32_t* tile_ctr, unsigned long long* counts,
                  uint32_t stride) {
    switch (ctx().tune.trace_min_blocks) {
        case 2: launch_variant<2, kStackN>(p, sm_count, s, tile_ctr, counts, stride); break;
        case 4: launch_variant<4, kStackN>(p, sm_count, s, tile_ctr, counts, stride); break;
        default: launch_variant<3, kStackN>(p, sm_count, s, tile_ctr, counts, stride); break;
    }
}

int launch_trace(const TraceParams& p, int sm_count, cudaStream_t s, unsigned long long* counts, uint32_t stride) {
    // the tile counter sits in the word after the error word
    uint32_t* tile_ctr = p.err_word + 1;
    cudaMemsetAsync(tile_ctr, 0, 4, s);
    if (ctx().tune.trace_stack <= 48 && p.stack_need <= 48)
        launch_stack<48>(p, sm_count, s, tile_ctr, counts, stride);
    else
        launch_stack<kStack>(p, sm_count, s, tile_ctr, counts, stride);
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}

int launch_occluded(const Node4* nodes, const LeafTri* tris, int has_geometry, const float* rays, const float* tmax,
                    uint32_t n, uint8_t* hit, uint32_t* err_word, cudaStream_t s) {
    if (n == 0) return RN_OK;
    occluded_kernel<<<(n + 255) / 256, 256, 0, s>>>(nodes, tris, has_geometry, rays, tmax, n, hit, err_word);
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}

}  // namespace rn
