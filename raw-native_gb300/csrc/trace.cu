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
template <bool kCount, int kMinBlocks, int kStackN>
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
        if (x < p.w && y < p.h) trace_pixel<kCount, kStackN>(p, x, y, toLight, cn, F, fn);
        __syncwarp();                              // the frontier is rebuilt for the next tile
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
    if (counts)
        trace_kernel<true, kMB, kStack><<<blocks, 256, 0, s>>>(p, tile_ctr, counts, stride < 1 ? 1 : stride);
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
