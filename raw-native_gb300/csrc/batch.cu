// batch.cu -- many views of one scene in one launch (the batched multi-view form).
//
// A batch is a table of views of uneven size and spp over one accelerator. One frame of the
// batch is three device steps, captured once into a CUDA graph and replayed:
//   1. clear the work counter and the per-view reduction counters;
//   2. one persistent traversal launch: every warp takes the next 8 x 4 tile from a single
//      device counter over the tiles of all views, finds its view by binary search over the
//      views' first-tile offsets (staged in shared memory with the views' parameters), and
//      traces it as the single-frame kernel does (trace_device.cuh);
//   3. one SSAO launch over the 32 x 8 tiles of all views, the reconcile against each view's
//      ray-traced AO fused in; each view's last block to finish reduces that view's partials;
//   4. the per-view reconcile sums copied to pinned host memory.
// No host round trip happens inside a frame; the host reads the results after the graph.
#include "rn_internal.h"
#include "trace_device.cuh"
#include "ssao_device.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace rn {

constexpr int kMaxViews = 256;

struct BatchView {
    TraceParams tp;          // the view's traversal parameters (its G-buffer, outputs, spp, radius)
    uint32_t tile_begin;     // the view's first traversal tile in the batch
    uint32_t ssao_begin;     // its first SSAO block
    uint32_t ssao_count;     // its SSAO blocks (0: no SSAO for this view)
    uint32_t ssao_tiles_x;
    float* ss;
    float* err;
};

namespace {

using trace_dev::Counts;
using trace_dev::kTileW;
using trace_dev::kTileH;

__device__ __forceinline__ int find_view(const uint32_t* begins, int n, uint32_t i) {
    int lo = 0, hi = n - 1;                 // the last view whose begin is <= i
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (begins[mid] <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <int kMinBlocks>
__global__ void __launch_bounds__(256, kMinBlocks) trace_batch_kernel(const BatchView* __restrict__ views, int nviews,
                                                                      uint32_t total_tiles, uint32_t* tile_ctr) {
    __shared__ TraceParams sp[kMaxViews];
    __shared__ uint32_t begins[kMaxViews];
    for (int v = threadIdx.x; v < nviews; v += blockDim.x) { sp[v] = views[v].tp; begins[v] = views[v].tile_begin; }
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u;
    __shared__ trace_dev::FrontierEntry frontier[8][trace_dev::kFrontier];
    trace_dev::FrontierEntry* F = frontier[threadIdx.x >> 5];
    Counts cn;
    while (true) {
        uint32_t tile = 0;
        if (lane == 0) tile = atomicAdd(tile_ctr, 1u);
        tile = __shfl_sync(0xffffffffu, tile, 0);
        if (tile >= total_tiles) break;
        const int v = find_view(begins, nviews, tile);
        const TraceParams& p = sp[v];
        const uint32_t local = tile - begins[v];
        const int tiles_x = (p.w + kTileW - 1) / kTileW;
        const int x = (int)(local % tiles_x) * kTileW + (int)(lane % kTileW);
        const int y = (int)(local / tiles_x) * kTileH + (int)(lane / kTileW);
        const v3 toLight = normalize(mk(p.lx, p.ly, p.lz));
        const int fn = (!p.want_sky && p.has_geometry && p.frontier)
                            ? trace_dev::tile_frontier(p, x, y, x < p.w && y < p.h, F) : 0;
        if (x < p.w && y < p.h) trace_dev::trace_pixel<false>(p, x, y, toLight, cn, F, fn);
        __syncwarp();
    }
}

__global__ void __launch_bounds__(ssao_dev::kThreads) ssao_batch_kernel(const BatchView* __restrict__ views, int nviews,
                                                                        int samples, RecPartial* parts, RecOut* outs) {
    __shared__ float4 win[ssao_dev::kSH][ssao_dev::kSW];
    __shared__ uint32_t begins[kMaxViews];
    for (int v = threadIdx.x; v < nviews; v += blockDim.x) begins[v] = views[v].ssao_begin;
    __syncthreads();
    const int v = find_view(begins, nviews, blockIdx.x);
    const BatchView& bv = views[v];
    if (bv.ssao_count == 0) return;             // uniform per block
    const uint32_t lb = blockIdx.x - begins[v];
    const int bx = (int)(lb % bv.ssao_tiles_x), by = (int)(lb / bv.ssao_tiles_x);
    RecAcc acc;
    ssao_dev::ssao_tile<true>(win, bx, by, bv.tp.w, bv.tp.h, bv.tp.pos, bv.tp.nrm, bv.tp.mask, samples, bv.tp.radius,
                              bv.tp.corr, bv.ss, bv.tp.ao, bv.err, acc);
    rec_block_finish<ssao_dev::kThreads>(acc, parts + bv.ssao_begin, outs + v, lb, bv.ssao_count);
}

}  // namespace
}  // namespace rn

using namespace rn;

struct rn_batch {
    int device = -1;
    int nviews = 0;
    float tolerance = 0.0f;
    bool want_ssao = false;
    cudaStream_t capture = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    char* dmem = nullptr;            // views table, partials, per-view RecOut, tile counter
    RecOut* host_out = nullptr;      // pinned
    uint64_t total_tiles = 0;
    uint64_t total_rays = 0;
};

namespace {

void batch_release(rn_batch* b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->capture) cudaStreamDestroy(b->capture);
    if (b->dmem) cudaFree(b->dmem);
    if (b->host_out) cudaFreeHost(b->host_out);
    delete b;
}

}  // namespace

extern "C" {

int rn_batch_create(const rn_accel* accel, const rn_view* views, int nviews, int ss_samples, float tolerance,
                    const float* to_light, int flags, rn_batch** out, rn_status* st) {
    if (!out) return fail(st, RN_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (!accel || !views || nviews <= 0) return fail(st, RN_ERR_INVALID, "no views or no accelerator");
    if (nviews > kMaxViews) return fail(st, RN_ERR_INVALID, "%d views: at most %d per batch", nviews, kMaxViews);
    if ((flags & RN_SKY) && !to_light) return fail(st, RN_ERR_INVALID, "RN_SKY needs to_light");
    if (ss_samples < 0) return fail(st, RN_ERR_INVALID, "ss_samples %d < 0", ss_samples);
    RN_TRY(ensure_ctx(st));
    Context& c = ctx();
    if (accel->device != c.device) return fail(st, RN_ERR_STATE, "accelerator belongs to device %d", accel->device);
    std::vector<BatchView> table((size_t)nviews);
    uint32_t tiles = 0, ssao_blocks_total = 0;
    uint64_t rays = 0;
    bool any_ssao = false;
    for (int v = 0; v < nviews; ++v) {
        const rn_view& in = views[v];
        if (in.w <= 0 || in.h <= 0 || (size_t)in.w * in.h > ((size_t)1 << 31))
            return fail(st, RN_ERR_INVALID, "view %d: size %dx%d", v, in.w, in.h);
        if (in.spp <= 0) return fail(st, RN_ERR_INVALID, "view %d: spp %d", v, in.spp);
        if (!in.position || !in.normal || !in.mask || !in.ao) return fail(st, RN_ERR_INVALID, "view %d: null buffer", v);
        if ((flags & RN_SKY) && (!in.sky || !in.sun)) return fail(st, RN_ERR_INVALID, "view %d: RN_SKY needs sky and sun", v);
        BatchView& b = table[(size_t)v];
        TraceParams& p = b.tp;
        p = TraceParams{};
        p.w = in.w; p.h = in.h;
        p.pos = in.position; p.nrm = in.normal; p.mask = in.mask;
        p.nodes = accel->d_nodes; p.tris = accel->d_tris; p.has_geometry = accel->ntri > 0;
        p.spp = in.spp; p.radius = in.radius;
        p.want_sky = (flags & RN_SKY) != 0;
        p.sun_forced = (flags & RN_SUN_FORCED) != 0;
        p.lx = p.want_sky ? to_light[0] : 0.0f; p.ly = p.want_sky ? to_light[1] : 1.0f; p.lz = p.want_sky ? to_light[2] : 0.0f;
        p.corr = (flags & RN_DEVICE_TRIG) ? nullptr : c.trig_corr;
        p.ao = in.ao; p.sky = in.sky; p.sun = in.sun;
        p.err_word = c.dev_error;
        apply_tune(p, accel);
        p.packet_log2 = 3;                       // the batch's work queue uses 8 x 4 packets
        b.tile_begin = tiles;
        tiles += (uint32_t)(((in.w + 7) / 8) * ((in.h + 3) / 4));
        b.ssao_begin = ssao_blocks_total;
        b.ssao_tiles_x = (uint32_t)((in.w + 31) / 32);
        b.ssao_count = in.ao_ss ? (uint32_t)(b.ssao_tiles_x * ((in.h + 7) / 8)) : 0u;
        ssao_blocks_total += b.ssao_count;
        any_ssao = any_ssao || in.ao_ss;
        b.ss = in.ao_ss;
        b.err = in.err;
        rays += (uint64_t)in.w * in.h * (uint64_t)in.spp;
    }
    rn_batch* b = new rn_batch();
    b->device = c.device;
    b->nviews = nviews;
    b->tolerance = tolerance;
    b->want_ssao = any_ssao;
    b->total_tiles = tiles;
    b->total_rays = rays;
    const size_t tbl = ((size_t)nviews * sizeof(BatchView) + 255) & ~size_t(255);
    const size_t prt = ((size_t)std::max<uint32_t>(ssao_blocks_total, 1) * sizeof(RecPartial) + 255) & ~size_t(255);
    const size_t outs = ((size_t)nviews * sizeof(RecOut) + 255) & ~size_t(255);
    int rc = RN_OK;
    auto chk = [&](cudaError_t e, const char* what) {
        if (rc == RN_OK && e != cudaSuccess) rc = cuda_fail(st, e, what);
    };
    chk(cudaMalloc((void**)&b->dmem, tbl + prt + outs + 256), "batch device memory");
    chk(cudaMallocHost((void**)&b->host_out, (size_t)nviews * sizeof(RecOut)), "batch pinned results");
    chk(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking), "batch stream");
    if (rc != RN_OK) { batch_release(b); return rc; }
    BatchView* d_views = (BatchView*)b->dmem;
    RecPartial* d_parts = (RecPartial*)(b->dmem + tbl);
    RecOut* d_outs = (RecOut*)(b->dmem + tbl + prt);
    uint32_t* d_ctr = (uint32_t*)(b->dmem + tbl + prt + outs);
    chk(cudaMemcpy(d_views, table.data(), (size_t)nviews * sizeof(BatchView), cudaMemcpyHostToDevice), "view table");
    // capture one frame: counters, traversal, SSAO + reconcile, results to pinned memory
    chk(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal), "begin capture");
    if (rc == RN_OK) {
        cudaMemsetAsync(d_ctr, 0, 4, b->capture);
        cudaMemsetAsync(d_outs, 0, (size_t)nviews * sizeof(RecOut), b->capture);
        const int mb = c.tune.batch_min_blocks;
        if (mb == 2) trace_batch_kernel<2><<<c.sm_count * 2, 256, 0, b->capture>>>(d_views, nviews, tiles, d_ctr);
        else if (mb == 4) trace_batch_kernel<4><<<c.sm_count * 4, 256, 0, b->capture>>>(d_views, nviews, tiles, d_ctr);
        else trace_batch_kernel<3><<<c.sm_count * 3, 256, 0, b->capture>>>(d_views, nviews, tiles, d_ctr);
        if (ssao_blocks_total)
            ssao_batch_kernel<<<ssao_blocks_total, ssao_dev::kThreads, 0, b->capture>>>(d_views, nviews, ss_samples,
                                                                                       d_parts, d_outs);
        cudaMemcpyAsync(b->host_out, d_outs, (size_t)nviews * sizeof(RecOut), cudaMemcpyDeviceToHost, b->capture);
        chk(cudaGetLastError(), "batch kernels");
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(b->capture, &g);
        b->graph = g;
        chk(e, "end capture");
    }
    if (rc == RN_OK) chk(cudaGraphInstantiate(&b->exec, b->graph, 0), "graph instantiate");
    if (rc != RN_OK) { batch_release(b); return rc; }
    *out = b;
    return ok(st);
}

int rn_batch_run(rn_batch* b, rn_reconcile_result* results, rn_status* st) {
    if (!b) return fail(st, RN_ERR_INVALID, "null batch");
    RN_TRY(ensure_ctx(st));
    Context& c = ctx();
    if (b->device != c.device) return fail(st, RN_ERR_STATE, "batch belongs to device %d", b->device);
    RN_CUDA(cudaGraphLaunch(b->exec, c.stream), st);
    RN_CUDA(cudaStreamSynchronize(c.stream), st);
    RN_TRY(check_device_error(st, "rn_batch_run"));
    if (results)
        for (int v = 0; v < b->nviews; ++v) {
            const RecOut& r = b->host_out[v];
            rn_reconcile_result& o = results[v];
            o.sum_sq = r.sum;
            o.pixels = r.n;
            o.max_error = r.max;
            o.rmse = r.n > 0 ? (float)std::sqrt(r.sum / (double)r.n) : 0.0f;
            o.within_tolerance = o.rmse <= b->tolerance ? 1 : 0;
        }
    return ok(st);
}

int rn_batch_info(const rn_batch* b, uint64_t* tiles, uint64_t* pixel_samples, rn_status* st) {
    if (!b) return fail(st, RN_ERR_INVALID, "null batch");
    if (tiles) *tiles = b->total_tiles;
    if (pixel_samples) *pixel_samples = b->total_rays;
    return ok(st);
}

void rn_batch_free(rn_batch* b) { batch_release(b); }

int rn_ao_batch(const rn_accel* accel, const rn_view* views, int nviews, int ss_samples, float tolerance,
                const float* to_light, int flags, rn_reconcile_result* results, rn_status* st) {
    rn_batch* b = nullptr;
    RN_TRY(rn_batch_create(accel, views, nviews, ss_samples, tolerance, to_light, flags, &b, st));
    const int rc = rn_batch_run(b, results, st);
    rn_batch_free(b);
    return rc;
}

}  // extern "C"
