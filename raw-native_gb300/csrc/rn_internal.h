// rn_internal.h -- host-side internals of librn_ao.so: the process-wide device context,
// its workspace, error reporting, and the launchers each kernel file exports.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include "../../include/rn_ao.h"

namespace rn {

// Error word written by kernels whose device-side loops have budgets (traversal guard,
// stack overflow, PLOC rounds). The host reads it after the work completes.
enum DeviceError : uint32_t {
    DEV_OK = 0,
    DEV_STACK_OVERFLOW = 1u << 0,
    DEV_GUARD = 1u << 1,
    DEV_PLOC_NO_MERGE = 1u << 2,
    DEV_QUEUE_OVERFLOW = 1u << 3,
};

// A device buffer that grows on demand and is reused across calls.
struct DevBuf {
    void* ptr = nullptr;
    size_t cap = 0;
};

// A call-local device allocation, freed on every return path.
struct ScopedDev {
    void* p = nullptr;
    ScopedDev() = default;
    ScopedDev(const ScopedDev&) = delete;
    ScopedDev& operator=(const ScopedDev&) = delete;
    ~ScopedDev() { if (p) cudaFree(p); }
};

// Workspace slots of the context. Each entry point uses fixed slots, so repeated calls of
// the same size allocate nothing.
enum Slot {
    WS_POS, WS_NRM, WS_MASK, WS_AO, WS_SKY, WS_SUN, WS_SS, WS_ERR, WS_TRUTH, WS_APPROX,
    WS_PARTIALS, WS_WORKLIST, WS_COUNTERS, WS_RAYS, WS_TMAX, WS_HITS, WS_TRIS_IN,
    WS_NRM_IN, WS_RASTER, WS_DEPTH, WS_STATS,
    WS_SUR_AO4, WS_SUR_PRED, WS_SUR_FB, WS_SUR_AOFB, WS_SUR_STATS, WS_VPOS, WS_VNRM, WS_VDEPTH, WS_GTAO,
    WS_ALB_IN, WS_ALB, WS_MOTION, WS_FRAME, WS_HDR, WS_FRAME_SMALL, WS_MIRROR,
    WS_HYB_LIT, WS_HYB_TRI, WS_HYB_T, WS_HYB_NG, WS_CLOSEST_TRI, WS_CLOSEST_T,
    WS_PT_SAMPLES, WS_PT_ACC, WS_PT_OUT, WS_PT_CTR, WS_PT_WAVE, WS_PLOC, WS_COLLAPSE,
    WS_COUNT
};

// Launch shapes the autotuner may change (rn_tune_set / rn_tune_load, and RN_TUNE_<KEY>
// environment variables at the first rn_init). None of them changes a result bit.
struct Tune {
    int trace_min_blocks = 3;   // resident 256-thread traversal blocks per SM: 2, 3 or 4
    int batch_min_blocks = 3;   // ... of the batched multi-view traversal
    int trace_frontier = 1;     // per-warp frontier for AO-only walks
    int trace_frontier_min_spp = 16;  // ... built only when spp reaches this (its cost is per packet)
    int trace_frontier_tail = 0;      // greedy largest-first steps after the level-by-level build (at most spp / 16)
    int trace_packet = 8;       // a warp's pixel packet: trace_packet x (32 / trace_packet); 4, 8 or 16
    int trace_stack = 96;       // traversal stack entries: 48 or 96 (48 only where the tree's depth allows)
    int ssao_tile_h = 8;        // SSAO tile: 32 x ssao_tile_h pixels, one thread each; 4, 8 or 16
    int conv_bn_max = 256;      // largest GEMM tile width (columns of C per CTA): 64, 128 or 256
    int conv_halo = 1;          // 128-pixel row tiles from a ring of one-row boxes (where they fit)
    int conv_pair = 1;          // per-tap convolutions: two 128-pixel tiles per weight box
    int accel_radius = 16;      // PLOC search radius of the traversal accelerators built next
    int accel_leaf = 4;         // largest leaf (triangles) of the traversal accelerators built next
    int accel_leaf_small = 4;   // ... of those with fewer than kSmallScene triangles
    int frame_direct = 1;       // host-buffer frames: the passes read and write mapped host memory
    int hybrid_min_blocks = 6;  // resident 128-thread hybrid-pass blocks per SM: 5, 6 or 8
    int trace_leaf_pass = 1;    // traversal: a node's leaf children tested in one loop after its slab tests
    int conv_tmem_a = 0;        // row-ring convolutions of 32 -> 32 or 16 -> 32 channels: A operands kept in TMEM
    int conv_fan = 1;           // row-ring convolutions: each input row's MMAs feed its three output rows (N = 3 x BN)
    int conv_fan_bn = 64;       // ... widest output-channel slice: 64 (where its weights fit, else 32) or 32
    int ploc_tail = 4096;       // PLOC: the rounds from this many clusters on run in one launch (0: never)
    int ploc_tail_ctas = 1;     // ... in one block (1) or one thread-block cluster of this many CTAs
    int ploc_fused = 1;         // PLOC: a round's prefix sum and scatter in one launch (decoupled look-back)
    int collapse_block = 0;     // 4-wide collapse: trees of at most this many triangles in one block
    int trace_pool = 0;         // AO-only walks from a per-packet queue, lanes refilled below this many busy (0: off)
    int trace_pool_sort = 0;    // ... the queue ordered by the walks' direction octant (at most 16 spp)
    int pt_regen = 4;           // path tracer: persistent threads regenerating paths, blocks of 128 per SM (0: one thread a sample)
    int pt_wave = 1024;         // path tracer: the wavefront form over this many x 1024 path slots (0: off)
    int pt_shade_blocks = 6;    // ... its shade kernel's resident blocks of 128 per SM (register budget)
    int pt_slice = 0;           // path tracer: samples per slice at most (0: as many as 2 GiB of terms hold)
};
constexpr uint32_t kSmallScene = 1u << 16;

struct Context {
    bool ready = false;
    Tune tune;
    int device = -1;
    int sm_count = 0;
    cudaStream_t stream = nullptr;      // the stream all work goes to
    cudaStream_t own_stream = nullptr;  // the library's own stream
    uint8_t* trig_corr = nullptr;       // 2^24 bytes: host-libm correction per sample angle
    uint32_t* dev_error = nullptr;      // one DeviceError word
    cudaMemPool_t accel_pool = nullptr; // the accelerators' memory: freed blocks kept for reuse (up to 4 GiB)
    DevBuf ws[WS_COUNT];
};

Context& ctx();

// Status helpers: fill `st` and return the code.
int fail(rn_status* st, int code, const char* fmt, ...);
int ok(rn_status* st);
// Check a CUDA call; on failure fill `st` and return RN_ERR_CUDA (or RN_ERR_NO_MEMORY).
int cuda_fail(rn_status* st, cudaError_t e, const char* what);
#define RN_CUDA(call, st)                                          \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return ::rn::cuda_fail(st, e_, #call); \
    } while (0)
#define RN_TRY(expr)                 \
    do {                             \
        int rc_ = (expr);            \
        if (rc_ != RN_OK) return rc_; \
    } while (0)

// Make sure the context is open (device, stream, sampler table).
int ensure_ctx(rn_status* st);
// A workspace buffer of at least `bytes`.
int ws_get(Slot s, size_t bytes, void** out, rn_status* st);
// Read and clear the device error word (synchronizes the stream).
int check_device_error(rn_status* st, const char* where);

// ---------------------------------------------------------------- sampler table
int build_trig_correction(Context& c, rn_status* st);

// ---------------------------------------------------------------- reconcile / SSAO
struct RecPartial {   // one tile's share of the reconcile
    double sum;
    float max;
    int32_t n;
};
struct RecOut {       // the reduction's device-side result
    double sum;
    float max;
    int32_t n;
    uint32_t done;    // blocks finished (the last block reduces, then resets it to 0)
    uint32_t pad;
};
// Returns the launch's error (read once with cudaGetLastError, so the caller reports it).
cudaError_t launch_reconcile(const float* approx, const float* truth, const uint8_t* mask, size_t npx,
                             float* err, RecPartial* partials, int nblocks, RecOut* out, cudaStream_t s);
int reconcile_blocks(size_t npx);
int launch_ssao(int w, int h, const float* pos, const float* nrm, const uint8_t* mask, int samples,
                float radius, const uint8_t* corr, float* ao, const float* truth, float* err,
                RecPartial* partials, RecOut* out, cudaStream_t s);
int ssao_blocks(int w, int h);

// ---------------------------------------------------------------- accelerator
// A 4-wide BVH node: six 4-float planes of child boxes (SoA) then the 4 child words and
// per-node metadata. 128 bytes, 16-byte aligned for vector loads. Child word >= 0: index of
// an interior node; < 0: leaf, ~word = first << 3 | (count - 1) into the leaf triangles.
struct alignas(16) Node4 {
    float lox[4], hix[4], loy[4], hiy[4], loz[4], hiz[4];
    int32_t child[4];
    int32_t meta[4];   // meta[0] = number of valid children
};
static_assert(sizeof(Node4) == 128, "Node4 layout");
constexpr int kLeafCap = 8;   // triangles a leaf may hold (the child word's 3-bit count)

// A leaf triangle: vertices a, b, c as float4 (w of a = input triangle index).
struct alignas(16) LeafTri {
    float ax, ay, az, id;
    float bx, by, bz, pad0;
    float cx, cy, cz, pad1;
};

}  // namespace rn

// The accelerator handle of the C ABI.
struct rn_accel {
    int device = -1;
    uint32_t ntri = 0;
    uint32_t nodes = 0;        // wide nodes
    uint32_t rounds = 0;       // PLOC rounds
    uint32_t depth = 0;        // wide-tree depth (levels)
    rn::Node4* d_nodes = nullptr;
    rn::LeafTri* d_tris = nullptr;
};

namespace rn {
// PLOC: build the binary tree on the device. Outputs (device): nodes9 (2n-1 x 9 int32 in
// the reference's layout) when non-null; the binary tree in SoA form for the collapse.
struct PlocTree {
    uint32_t n = 0;
    int32_t root = -1;
    uint32_t rounds = 0;
    float* box = nullptr;      // (2n-1) x 6: lo.x lo.y lo.z hi.x hi.y hi.z
    int32_t* left = nullptr;   // (2n-1)
    int32_t* right = nullptr;  // (2n-1)
    int32_t* tri = nullptr;    // (2n-1)
    void* mem = nullptr;       // the workspace block holding the arrays above (not owned)
};
int ploc_build(const float* d_tris, uint32_t n, int radius, PlocTree* out, cudaStream_t s, rn_status* st);
void ploc_free(PlocTree* t);
int ploc_export(const PlocTree& t, int32_t* d_nodes9, cudaStream_t s, rn_status* st);
int collapse_bvh4(const PlocTree& t, const float* d_tris, rn_accel* acc, int leaf_max, cudaStream_t s,
                  rn_status* st);

// ---------------------------------------------------------------- traversal
struct TraceParams {
    int w, h;
    const float* pos;
    const float* nrm;
    const uint8_t* mask;
    const Node4* nodes;
    const LeafTri* tris;
    int has_geometry;
    int spp;
    float radius;
    float lx, ly, lz;     // to_light (normalized on the device)
    int want_sky, sun_forced;
    const uint8_t* corr;
    float* ao;
    float* sky;
    float* sun;
    uint32_t* err_word;
    int frontier;         // AO-only walks start from a per-warp frontier (0: from the root)
    int packet_log2;      // log2 of the packet width (pixels per warp row): 2, 3 or 4
    int frontier_tail;    // greedy single-entry steps after the breadth-first frontier build
    int stack_need;       // entries the walk can push on this tree: 16 + 3 x wide depth
    // copy-through of a G-buffer read from host memory (null: none): every pixel's position,
    // normal, AO and mask are also written to a device buffer laid out as
    // [position w*h*12 B][normal w*h*12 B][ao w*h*4 B][mask w*h B] (mirror_* below)
    uint8_t* mirror;
};
__host__ __device__ inline float* mirror_pos(uint8_t* m, size_t) { return (float*)m; }
__host__ __device__ inline float* mirror_nrm(uint8_t* m, size_t np) { return (float*)(m + np * 12); }
__host__ __device__ inline float* mirror_ao(uint8_t* m, size_t np) { return (float*)(m + np * 24); }
__host__ __device__ inline uint8_t* mirror_mask(uint8_t* m, size_t np) { return m + np * 28; }
// Traced AO (AO only, the library's sampler and tuning) of a device G-buffer into a device
// image, on the library's stream.
int trace_ao_device(const float* pos, const float* nrm, const uint8_t* mask, int w, int h, const rn_accel* accel,
                    int spp, float radius, float* ao, rn_status* st);
// AO-only sample-parallel trace of the pixels list[0 .. *count) (indices into the frame,
// count on the device): open[px] += open rays of pixel px (the caller zeroes `open`).
int launch_ao_samples(const TraceParams& p, const uint32_t* list, const uint32_t* count, uint32_t* open,
                      int sm_count, cudaStream_t s);
// TraceParams for an AO-only trace of a device G-buffer with the library's sampler and tuning.
TraceParams ao_trace_params(const float* pos, const float* nrm, const uint8_t* mask, int w, int h,
                            const rn_accel* accel, int spp, float radius);
// The tuned trace fields of p (frontier, packet, stack bound for this tree).
void apply_tune(TraceParams& p, const rn_accel* accel);
int launch_trace(const TraceParams& p, int sm_count, cudaStream_t s, unsigned long long* counts = nullptr,
                 uint32_t stride = 1);

// ---------------------------------------------------------------- closest hit, hybrid (hybrid.cu)
// Nearest hits (triangle index, t; -1 / -1 for none) of n rays (6 floats each) below tmax.
int launch_closest(const Node4* nodes, const LeafTri* tris, int has_geometry, const float* rays, const float* tmax,
                   uint32_t n, int32_t* tri, float* t, uint32_t* err, cudaStream_t s);
// The hybrid pass over a G-buffer: sun shadows and mirror reflections per covered pixel.
int launch_hybrid(int w, int h, const float* pos, const float* nrm, const float* geo_nrm, const uint8_t* mask,
                  const rn_accel* accel,
                  const float eye[3], const float to_sun[3], float* lit, int32_t* refl_tri, float* refl_t,
                  uint32_t* err, cudaStream_t s);

// ---------------------------------------------------------------- shading and motion (frame.cu)
// shadeV2 / shadeHDRV2 (model 2: a_or_sky = sky) or shade / shadeHDR (model 1: a_or_sky = the
// AO), frame and hdr 3 floats a pixel; motion: current minus previous clip UV (2 floats a
// pixel), the valid count added to valid[0] and the covered count to valid[1].
int launch_shade(int w, int h, const float* nrm, const float* albedo, const uint8_t* mask, int model,
                 const float* a_or_sky, const float* sun, const float ldir[3], float li, float* frame, float* hdr,
                 cudaStream_t s);
int launch_motion(int w, int h, const float* pos, const uint8_t* mask, const float* vp16, const float* prev16,
                  float* motion, unsigned* valid, cudaStream_t s);

// ---------------------------------------------------------------- GTAO (gtao.cu)
// The view-space G-buffer (view16: the camera's row-major view matrix) into vpos/vnrm/vdepth,
// then GTAO (radius, slices, steps; fovy and aspect w / h of the camera) into out.
int launch_gtao(int w, int h, const float* pos, const float* nrm, const uint8_t* mask, const float* view16,
                float fovy, float radius, int slices, int steps, float* vpos, float* vnrm, float* vdepth, float* out,
                cudaStream_t s);

// ---------------------------------------------------------------- G-buffer
// Scratch bytes for ntri triangles, npx pixels and npairs (record, 8x8 bin) pairs.
size_t raster_scratch_bytes(uint32_t ntri, size_t npx, size_t npairs);
// RN_ERR_NO_MEMORY with *pairs_needed set when the scratch holds too few pairs.
int launch_raster(const float* tris, const float* nrm, uint32_t ntri, const float* d_vp, float nearZ, int w, int h,
                  char* scratch, size_t scratch_bytes, float* depth, float* pos, float* nrm_out, uint8_t* mask,
                  cudaStream_t s, size_t* pairs_needed, const float* albedo_tri = nullptr, float* albedo = nullptr);
int scan_exclusive_u32(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* bsum, uint32_t* total, cudaStream_t s);
int launch_occluded(const Node4* nodes, const LeafTri* tris, int has_geometry, const float* rays,
                    const float* tmax, uint32_t n, uint8_t* hit, uint32_t* err_word, cudaStream_t s);

}  // namespace rn
