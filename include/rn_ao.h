/*
 * rn_ao.h -- C ABI of the GB300 (sm_103a) ambient-occlusion path of raw-native.
 *
 * One shared library, librn_ao.so, replaces the CPU bodies of the reference's AO oracle
 * ("raw-rt-ao-v1"), its screen-space AO pass and the reconcile between them. The C++ shim
 * in raw-native_gb300/host/ implements the reference's own symbols (computeRTAO,
 * computeRTVisibility, computeSSAO, reconcile, LinearAccel) over these entry points, so
 * raw_native_cli and `raw_native_cli verify` run their AO passes on one GPU with no source
 * change. Plain pointers and sizes only; no C++ or torch types cross this boundary.
 *
 * Conventions
 *  - Every entry point returns an rn_code (0 = RN_OK) and, when `st` is not NULL, fills
 *    it with the code and a one-line message. Nothing throws, nothing aborts, and there is
 *    no CPU fallback: without a usable GPU every call returns RN_ERR_NO_DEVICE (the
 *    reference maps "no device" to exit 4 and the verdict "unverifiable",
 *    src/tools/gpu_run.cpp:52-59).
 *  - Pointers are HOST pointers unless the call's flags include RN_DEVICE_PTRS, in which
 *    case every buffer argument is a device pointer on the current device. Host calls copy
 *    in, compute and copy out on the library's stream and return when the results are in
 *    host memory. Device-pointer calls are asynchronous on the library's stream
 *    (rn_set_stream) unless the call returns a host-side scalar result, in which case it
 *    synchronizes that stream.
 *  - Images are row-major, row 0 at the top, w * h pixels. A position or normal plane is
 *    3 floats per pixel (x, y, z), as raw::Buffer<raw::Vec3> stores it
 *    (raw/core/image.hpp:8-16). A mask is one byte per pixel, nonzero = covered.
 *  - Triangles are 9 floats each (a, b, c), in the order raw::LinearAccel::build flattens
 *    the scene's meshes (src/renderer/accel.cpp:13-25).
 *  - The library keeps one process-wide device context (the reference's device is a
 *    process singleton, src/renderer/gpu/gpu_renderer.cpp:72-77). Calls must come from one
 *    host thread at a time.
 */
#ifndef RN_AO_H
#define RN_AO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RN_AO_ABI_VERSION 1

typedef enum rn_code {
    RN_OK = 0,
    RN_ERR_INVALID = 1,    /* bad argument: null pointer, size, spp, radius */
    RN_ERR_NO_DEVICE = 2,  /* no CUDA device, or the device is not sm_103 */
    RN_ERR_CUDA = 3,       /* a CUDA runtime call failed; message names it */
    RN_ERR_NO_MEMORY = 4,  /* device or pinned-host allocation refused */
    RN_ERR_OVERFLOW = 5,   /* a traversal stack or a build queue ran out of room */
    RN_ERR_BUDGET = 6,     /* a device-side loop hit its iteration budget and gave up */
    RN_ERR_STATE = 7       /* call sequence error (e.g. an accel from another context) */
} rn_code;

typedef struct rn_status {
    int code;
    char message[240];
} rn_status;

/* Flags shared by the entry points. */
#define RN_DEVICE_PTRS  0x1   /* buffer arguments are device pointers */
#define RN_SKY          0x2   /* rn_ao_visibility: also write sky (and sun) */
#define RN_SUN_FORCED   0x4   /* rn_ao_visibility: sun = 1 everywhere (lighting v2-nosun) */
#define RN_EXACT_TRIG   0x0   /* default: sample angles use the host libm's cosf/sinf bits */
#define RN_DEVICE_TRIG  0x8   /* sample angles use the device sincosf alone (no calibration) */

/* A G-buffer as the AO passes read it: raw::GBuffer's position, normal and mask planes
 * (raw/renderer/gbuffer.hpp:7-21). */
typedef struct rn_gbuf {
    int w, h;
    const float* position;   /* 3 floats per pixel */
    const float* normal;     /* 3 floats per pixel */
    const uint8_t* mask;     /* 1 byte per pixel */
} rn_gbuf;

/* The scalar half of raw::ReconcileResult (raw/cert/reconcile.hpp:6-11) plus the FP64 sum
 * of squares it derives rmse from. */
typedef struct rn_reconcile_result {
    float rmse;
    float max_error;
    int32_t pixels;
    int32_t within_tolerance;
    double sum_sq;
} rn_reconcile_result;

/* Opaque occlusion accelerator: the GPU-built BVH over one triangle list. Replaces the
 * heap Bvh inside raw::LinearAccel (raw/renderer/accel.hpp:15-23). */
typedef struct rn_accel rn_accel;

/* Library ABI version (RN_AO_ABI_VERSION). No counterpart in the reference. */
int rn_ao_version(void);

/* Open the process-wide context on the current CUDA device: checks for sm_103, creates the
 * library stream and builds the sampler's angle table. Every other entry point calls it
 * on first use; call it early to keep that set-up out of a timed region or a capture. */
int rn_init(rn_status* st);

/* Use `stream` (a cudaStream_t; NULL = the library's own non-blocking stream; pass
 * cudaStreamLegacy to order with the legacy default stream) for all later work. */
int rn_set_stream(void* stream, rn_status* st);

/* Wait for all work queued on the library's stream. */
int rn_synchronize(rn_status* st);

/* The device the library runs on, for the reference's adapter record (rhi::AdapterInfo,
 * raw/rhi/rhi.hpp:39-41, which raw::gpuInit fills: raw/renderer/gpu.hpp:27). Opens the
 * context as rn_init does (RN_ERR_NO_DEVICE without a usable GPU). */
typedef struct rn_device_desc {
    char name[256];
    int cc_major, cc_minor;   /* compute capability (10.3 on GB300) */
    int sm_count;
    int driver_version;       /* cudaDriverGetVersion: 1000 x major + 10 x minor */
    int runtime_version;      /* cudaRuntimeGetVersion, same encoding */
    uint64_t total_bytes;     /* device memory */
} rn_device_desc;
int rn_device_info(rn_device_desc* out, rn_status* st);

/* Build the accelerator for `ntri` triangles (9 floats each). Replaces
 * raw::LinearAccel::build + raw::Bvh::build (src/renderer/accel.cpp:13-25,
 * src/renderer/bvh.cpp:35-92): on the GPU a PLOC binary tree (Morton codes, radix sort,
 * nearest-neighbour merge rounds) collapsed into 4-wide nodes. ntri may be 0 (every ray
 * is then open, as an empty Bvh answers). */
int rn_accel_build(const float* tris, uint32_t ntri, int flags, rn_accel** out, rn_status* st);

/* Release an accelerator (NULL is a no-op). */
void rn_accel_free(rn_accel* accel);

/* Node and triangle counts of an accelerator (for reports; any pointer may be NULL). */
int rn_accel_info(const rn_accel* accel, uint32_t* wide_nodes, uint32_t* leaf_tris,
                  uint32_t* ploc_rounds, rn_status* st);

/* Ray-traced AO and lighting model 2's visibility from the same rays.
 * Replaces raw::computeRTAO and raw::computeRTVisibility (raw/renderer/ray_ao.hpp:6-14,
 * src/renderer/ray_ao.cpp:20-63): per covered pixel `spp` cosine-weighted hemisphere rays
 * from p + 1e-3 n; ao = open / spp where open = no hit within `radius`. With RN_SKY also
 * sky = free / spp (free = open and no hit at any distance) and sun = 1 when the ray
 * towards normalize(to_light) hits nothing (or RN_SUN_FORCED). Uncovered pixels get 1.
 * `sky` and `sun` may be NULL without RN_SKY; `to_light` is read only with RN_SKY. */
int rn_ao_visibility(const rn_gbuf* g, const rn_accel* accel, int spp, float radius,
                     const float* to_light, int flags, float* ao, float* sky, float* sun,
                     rn_status* st);

/* Screen-space AO. Replaces raw::computeSSAO (raw/renderer/ssao.hpp:5-6,
 * src/renderer/ssao.cpp:11-39): `samples` taps within 6 pixels, occluded when
 * 1e-4 <= |d| <= radius and n . d/|d| > 0.15; ao = max(0, 1 - occ/used), 1 when unused. */
int rn_ssao(const rn_gbuf* g, int samples, float radius, int flags, float* ao_ss, rn_status* st);

/* Reconcile an approximation against the truth over the mask. Replaces raw::reconcile
 * (raw/cert/reconcile.hpp:12-13, src/cert/reconcile.cpp:4-21): err = |approx - truth| on
 * covered pixels and 0 elsewhere; rmse = (float)sqrt(sum_sq / pixels) with sum_sq
 * accumulated in FP64 (a fixed-order tile reduction; run-to-run deterministic);
 * within = rmse <= tolerance. `err` may be NULL. The result is written to host memory. */
int rn_reconcile(const float* approx, const float* truth, const uint8_t* mask, int w, int h,
                 float tolerance, int flags, float* err, rn_reconcile_result* out, rn_status* st);

/* The AO part of one CPU-reference frame in one call, the three passes of
 * src/renderer/render.cpp:29-54 on one stream: visibility (ao, sky, sun), SSAO with the
 * reconcile fused into its epilogue (error map, FP64 sum, max, count). Any of sky/sun/err
 * may be NULL when not wanted (sky and sun need RN_SKY). */
int rn_ao_frame(const rn_gbuf* g, const rn_accel* accel, int spp, float radius, int ss_samples,
                float tolerance, const float* to_light, int flags, float* ao, float* sky,
                float* sun, float* ao_ss, float* err, rn_reconcile_result* out, rn_status* st);

/* The PLOC binary tree exactly as raw::rt::buildPloc builds it (raw/renderer/rt_bvh.hpp:45,
 * src/renderer/rt_bvh.cpp:112-172), built on the GPU: nodes_out receives 2*ntri-1 nodes of
 * 9 int32 {left, right, tri, bits(lo.x), bits(hi.x), bits(lo.y), bits(hi.y), bits(lo.z),
 * bits(hi.z)} (leaves 0..n-1 in sorted order, then internal nodes in creation order).
 * `tris` and `nodes_out` follow RN_DEVICE_PTRS; root and rounds are host pointers. */
int rn_ploc_build(const float* tris, uint32_t ntri, int radius, int flags, int32_t* nodes_out,
                  int32_t* root, uint32_t* rounds, rn_status* st);

/* Any-hit queries for a list of rays through an accelerator: hit[i] = 1 when some
 * triangle is hit at 1e-4 < t < t_max[i] (raw::rt::occluded / raw::Bvh::occluded,
 * src/renderer/bvh.cpp:119-138). rays: 6 floats each (origin, direction). The ray-list
 * mode of the rt_trace pass (src/renderer/gpu/shaders/rt.wgsl:306-446). */
int rn_occluded(const rn_accel* accel, const float* rays, const float* t_max, uint32_t nrays,
                int flags, uint8_t* hit, rn_status* st);

/* raw::rt::closest (src/renderer/rt_bvh.cpp:125-152): for each of nrays rays (origin xyz,
 * direction xyz: 6 floats) the nearest triangle hit with 1e-4 < t < t_max[i] under the
 * reference's watertight test, ties to the lowest triangle index; tri[i] its index in the
 * accelerator's input order (-1: none), t[i] its t (-1: none). Host or device pointers. */
int rn_closest(const rn_accel* accel, const float* rays, const float* t_max, uint32_t nrays, int flags, int32_t* tri,
               float* t, rn_status* st);

/* The hybrid pass (raw::gpu_check::hybridGpu, src/renderer/gpu/rt_hybrid.cpp:43-83, with the
 * per-pixel rule of its CPU reference, src/renderer/gpu/rt_hybrid_parity.cpp:14-82) over a
 * G-buffer: for each covered pixel, d = normalize(position - eye); the geometric normal ng
 * (`geo_normal`, w x h x 3 floats, the surface triangle's normalize(cross(b - a, c - a));
 * NULL: the G-buffer normal) turned to face the viewer, and the shading normal n (the
 * G-buffer normal) turned to ng's side; each ray's origin pushed off the surface by
 * 2e-4 (1 + max |position|) along ng toward the ray; lit = 1 when nothing is hit toward
 * normalize(to_sun) below 1e30, else 0; refl_tri / refl_t = the nearest hit of the mirror
 * ray d - 2 (d.n) n (-1 / -1: none). Uncovered pixels: lit -1, refl_tri -1, refl_t -1. */
int rn_hybrid(const rn_gbuf* g, const float* geo_normal, const rn_accel* accel, const float* eye, const float* to_sun,
              int flags, float* lit, int32_t* refl_tri, float* refl_t, rn_status* st);

/* One view of a batch: its G-buffer and outputs, all DEVICE pointers. `sky`/`sun` are used
 * with RN_SKY; `ao_ss` (and `err`, optional) turn on SSAO and the reconcile for the view. */
typedef struct rn_view {
    int w, h;
    int spp;
    float radius;
    const float* position;
    const float* normal;
    const uint8_t* mask;
    float* ao;
    float* sky;
    float* sun;
    float* ao_ss;
    float* err;
} rn_view;

/* A prepared batch of views over one accelerator. */
typedef struct rn_batch rn_batch;

/* Prepare a batch (no counterpart in the reference; the batched multi-view form): up to 256
 * views of uneven size and spp over one scene. One frame of the batch is one persistent
 * traversal launch fed by a device-side tile queue over all views, one SSAO launch with each
 * view's reconcile fused in, and the copy of the per-view results; the sequence is captured
 * once into a CUDA graph here and replayed by rn_batch_run. Each view's outputs equal those
 * of rn_ao_frame on that view alone. */
int rn_batch_create(const rn_accel* accel, const rn_view* views, int nviews, int ss_samples, float tolerance,
                    const float* to_light, int flags, rn_batch** out, rn_status* st);

/* Run one frame of the batch on the library's stream and wait for it; `results` (host,
 * nviews entries, may be NULL) receives each view's reconcile. */
int rn_batch_run(rn_batch* batch, rn_reconcile_result* results, rn_status* st);

/* Traversal tiles and pixel-samples (w * h * spp summed over views) of a batch. */
int rn_batch_info(const rn_batch* batch, uint64_t* tiles, uint64_t* pixel_samples, rn_status* st);

/* Release a batch (NULL is a no-op). */
void rn_batch_free(rn_batch* batch);

/* rn_batch_create + rn_batch_run + rn_batch_free. */
int rn_ao_batch(const rn_accel* accel, const rn_view* views, int nviews, int ss_samples, float tolerance,
                const float* to_light, int flags, rn_reconcile_result* results, rn_status* st);

/* The G-buffer planes the AO passes read, rasterized on the GPU. Replaces raw::rasterize
 * (raw/renderer/raster.hpp:9, src/renderer/raster.cpp:92-126) with its default options:
 * `tris` and `nrm` hold 9 floats per triangle (the corners' positions and vertex normals,
 * in scene order); `cam` (host, 10 floats) = eye, target, up, fovy, with aspect w / h and
 * near/far 0.1/100 as raw::Camera (raw/scene/scene.hpp:12-17). Bit-identical to the CPU
 * rasterizer: the winner per pixel, its screen-linear depth, position and normal. Uncovered
 * pixels: depth +inf, position and normal 0, mask 0. `depth` may be NULL. */
int rn_raster_gbuffer(const float* tris, const float* nrm, uint32_t ntri, const float* cam, int w, int h,
                      int flags, float* depth, float* position, float* normal, uint8_t* mask,
                      rn_status* st);

/* Traversal counters for roofline accounting (no counterpart in the reference): runs the
 * visibility pass with per-ray counting on every `tile_stride`-th 8x4 tile and writes
 * counts[0] = hemisphere rays, [1] = 4-wide node fetches (128 B each), [2] = leaf-triangle
 * fetches (48 B each), [3] = sky continuation rays. Writes no image outputs. */
int rn_ao_trace_stats(const rn_gbuf* g, const rn_accel* accel, int spp, float radius,
                      const float* to_light, int flags, uint32_t tile_stride, uint64_t* counts,
                      rn_status* st);

/* rn_reconcile without any allocation, for callers that cannot let this library allocate
 * GPU memory: a host that budgets all device memory up front and refuses growth (as
 * raw-native's fail-closed frame arena does), a frame loop that must not stall on
 * cudaMalloc/cudaFree, or code that owns the device's memory through its own pool. No
 * counterpart in the reference. Same results as rn_reconcile; every buffer is a DEVICE
 * pointer (err may be NULL); work goes to `stream` (NULL = the legacy default stream) and
 * the call returns when `out` is filled. Scratch comes from a fixed 33 KiB device array in
 * the library, held on every GPU that loads it until exit; at most 2^31-1 pixels. The first
 * call on a device looks the array's address up and keeps it (not valid across a
 * cudaDeviceReset of that device: do not call it again there after a reset). No call may be
 * made on a stream under capture: each reads its result back to host memory and synchronizes
 * the stream. Calls share the array: calls that overlap on the GPU race and must be
 * serialized. */
int rn_reconcile_noalloc(const float* approx, const float* truth, const uint8_t* mask, int w, int h,
                         float tolerance, void* stream, float* err, rn_reconcile_result* out,
                         rn_status* st);

/* The whole frame (raw::renderWithParams, raw/renderer/render.hpp:43-55; src/renderer/render.cpp:99-137)
 * on the GPU: G-buffer with albedo, the AO passes, the shaded frame and its HDR view, motion.
 * tris / normals: 9 floats per triangle; albedo: 3 floats per triangle (its mesh's material
 * albedo); the light is scene.lights[0] (has_light 0: direction (0,-1,0), intensity 1).
 * camera: eye(3), target(3), up(3), fovy (aspect w / h, near 0.1, far 100). prev_view_proj:
 * the previous frame's view-projection (16 floats, row-major) for motion, or NULL (static
 * frame: zero motion). options NULL: tolerance 0.12, rtao 1, lighting 2, spp 64, radius 2,
 * ss_samples 24 (the CLI's). Any output plane may be NULL; host pointers by default, device
 * pointers with RN_DEVICE_PTRS. Every plane equals the CPU path's bit for bit. */
typedef struct rn_frame_scene {
    const float* tris;
    const float* normals;
    const float* albedo;
    uint32_t ntri;
    float light_dir[3];
    float light_intensity;
    int has_light;
} rn_frame_scene;
typedef struct rn_frame_options {
    float tolerance;
    int rtao;        /* 0: no ray-traced pass; the frame is lit with SSAO (model 1), verdict unverifiable */
    int lighting;    /* 2: sky and sun traced (the CLI default); 1: (0.2 + sun) x AO */
    int spp;
    float radius;
    int ss_samples;
} rn_frame_options;
typedef struct rn_frame_out {
    float* depth;      /* 1 float a pixel (screen-linear; +inf uncovered) */
    float* position;   /* 3 */
    float* normal;     /* 3 */
    float* albedo;     /* 3 */
    float* motion;     /* 2: current minus previous clip UV */
    uint8_t* mask;     /* 1 byte */
    float* ao_rt;      /* ray-traced AO */
    float* sky;        /* lighting model 2 */
    float* sun;
    float* ao_ss;
    float* error_map;
    float* frame;      /* 3, clamped to [0, 1] */
    float* hdr;        /* 3, unclamped linear radiance */
    rn_reconcile_result rec;
    int motion_valid, motion_total;
    float view_proj[16];
} rn_frame_out;
int rn_render_frame(const rn_frame_scene* scene, const float* camera, const float* prev_view_proj, int w, int h,
                    const rn_frame_options* options, int flags, rn_frame_out* out, rn_status* st);

/* GTAO (ground-truth-based ambient occlusion, Jimenez et al. 2016): raw::post::gtao over
 * raw::post::viewGBuffer (raw/renderer/post.hpp:23-30; src/renderer/post_gtao.cpp:36-135),
 * the screen-space approximation judged, like SSAO, by the traced AO through rn_reconcile.
 * camera: eye(3), target(3), up(3), fovy (aspect w / h). radius in world units (the
 * reference's default 0.5), slices and steps per side (16, 16). ao receives 1 off the
 * coverage. FP32 on the GPU against the reference's FP64: |gpu - cpu| <= 1e-3 on all but
 * 0.1 % of pixels, the reference's own bound for its GPU pass (raw/renderer/post_parity.hpp:15-19). */
int rn_gtao(const rn_gbuf* g, const float* camera, float radius, int slices, int steps, int flags, float* ao,
            rn_status* st);

/* Self-test of the device-side wait budget (no counterpart in the reference): runs a small
 * tensor-core GEMM with one stage's copies withheld, so that its bounded mbarrier wait runs
 * out after spin_limit rounds (1 .. 2^24). Returns RN_ERR_BUDGET from the device error word,
 * with the kernel having freed its TMEM and returned; the context stays usable. */
int rn_selftest_wait_budget(uint32_t spin_limit, rn_status* st);

/* Launch-shape tuning (no counterpart in the reference; no key changes a per-pixel result).
 * Keys and values:
 *   trace_min_blocks  2 | 3 | 4      resident traversal blocks per SM (register budget)
 *   batch_min_blocks  2 | 3 | 4      ... of the batched multi-view traversal (rn_batch_*)
 *   trace_frontier    0 | 1          per-warp frontier for AO-only walks
 *   trace_frontier_min_spp 1|8|16|32 ... built only at this spp or more
 *   trace_frontier_tail 0|4|8|16     greedy steps after the level-by-level build (<= spp / 16)
 *   trace_packet      4 | 8 | 16     a warp's pixel packet: packet x (32 / packet)
 *   trace_stack       48 | 96        traversal stack entries (48 only where the tree allows)
 *   ssao_tile_h       4 | 8 | 16     SSAO tile 32 x h (the fused FP64 sum follows the tiling)
 *   conv_bn_max       64 | 128 | 256 widest GEMM tile of the surrogate's convolutions
 *   conv_halo         0 | 1          128-pixel row tiles from a ring of one-row boxes (where they fit)
 *   conv_pair         0 | 1          per-tap convolutions: two 128-pixel tiles per weight box
 *   accel_radius      8|16|32|64     PLOC search radius of accelerators built afterwards
 *   accel_leaf        1 | 2 | 4 | 8  their largest leaf (triangles), 65,536 triangles or more
 *   accel_leaf_small  1 | 2 | 4 | 8  ... below 65,536 triangles
 *   frame_direct      0 | 1          rn_ao_frame on pinned, mapped host buffers without copies
 *   hybrid_min_blocks 5 | 6 | 8      resident rn_hybrid blocks per SM (register budget)
 *   trace_leaf_pass   0 | 1          rn_ao_visibility: a node's leaf children tested after its
 *                                    four slab tests, in one loop
 *   conv_tmem_a       0 | 1          row-ring convolutions with at most 32 input and 32 output
 *                                    channels keep each input row's A operands in TMEM
 *   ploc_tail         0|4096|16384|32768|65536|262144  accelerator builds: the PLOC rounds
 *                                    from this many clusters on run in one launch (0: a launch
 *                                    per step)
 *   ploc_tail_ctas    1|4|8|16       ... in one block of 1024 threads (1) or one thread-block
 *                                    cluster of this many such blocks
 *   ploc_fused        0 | 1          accelerator builds: a PLOC round's prefix sum, scatter and
 *                                    commit in one launch (decoupled look-back) instead of four
 *   collapse_block    0|16384|65536|262144  accelerator builds of at most this many triangles
 *                                    collapse to 4-wide nodes in one block (0: a launch per level)
 *   trace_pool        0|16|24|32     AO-only walks: one queue of a packet's walks, idle lanes
 *                                    refilled when fewer than this many walk (0: one pixel per lane)
 *   trace_pool_sort   0 | 1          ... the queue ordered by the walks' direction octant (at most
 *                                    16 spp)
 *   pt_wave           0|1|64|256|1024|2048  rn_pathtrace: the wavefront form (a bounce as shade, shadow-ray
 *                                    and closest-hit kernels over this many x 1024 path slots;
 *                                    0: one kernel a path, below)
 *   pt_shade_blocks   4|6|8          rn_pathtrace: the wavefront shade kernel's resident
 *                                    128-thread blocks per SM (its register budget)
 *   pt_regen          0|4|8|16       rn_pathtrace: persistent threads that start a new path when
 *                                    theirs ends, this many 128-thread blocks per SM (0: a thread a sample)
 *   pt_slice          0|1|4|16       rn_pathtrace: samples traced per slice at most (0: as many
 *                                    as 2 GiB of per-sample terms hold)
 * Process-wide; RN_TUNE_<KEY> environment variables apply before the first call.
 * rn_tune_load reads "key = value" lines ('#' comments), all or nothing. */
int rn_tune_set(const char* key, int value, rn_status* st);
int rn_tune_get(const char* key, int* value, rn_status* st);
int rn_tune_load(const char* path, rn_status* st);

/* The learned surrogate's tensor-core GEMM (no counterpart in the reference): C = P * Q^T,
 * P (M x K) and Q (N x K) BF16 row-major with K contiguous (row strides ldp, ldq, multiples
 * of 8), FP32 accumulation on tcgen05 with TMEM, output FP32 (`c32`) and/or BF16 (`c16`) with
 * row stride ldc, optional bias[N] and ReLU. M % 128 == 0; N one of 32, 64, 128, 256 or a
 * multiple of 128; K % (64 * splits) == 0; splits > 1 adds FP32 partials atomically into c32
 * (which the caller zeroes). Device pointers, the library's stream, asynchronous. */
int rn_tc_gemm(const void* P, int ldp, const void* Q, int ldq, int M, int N, int K, int splits, float* c32,
               void* c16, int ldc, const float* bias, int relu, rn_status* st);

/* The surrogate's implicit-GEMM 3x3 convolution (no counterpart in the reference), stride 1,
 * zero padding 1: out[b,y,x,n] = bias[n] + sum over taps t = 3 (dy+1) + (dx+1) and input
 * channels ci of in[b, y+dy, x+dx, ci] * w[n][t * Cin + ci], the input being src0's c0
 * channels followed by src1's c1 (src1 may be null). Sources are NHWC BF16 [B][H][W][c],
 * c a multiple of 32 (or of 16 when W is a multiple of 128, N is 32 or 64 and the weights
 * fit in shared memory); w is BF16 [N][ldw], ldw >= 9 Cin, N <= 512 (32, 64, 128, 256 or a
 * multiple of 128); outputs [B][H][W][N] as FP32 (c32)
 * and/or BF16 (c16), optional ReLU; up16 (with c16) also receives the BF16 output upsampled
 * 2x by nearest neighbour, [B][2H][2W][N]. W's largest power-of-two divisor (at most 128),
 * TW, sets the tile (128 / TW rows must divide H). Device pointers, the library's stream. */
int rn_tc_conv3x3(const void* src0, int c0, const void* src1, int c1, int B, int H, int W, const void* w, int ldw,
                  int N, float* c32, void* c16, void* up16, const float* bias, int relu, rn_status* st);

/* The learned AO surrogate (no counterpart in the reference): a BF16 U-Net, 4 levels of
 * 32/64/128/256 channels, two 3x3 convolutions + ReLU per level, average-pool down, nearest up
 * with skip concatenation, a 1x1 sigmoid head; every convolution (forward, data gradient,
 * weight gradient) on the tcgen05 GEMM, FP32 accumulation, Adam on FP32 master weights.
 * A network is created for one input shape: batch x height x width, height and width
 * multiples of 16 and batch * (height/8) * (width/8) a multiple of 128. Inputs are DEVICE
 * FP32 [batch][height][width][5] (depth / radius, normal xyz, 4-spp AO); outputs and targets
 * DEVICE FP32 [batch][height][width]. */
typedef struct rn_unet rn_unet;
/* flags: RN_UNET_INFERENCE creates a forward-only network (no gradient storage;
 * rn_unet_train_step is refused). Convolutions with >= 32 input channels run as implicit
 * GEMMs (rn_tc_conv3x3) when every level's size can be tiled, else on explicit im2col rows
 * and the GEMM; RN_UNET_EXPLICIT forces the latter (same arithmetic, for comparison). */
#define RN_UNET_INFERENCE 1u
#define RN_UNET_EXPLICIT 2u
int rn_unet_create(int batch, int height, int width, uint64_t seed, uint32_t flags, rn_unet** out, rn_status* st);
void rn_unet_free(rn_unet* net);
int rn_unet_param_count(const rn_unet* net, uint64_t* count, rn_status* st);
/* Predicted AO into `output` (asynchronous on the library's stream). */
int rn_unet_forward(rn_unet* net, const float* input, int batch, float* output, rn_status* st);
/* One Adam step on the mean squared error against `target` (lr 0: gradients only); writes
 * the batch's loss to *loss (host). */
int rn_unet_train_step(rn_unet* net, const float* input, const float* target, int batch, float lr, float* loss,
                       rn_status* st);
/* Parameters / last gradients as FP32 host arrays: per convolution w[cout][9 cin] (tap-major,
 * input channel fastest) then b[cout], then the head's w[32] and b. */
/* Data-parallel training: a step in two halves with the gradients exchanged between them
 * (rn_unet_train_step is rn_unet_backward then rn_unet_apply). rn_unet_backward runs the
 * forward and backward passes on this rank's batch and leaves the gradients in the network
 * (loss: the batch's mean squared error); rn_unet_grads_flat copies them to (to_flat 1) or
 * from (0) a flat DEVICE FP32 array of rn_unet_grad_count values, asynchronously on the
 * library's stream, for an all-reduce between the ranks; rn_unet_apply clips and takes the
 * Adam step (lr 0: no update) from the gradients the network then holds. */
int rn_unet_backward(rn_unet* net, const float* input, const float* target, int batch, float* loss, rn_status* st);
int rn_unet_grad_count(const rn_unet* net, uint64_t* count, rn_status* st);
int rn_unet_grads_flat(rn_unet* net, float* dev, int to_flat, rn_status* st);
int rn_unet_apply(rn_unet* net, float lr, rn_status* st);
int rn_unet_get_params(rn_unet* net, float* host, rn_status* st);
int rn_unet_set_params(rn_unet* net, const float* host, rn_status* st);
int rn_unet_get_grads(rn_unet* net, float* host, rn_status* st);
/* Adaptive gradient clipping for later train steps: the global gradient norm is limited to
 * ratio x a running mean of the past clipped norms (0, the default, turns it off); a
 * non-finite gradient skips the update. The last step's norm and applied factor: */
int rn_unet_set_clip(rn_unet* net, float ratio, rn_status* st);
int rn_unet_last_grad_norm(const rn_unet* net, float* norm, float* scale, rn_status* st);
/* Training state for checkpoints: 3 x param_count FP32 host values (master weights, Adam's
 * first moments, second moments, each in the parameters' layout) and the step count. */
int rn_unet_get_state(rn_unet* net, float* host, uint64_t* step, rn_status* st);
int rn_unet_set_state(rn_unet* net, const float* host, uint64_t step, rn_status* st);

/* One AO frame by the surrogate (no counterpart in the reference): the 4-spp trace of the
 * G-buffer, the network on (depth over radius relative to the covered pixels' mean depth,
 * normal, 4-spp AO), then per 16 x 16 tile the confidence-band test: a tile whose predicted
 * mean leaves mean(ao4) +- k sigma (sigma = max(sqrt(sum p (1 - p) / 4) / n, 0.5 / sqrt(4 n))
 * over its n covered pixels) is traced at spp_full and its traced values replace the
 * prediction. ao receives the frame (1 off the coverage). Optional outputs: ao4 (the 4-spp
 * trace), pred (the network alone), tile_flags (ceil(h/16) x ceil(w/16), 1 = traced).
 * DEVICE pointers only (G-buffer planes, depth, outputs); `net` was created with batch 1 for
 * a shape covering w x h. Synchronizes the library's stream to return the stats. */
typedef struct rn_surrogate_stats {
    uint32_t tiles_covered;   /* tiles with a covered pixel */
    uint32_t tiles_fallback;  /* of those, traced at spp_full */
    float mean_depth;         /* the covered pixels' mean depth the features used */
    float reserved;
} rn_surrogate_stats;
int rn_surrogate_ao(rn_unet* net, const rn_gbuf* g, const float* depth, const rn_accel* accel, int spp_full,
                    float radius, float k, float* ao, float* ao4, float* pred, uint8_t* tile_flags,
                    rn_surrogate_stats* stats, rn_status* st);

/* ------------------------------------------------------------------ path tracer
 * raw-native's path tracer, interface v4 (raw/renderer/rt_pathtrace.hpp), for scenes that set
 * no v3 field: the v4 lobe (Lambert base under GGX with height-correlated Smith, Schlick
 * Fresnel and Kulla-Conty multiple scattering, weighted by the float64-built energy table of
 * src/renderer/rt_pt_energy.cpp), next-event estimation for the sun and for emissive
 * triangles with MIS, Russian roulette after bounce 3, and every AOV, each equal to
 * raw::rt::pathTraceCpu's (src/renderer/rt_pt_cpu.cpp) bit for bit for the same scene and
 * description: counter-based random numbers, the CPU's float32 operation order, the host
 * libm's cos/sin bits and the moments in float64. Scenes with v3 fields (punctual lights,
 * an environment, full glTF materials) are CPU-only in the reference too. */
typedef struct rn_pt_material {   /* raw::rt::PtMaterial (rt_pathtrace.hpp:43-49) */
    float base_factor;            /* base colour = texel / 255 x base_factor */
    float roughness;              /* GGX alpha = roughness^2 */
    float metallic;
    float specular;               /* scales the dielectric F0 of 0.04; 0: pure Lambert */
    float emission[3];            /* two-sided radiance */
} rn_pt_material;
/* The scene as raw::rt::PtScene holds it (swr::Geometry, swr::TextureSet, one material per
 * texture id, sun and sky; rt_pathtrace.hpp:50-63): vertex positions, normals and uvs;
 * three vertex indices and one texture id a triangle; per texture its texel offset, width
 * and height (powers of two), RGBA8 texels with red in the low byte. HOST pointers. */
typedef struct rn_pt_scene_desc {
    const float* pos;             /* 3 a vertex */
    const float* nrm;             /* 3 a vertex */
    const float* uv;              /* 2 a vertex */
    uint32_t nvert;
    const uint32_t* idx;          /* 3 a triangle */
    const uint32_t* tri_texture;  /* 1 a triangle */
    uint32_t ntri;
    const uint32_t* tex_entries;  /* offset, width, height a texture */
    uint32_t ntex;
    const uint32_t* texels;
    uint32_t ntexels;
    const rn_pt_material* materials;   /* ntex of them */
    float sun_dir[3];             /* toward the sun; normalized by the tracer */
    float sun_irradiance[3];      /* 0: no sun */
    float sky[3];                 /* constant radiance on escape */
} rn_pt_scene_desc;
typedef struct rn_ptscene rn_ptscene;
/* raw::rt::finishPtScene (src/renderer/rt_pt_scene.cpp:31-45) on the GPU: the scene copied to
 * the device, its triangle list's accelerator (rn_accel_build), the emitter list and its
 * inclusive area CDF (float, in triangle order, formed on the host as the reference forms it),
 * and the lobe's energy table (built once per process on the host in float64, the
 * reference's construction, then kept on the device). */
int rn_pt_scene_create(const rn_pt_scene_desc* scene, rn_ptscene** out, rn_status* st);
void rn_pt_scene_free(rn_ptscene* scene);
/* Emitter count and total emitter area of a scene (finishPtScene's emitters / emitterArea). */
int rn_pt_scene_info(const rn_ptscene* scene, uint32_t* emitters, float* emitter_area, rn_status* st);

#define RN_PT_DROP_LAMBERT_COSINE     0x01   /* raw::rt::PtControls (rt_pathtrace.hpp:72-80) */
#define RN_PT_MIS_WEIGHT_ONE          0x02
#define RN_PT_AOV_DROP_SPECULAR_INDIRECT 0x04
#define RN_PT_AOV_EMISSION_TO_DIFFUSE 0x08
#define RN_PT_LEGACY_LOBE_V2          0x10
/* raw::rt::PathTraceDesc (rt_pathtrace.hpp:82-92). Cameras: eye(3), target(3), up(3), fovy. */
typedef struct rn_pt_desc {
    uint64_t seed;
    uint32_t spp, spp_begin, max_bounces;
    int32_t width, height;
    float camera[10];
    float previous[10];           /* for motion; equal to camera for a still frame */
    int32_t jitter;
    int32_t russian_roulette;
    uint32_t controls;            /* RN_PT_* */
} rn_pt_desc;
/* raw::rt::PathTraceOutput's planes (rt_pathtrace.hpp:94-104); any may be NULL. */
typedef struct rn_pt_out {
    float* radiance;              /* 3 a pixel */
    float* albedo;                /* 3 */
    float* normal;                /* 3 */
    float* depth;                 /* 1 */
    float* variance;              /* 1 */
    int32_t* triangle;            /* 1 */
    float* motion;                /* 2 */
    float* diffuse;               /* 3 */
    float* specular;              /* 3 */
    float* emission;              /* 3 */
    float* diffuse_albedo;        /* 3 */
    float* specular_albedo;       /* 3 */
    float* diffuse_variance;      /* 1 */
    float* specular_variance;     /* 1 */
} rn_pt_out;
/* raw::rt::pathTraceCpu / raw::gpu_check::pathTraceGpu (rt_pathtrace.hpp:135-136,
 * rt_pt_gpu.hpp:13) on the GPU. Output planes are host pointers unless flags has
 * RN_DEVICE_PTRS. Samples are traced in parallel and summed per pixel in sample order, so
 * the result is pathTraceCpu's for any launch shape. */
int rn_pathtrace(const rn_ptscene* scene, const rn_pt_desc* desc, int flags, rn_pt_out* out, rn_status* st);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif  /* RN_AO_H */
