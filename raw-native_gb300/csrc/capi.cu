// capi.cu -- the C ABI of librn_ao.so (include/rn_ao.h): the process-wide device context,
// the sampler's host-libm calibration, workspace management, and the entry points that
// stage host buffers, launch the kernels and return results.
#include "rn_internal.h"
#include "rn_device.cuh"
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <thread>
#include <vector>

namespace rn {

Context& ctx() {
    static Context c;
    return c;
}

int fail(rn_status* st, int code, const char* fmt, ...) {
    if (st) {
        st->code = code;
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(st->message, sizeof st->message, fmt, ap);
        va_end(ap);
    }
    return code;
}
int ok(rn_status* st) {
    if (st) { st->code = RN_OK; st->message[0] = '\0'; }
    return RN_OK;
}
int cuda_fail(rn_status* st, cudaError_t e, const char* what) {
    int code = RN_ERR_CUDA;
    if (e == cudaErrorMemoryAllocation) code = RN_ERR_NO_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) code = RN_ERR_NO_DEVICE;
    return fail(st, code, "%s: %s", what, cudaGetErrorString(e));
}

// ---------------------------------------------------------------- sampler calibration
namespace {
constexpr uint32_t kAngles = 1u << 24;

// One byte per sample angle: host-minus-device bit difference of cos (low nibble) and sin
// (high nibble). `bad` counts angles whose difference does not fit in [-8, 7].
__global__ void trig_corr_kernel(const float2* __restrict__ host_cs, uint8_t* __restrict__ corr, uint32_t* bad) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= kAngles) return;
    float s, c;
    angle_sincos(sample_angle(k), s, c);
    const float2 h = host_cs[k];
    const int dc = __float_as_int(h.x) - __float_as_int(c);
    const int ds = __float_as_int(h.y) - __float_as_int(s);
    uint8_t v = 0;
    if (dc >= -8 && dc <= 7 && ds >= -8 && ds <= 7)
        v = (uint8_t)((dc & 15) | ((ds & 15) << 4));
    else
        atomicAdd(bad, 1u);
    corr[k] = v;
}
}  // namespace

// The reference's directions depend on the host libm's cosf/sinf at phi = 6.2831853f * k/2^24.
// Evaluate both on every one of the 2^24 angles (host threads), upload, and let the device
// record its own angle_sincos's difference from them.
int build_trig_correction(Context& c, rn_status* st) {
    std::vector<float> host((size_t)kAngles * 2);
    unsigned nt = std::thread::hardware_concurrency();
    if (nt < 1) nt = 1;
    if (nt > 64) nt = 64;
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; ++t)
        pool.emplace_back([&host, t, nt] {
            for (uint32_t k = t; k < kAngles; k += nt) {
                const float u = (float)k / 16777216.0f;
                const float phi = 6.2831853f * u;
                host[2 * (size_t)k] = ::cosf(phi);
                host[2 * (size_t)k + 1] = ::sinf(phi);
            }
        });
    for (auto& th : pool) th.join();
    ScopedDev host_buf, bad_buf;
    RN_CUDA(cudaMalloc((void**)&c.trig_corr, kAngles), st);
    RN_CUDA(cudaMalloc(&host_buf.p, (size_t)kAngles * sizeof(float2)), st);
    RN_CUDA(cudaMalloc(&bad_buf.p, 4), st);
    float2* d_host = (float2*)host_buf.p;
    uint32_t* d_bad = (uint32_t*)bad_buf.p;
    RN_CUDA(cudaMemsetAsync(d_bad, 0, 4, c.stream), st);
    RN_CUDA(cudaMemcpyAsync(d_host, host.data(), (size_t)kAngles * sizeof(float2), cudaMemcpyHostToDevice, c.stream), st);
    trig_corr_kernel<<<kAngles / 256, 256, 0, c.stream>>>(d_host, c.trig_corr, d_bad);
    RN_CUDA(cudaGetLastError(), st);
    uint32_t bad = 0;
    RN_CUDA(cudaMemcpyAsync(&bad, d_bad, 4, cudaMemcpyDeviceToHost, c.stream), st);
    RN_CUDA(cudaStreamSynchronize(c.stream), st);
    if (bad) return fail(st, RN_ERR_STATE, "sampler calibration: %u angles differ by more than 7 ulp", bad);
    return RN_OK;
}

// ------------------------------------------------------------------ launch-shape tuning
namespace {
struct TuneKey {
    const char* name;
    const char* env;
    int Tune::*field;
    int allowed[6];
    int nallowed;
};
const TuneKey kTuneKeys[] = {
    {"trace_min_blocks", "RN_TUNE_TRACE_MIN_BLOCKS", &Tune::trace_min_blocks, {2, 3, 4}, 3},
    {"batch_min_blocks", "RN_TUNE_BATCH_MIN_BLOCKS", &Tune::batch_min_blocks, {2, 3, 4}, 3},
    {"trace_frontier", "RN_TUNE_TRACE_FRONTIER", &Tune::trace_frontier, {0, 1}, 2},
    {"trace_frontier_min_spp", "RN_TUNE_TRACE_FRONTIER_MIN_SPP", &Tune::trace_frontier_min_spp, {1, 8, 16, 32}, 4},
    {"trace_frontier_tail", "RN_TUNE_TRACE_FRONTIER_TAIL", &Tune::trace_frontier_tail, {0, 4, 8, 16}, 4},
    {"trace_packet", "RN_TUNE_TRACE_PACKET", &Tune::trace_packet, {4, 8, 16}, 3},
    {"trace_stack", "RN_TUNE_TRACE_STACK", &Tune::trace_stack, {48, 96}, 2},
    {"ssao_tile_h", "RN_TUNE_SSAO_TILE_H", &Tune::ssao_tile_h, {4, 8, 16}, 3},
    {"conv_bn_max", "RN_TUNE_CONV_BN_MAX", &Tune::conv_bn_max, {64, 128, 256}, 3},
    {"conv_halo", "RN_TUNE_CONV_HALO", &Tune::conv_halo, {0, 1}, 2},
    {"conv_pair", "RN_TUNE_CONV_PAIR", &Tune::conv_pair, {0, 1}, 2},
    {"accel_radius", "RN_TUNE_ACCEL_RADIUS", &Tune::accel_radius, {8, 16, 32, 64}, 4},
    {"accel_leaf", "RN_TUNE_ACCEL_LEAF", &Tune::accel_leaf, {1, 2, 4, 8}, 4},
    {"accel_leaf_small", "RN_TUNE_ACCEL_LEAF_SMALL", &Tune::accel_leaf_small, {1, 2, 4, 8}, 4},
    {"frame_direct", "RN_TUNE_FRAME_DIRECT", &Tune::frame_direct, {0, 1}, 2},
    {"hybrid_min_blocks", "RN_TUNE_HYBRID_MIN_BLOCKS", &Tune::hybrid_min_blocks, {5, 6, 8}, 3},
    {"pt_slice", "RN_TUNE_PT_SLICE", &Tune::pt_slice, {0, 1, 4, 16}, 4},
    {"pt_regen", "RN_TUNE_PT_REGEN", &Tune::pt_regen, {0, 4, 8, 16}, 4},
    {"pt_wave", "RN_TUNE_PT_WAVE", &Tune::pt_wave, {0, 1, 64, 256, 1024, 2048}, 6},
    {"pt_shade_blocks", "RN_TUNE_PT_SHADE_BLOCKS", &Tune::pt_shade_blocks, {4, 6, 8}, 3},
    {"trace_pool", "RN_TUNE_TRACE_POOL", &Tune::trace_pool, {0, 16, 24, 32}, 4},
    {"ploc_tail", "RN_TUNE_PLOC_TAIL", &Tune::ploc_tail, {0, 4096, 16384, 32768, 65536, 262144}, 6},
    {"ploc_tail_ctas", "RN_TUNE_PLOC_TAIL_CTAS", &Tune::ploc_tail_ctas, {1, 4, 8, 16}, 4},
    {"ploc_fused", "RN_TUNE_PLOC_FUSED", &Tune::ploc_fused, {0, 1}, 2},
    {"collapse_block", "RN_TUNE_COLLAPSE_BLOCK", &Tune::collapse_block, {0, 16384, 65536, 262144}, 4},
    {"conv_tmem_a", "RN_TUNE_CONV_TMEM_A", &Tune::conv_tmem_a, {0, 1}, 2},
    {"conv_fan", "RN_TUNE_CONV_FAN", &Tune::conv_fan, {0, 1}, 2},
    {"conv_fan_bn", "RN_TUNE_CONV_FAN_BN", &Tune::conv_fan_bn, {32, 64}, 2},
    {"trace_leaf_pass", "RN_TUNE_TRACE_LEAF_PASS", &Tune::trace_leaf_pass, {0, 1}, 2},
    {"trace_pool_sort", "RN_TUNE_TRACE_POOL_SORT", &Tune::trace_pool_sort, {0, 1}, 2},
};

const TuneKey* find_tune_key(const char* name) {
    for (const TuneKey& k : kTuneKeys)
        if (std::strcmp(k.name, name) == 0) return &k;
    return nullptr;
}

int tune_assign(const char* name, int value, rn_status* st) {
    const TuneKey* k = find_tune_key(name);
    if (!k) return fail(st, RN_ERR_INVALID, "unknown tuning key '%s'", name);
    for (int i = 0; i < k->nallowed; ++i)
        if (k->allowed[i] == value) {
            ctx().tune.*(k->field) = value;
            return RN_OK;
        }
    return fail(st, RN_ERR_INVALID, "tuning key '%s' does not take %d", name, value);
}

// RN_TUNE_<KEY> environment variables, applied once before any other tuning call.
void tune_env_once() {
    static bool done = false;
    if (done) return;
    done = true;
    for (const TuneKey& k : kTuneKeys)
        if (const char* v = getenv(k.env)) {
            rn_status ignored;
            tune_assign(k.name, atoi(v), &ignored);
        }
}

int packet_log2(int packet) { return packet == 4 ? 2 : packet == 16 ? 4 : 3; }

}  // namespace

TraceParams ao_trace_params(const float* pos, const float* nrm, const uint8_t* mask, int w, int h,
                            const rn_accel* accel, int spp, float radius) {
    Context& c = ctx();
    TraceParams p{};
    p.w = w; p.h = h;
    p.pos = pos; p.nrm = nrm; p.mask = mask;
    p.nodes = accel->d_nodes; p.tris = accel->d_tris;
    p.has_geometry = accel->ntri > 0;
    p.spp = spp; p.radius = radius;
    p.lx = 0.0f; p.ly = 1.0f; p.lz = 0.0f;
    p.corr = c.trig_corr;
    p.err_word = c.dev_error;
    apply_tune(p, accel);
    return p;
}

int trace_ao_device(const float* pos, const float* nrm, const uint8_t* mask, int w, int h, const rn_accel* accel,
                    int spp, float radius, float* ao, rn_status* st) {
    Context& c = ctx();
    TraceParams p{};
    p.w = w; p.h = h;
    p.pos = pos; p.nrm = nrm; p.mask = mask;
    p.nodes = accel->d_nodes; p.tris = accel->d_tris;
    p.has_geometry = accel->ntri > 0;
    p.spp = spp; p.radius = radius;
    p.want_sky = 0; p.sun_forced = 0;
    p.lx = 0.0f; p.ly = 1.0f; p.lz = 0.0f;
    p.corr = c.trig_corr;
    p.ao = ao; p.sky = nullptr; p.sun = nullptr;
    p.err_word = c.dev_error;
    apply_tune(p, accel);
    if (launch_trace(p, c.sm_count, c.stream) != RN_OK) return cuda_fail(st, cudaGetLastError(), "trace_kernel");
    return RN_OK;
}

void apply_tune(TraceParams& p, const rn_accel* accel) {
    const Tune& t = ctx().tune;
    p.frontier = t.trace_frontier && p.spp >= t.trace_frontier_min_spp;
    p.stack_need = 16 + 3 * (int)(accel ? accel->depth : 0);
    // the frontier's seeds sit under the walk's own pushes: without room for both, walk from the root
    if (p.stack_need > 96) p.frontier = 0;
    p.packet_log2 = packet_log2(t.trace_packet);
    // the greedy tail costs a node fetch per step and packet, and saves per ray: one step per
    // 16 samples, up to the tuned count
    p.frontier_tail = std::min(t.trace_frontier_tail, p.spp / 16);
}

int ensure_ctx(rn_status* st) {
    Context& c = ctx();
    if (c.ready) return RN_OK;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return fail(st, RN_ERR_NO_DEVICE, "no CUDA device (%s)", e == cudaSuccess ? "count 0" : cudaGetErrorString(e));
    int dev = 0;
    RN_CUDA(cudaGetDevice(&dev), st);
    cudaDeviceProp prop;
    RN_CUDA(cudaGetDeviceProperties(&prop, dev), st);
    if (!(prop.major == 10 && prop.minor == 3))
        return fail(st, RN_ERR_NO_DEVICE, "device %d (%s) is sm_%d%d; librn_ao.so is built for sm_103a", dev, prop.name,
                    prop.major, prop.minor);
    c.device = dev;
    c.sm_count = prop.multiProcessorCount;
    tune_env_once();
    RN_CUDA(cudaStreamCreateWithFlags(&c.own_stream, cudaStreamNonBlocking), st);
    c.stream = c.own_stream;
    RN_CUDA(cudaMalloc((void**)&c.dev_error, 64), st);
    RN_CUDA(cudaMemsetAsync(c.dev_error, 0, 64, c.stream), st);
    // the library's own pool for accelerators (rebuilt per scene, often per frame): a freed
    // accelerator's memory stays mapped for the next build instead of going back to the driver
    cudaMemPoolProps pp = {};
    pp.allocType = cudaMemAllocationTypePinned;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = dev;
    RN_CUDA(cudaMemPoolCreate(&c.accel_pool, &pp), st);
    uint64_t keep = (uint64_t)4 << 30;
    RN_CUDA(cudaMemPoolSetAttribute(c.accel_pool, cudaMemPoolAttrReleaseThreshold, &keep), st);
    RN_TRY(build_trig_correction(c, st));
    c.ready = true;
    return RN_OK;
}

int ws_get(Slot s, size_t bytes, void** out, rn_status* st) {
    DevBuf& b = ctx().ws[s];
    if (bytes == 0) bytes = 16;
    if (b.cap < bytes) {
        if (b.ptr) {
            RN_CUDA(cudaStreamSynchronize(ctx().stream), st);
            cudaFree(b.ptr);
            b.ptr = nullptr;
            b.cap = 0;
        }
        const size_t cap = (bytes + 4095) & ~size_t(4095);
        RN_CUDA(cudaMalloc(&b.ptr, cap), st);
        // reduction counters must start at zero; every kernel leaves them at zero
        RN_CUDA(cudaMemsetAsync(b.ptr, 0, cap, ctx().stream), st);
        b.cap = cap;
    }
    *out = b.ptr;
    return RN_OK;
}

int check_device_error(rn_status* st, const char* where) {
    Context& c = ctx();
    uint32_t word = 0;
    RN_CUDA(cudaMemcpyAsync(&word, c.dev_error, 4, cudaMemcpyDeviceToHost, c.stream), st);
    RN_CUDA(cudaStreamSynchronize(c.stream), st);
    if (word) {
        RN_CUDA(cudaMemsetAsync(c.dev_error, 0, 4, c.stream), st);
        const int code = (word & (DEV_STACK_OVERFLOW | DEV_QUEUE_OVERFLOW)) ? RN_ERR_OVERFLOW : RN_ERR_BUDGET;
        return fail(st, code, "%s: device error word 0x%x (%s)", where, word,
                    (word & DEV_STACK_OVERFLOW) ? "traversal stack overflow"
                    : (word & DEV_GUARD)        ? "iteration budget exhausted"
                                                : "queue overflow");
    }
    return RN_OK;
}

}  // namespace rn

using namespace rn;

namespace {

// Stage a host buffer into a workspace slot (or pass a device pointer through).
template <typename T>
int stage_in(const T* p, size_t count, bool dev, Slot slot, const T** out, rn_status* st) {
    if (dev || p == nullptr) { *out = p; return RN_OK; }
    void* d = nullptr;
    RN_TRY(ws_get(slot, count * sizeof(T), &d, st));
    RN_CUDA(cudaMemcpyAsync(d, p, count * sizeof(T), cudaMemcpyHostToDevice, ctx().stream), st);
    *out = (const T*)d;
    return RN_OK;
}
template <typename T>
int stage_out(T* p, size_t count, bool dev, Slot slot, T** out, rn_status* st) {
    if (dev || p == nullptr) { *out = p; return RN_OK; }
    void* d = nullptr;
    RN_TRY(ws_get(slot, count * sizeof(T), &d, st));
    *out = (T*)d;
    return RN_OK;
}
template <typename T>
int copy_back(T* host, const T* dev, size_t count, rn_status* st) {
    if (host == nullptr || host == dev) return RN_OK;
    RN_CUDA(cudaMemcpyAsync(host, dev, count * sizeof(T), cudaMemcpyDeviceToHost, ctx().stream), st);
    return RN_OK;
}

int check_gbuf(const rn_gbuf* g, rn_status* st) {
    if (!g) return fail(st, RN_ERR_INVALID, "null G-buffer");
    if (g->w <= 0 || g->h <= 0) return fail(st, RN_ERR_INVALID, "G-buffer size %dx%d", g->w, g->h);
    if ((size_t)g->w * (size_t)g->h > (size_t)1 << 31) return fail(st, RN_ERR_INVALID, "G-buffer larger than 2^31 pixels");
    if (!g->position || !g->normal || !g->mask) return fail(st, RN_ERR_INVALID, "G-buffer plane is null");
    return RN_OK;
}

struct StagedGbuf { const float* pos; const float* nrm; const uint8_t* mask; };

// A buffer of the frame: the caller's device array when it passed one, else workspace.
template <typename T>
int frame_buf(T* p, size_t count, bool dev, Slot slot, T** out, rn_status* st) {
    if (dev && p) { *out = p; return RN_OK; }
    void* d = nullptr;
    RN_TRY(ws_get(slot, count * sizeof(T), &d, st));
    *out = (T*)d;
    return RN_OK;
}

int stage_gbuf(const rn_gbuf* g, bool dev, StagedGbuf* s, rn_status* st) {
    const size_t np = (size_t)g->w * g->h;
    RN_TRY(stage_in(g->position, np * 3, dev, WS_POS, &s->pos, st));
    RN_TRY(stage_in(g->normal, np * 3, dev, WS_NRM, &s->nrm, st));
    RN_TRY(stage_in(g->mask, np, dev, WS_MASK, &s->mask, st));
    return RN_OK;
}

TraceParams vis_params(const StagedGbuf& g, int w, int h, const rn_accel* accel, int spp, float radius,
                       const float* to_light, int flags, float* ao, float* sky, float* sun) {
    Context& c = ctx();
    TraceParams p{};
    p.w = w; p.h = h;
    p.pos = g.pos; p.nrm = g.nrm; p.mask = g.mask;
    p.nodes = accel->d_nodes; p.tris = accel->d_tris;
    p.has_geometry = accel->ntri > 0;
    p.spp = spp; p.radius = radius;
    p.want_sky = (flags & RN_SKY) != 0;
    p.sun_forced = (flags & RN_SUN_FORCED) != 0;
    if (p.want_sky) { p.lx = to_light[0]; p.ly = to_light[1]; p.lz = to_light[2]; }
    else { p.lx = 0.0f; p.ly = 1.0f; p.lz = 0.0f; }
    p.corr = (flags & RN_DEVICE_TRIG) ? nullptr : c.trig_corr;
    p.ao = ao; p.sky = sky; p.sun = sun;
    p.err_word = c.dev_error;
    apply_tune(p, accel);
    return p;
}

int do_visibility(const StagedGbuf& g, int w, int h, const rn_accel* accel, int spp, float radius,
                  const float* to_light, int flags, float* ao, float* sky, float* sun, rn_status* st) {
    Context& c = ctx();
    const TraceParams p = vis_params(g, w, h, accel, spp, radius, to_light, flags, ao, sky, sun);
    if (launch_trace(p, c.sm_count, c.stream) != RN_OK) return cuda_fail(st, cudaGetLastError(), "trace_kernel");
    return RN_OK;
}

void fill_result(const RecOut& r, float tolerance, rn_reconcile_result* out);

// The device address of a pinned, mapped host buffer (nullptr for any other kind).
void* mapped(const void* p) {
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// rn_ao_frame with pinned, mapped host buffers and no copies. The traversal reads each
// pixel's G-buffer entry straight from host memory (25 bytes, once per pixel, against
// hundreds of rays), writes AO (sky, sun) straight into the caller's host images, and
// mirrors the G-buffer entry and the AO into HBM as it goes. The SSAO, whose taps re-read
// neighbours, and the fused reconcile then run on the mirror and write the SSAO image and the
// error map into host memory. No copy engine runs and nothing waits for one; every output is
// the device-buffer frame's bit for bit.
int direct_frame(const rn_gbuf* g, const rn_accel* accel, int spp, float radius, int ss_samples, float tolerance,
                 const float tl[3], int flags, float* h_ao, float* h_sky, float* h_sun, float* h_ss, float* h_err,
                 rn_reconcile_result* out, rn_status* st) {
    Context& c = ctx();
    const int w = g->w, h = g->h;
    const size_t np = (size_t)w * h;
    const bool want_sky = (flags & RN_SKY) != 0;
    const StagedGbuf hg{(const float*)mapped(g->position), (const float*)mapped(g->normal),
                        (const uint8_t*)mapped(g->mask)};
    void *vm, *parts, *ro;
    RN_TRY(ws_get(WS_MIRROR, np * 29, &vm, st));
    const int nb = ssao_blocks(w, h);
    RN_TRY(ws_get(WS_PARTIALS, (size_t)nb * sizeof(RecPartial), &parts, st));
    RN_TRY(ws_get(WS_COUNTERS, sizeof(RecOut), &ro, st));
    uint8_t* m = (uint8_t*)vm;
    TraceParams p = vis_params(hg, w, h, accel, spp, radius, tl, flags, (float*)mapped(h_ao),
                               want_sky ? (float*)mapped(h_sky) : nullptr, want_sky ? (float*)mapped(h_sun) : nullptr);
    p.mirror = m;
    if (launch_trace(p, c.sm_count, c.stream) != RN_OK) return cuda_fail(st, cudaGetLastError(), "trace_kernel");
    const uint8_t* corr = (flags & RN_DEVICE_TRIG) ? nullptr : c.trig_corr;
    if (launch_ssao(w, h, mirror_pos(m, np), mirror_nrm(m, np), mirror_mask(m, np), ss_samples, radius, corr,
                    (float*)mapped(h_ss), mirror_ao(m, np), h_err ? (float*)mapped(h_err) : nullptr,
                    (RecPartial*)parts, (RecOut*)ro, c.stream) != RN_OK)
        return cuda_fail(st, cudaGetLastError(), "ssao_kernel (fused reconcile)");
    RecOut r;
    RN_CUDA(cudaMemcpyAsync(&r, ro, sizeof r, cudaMemcpyDeviceToHost, c.stream), st);
    RN_TRY(check_device_error(st, "rn_ao_frame"));
    fill_result(r, tolerance, out);
    return ok(st);
}

int check_vis_args(const rn_gbuf* g, const rn_accel* accel, int spp, const float* to_light, int flags, const float* ao,
                   const float* sky, const float* sun, rn_status* st) {
    RN_TRY(check_gbuf(g, st));
    if (!accel) return fail(st, RN_ERR_INVALID, "null accelerator");
    if (spp <= 0) return fail(st, RN_ERR_INVALID, "samples per pixel %d <= 0", spp);
    if (!ao) return fail(st, RN_ERR_INVALID, "null ao output");
    if ((flags & RN_SKY) && (!sky || !sun || !to_light)) return fail(st, RN_ERR_INVALID, "RN_SKY needs sky, sun and to_light");
    if (accel->device != ctx().device) return fail(st, RN_ERR_STATE, "accelerator belongs to device %d", accel->device);
    return RN_OK;
}

// raw/math/mat.hpp:9-35 and raw/scene/scene.hpp:12-17 on the host: the view-projection
// matrix of a camera (eye, target, up, fovy; aspect = w / h; near 0.1, far 100), in the
// reference's float operation order (this file's host code builds with -ffp-contract=off).
struct M4 { float m[16]; };
M4 m4_mul(const M4& a, const M4& b) {
    M4 r{};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            float s = 0;
            for (int k = 0; k < 4; ++k) s += a.m[i * 4 + k] * b.m[k * 4 + j];
            r.m[i * 4 + j] = s;
        }
    return r;
}
void h_norm(const float v[3], float o[3]) {
    const float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (l > 0) { const float i = 1.0f / l; o[0] = v[0] * i; o[1] = v[1] * i; o[2] = v[2] * i; }
    else { o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; }
}
void h_cross(const float a[3], const float b[3], float o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
float h_dot(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
M4 view_matrix(const float* cam) {
    const float eye[3] = {cam[0], cam[1], cam[2]}, ctr[3] = {cam[3], cam[4], cam[5]}, up[3] = {cam[6], cam[7], cam[8]};
    const float d[3] = {ctr[0] - eye[0], ctr[1] - eye[1], ctr[2] - eye[2]};
    float f[3], s0[3], sv[3], u[3];
    h_norm(d, f);
    h_cross(f, up, s0);
    h_norm(s0, sv);
    h_cross(sv, f, u);
    M4 view{};
    view.m[0] = view.m[5] = view.m[10] = view.m[15] = 1;
    view.m[0] = sv[0]; view.m[1] = sv[1]; view.m[2] = sv[2]; view.m[3] = -h_dot(sv, eye);
    view.m[4] = u[0]; view.m[5] = u[1]; view.m[6] = u[2]; view.m[7] = -h_dot(u, eye);
    view.m[8] = -f[0]; view.m[9] = -f[1]; view.m[10] = -f[2]; view.m[11] = h_dot(f, eye);
    return view;
}
M4 view_proj(const float* cam, int w, int h, float nearZ, float farZ) {
    const M4 view = view_matrix(cam);
    const float aspect = h > 0 ? (float)w / (float)h : 1.0f;
    const float t = 1.0f / ::tanf(cam[9] * 0.5f);
    M4 proj{};
    proj.m[0] = t / aspect; proj.m[5] = t;
    proj.m[10] = (farZ + nearZ) / (nearZ - farZ); proj.m[11] = (2 * farZ * nearZ) / (nearZ - farZ);
    proj.m[14] = -1;
    return m4_mul(proj, view);
}

void fill_result(const RecOut& r, float tolerance, rn_reconcile_result* out) {
    out->sum_sq = r.sum;
    out->pixels = r.n;
    out->max_error = r.max;
    out->rmse = r.n > 0 ? (float)std::sqrt(r.sum / (double)r.n) : 0.0f;
    out->within_tolerance = out->rmse <= tolerance ? 1 : 0;
}

}  // namespace

extern "C" {

int rn_ao_version(void) { return RN_AO_ABI_VERSION; }

int rn_tune_set(const char* key, int value, rn_status* st) {
    if (!key) return fail(st, RN_ERR_INVALID, "null key");
    tune_env_once();
    RN_TRY(tune_assign(key, value, st));
    return ok(st);
}

int rn_tune_get(const char* key, int* value, rn_status* st) {
    if (!key || !value) return fail(st, RN_ERR_INVALID, "null argument");
    tune_env_once();
    const TuneKey* k = find_tune_key(key);
    if (!k) return fail(st, RN_ERR_INVALID, "unknown tuning key '%s'", key);
    *value = ctx().tune.*(k->field);
    return ok(st);
}

// "key = value" lines; '#' starts a comment. Every line is checked before any is applied; a
// key whose RN_TUNE_<KEY> environment variable is set keeps the variable's value.
int rn_tune_load(const char* path, rn_status* st) {
    if (!path) return fail(st, RN_ERR_INVALID, "null path");
    tune_env_once();
    FILE* f = std::fopen(path, "r");
    if (!f) return fail(st, RN_ERR_INVALID, "cannot open %s", path);
    std::vector<std::pair<std::string, int>> kv;
    char line[256];
    int lineno = 0, rc = RN_OK;
    while (rc == RN_OK && std::fgets(line, sizeof line, f)) {
        ++lineno;
        if (char* h = std::strchr(line, '#')) *h = 0;
        char key[64];
        int value = 0;
        char extra[8];
        const int n = std::sscanf(line, " %63[a-z0-9_] = %d %7s", key, &value, extra);
        if (n == EOF || (n <= 0 && std::strspn(line, " \t\r\n") == std::strlen(line))) continue;
        if (n != 2) { rc = fail(st, RN_ERR_INVALID, "%s:%d: expected 'key = value'", path, lineno); break; }
        const TuneKey* k = find_tune_key(key);
        if (!k) { rc = fail(st, RN_ERR_INVALID, "%s:%d: unknown tuning key '%s'", path, lineno, key); break; }
        kv.emplace_back(key, value);
    }
    std::fclose(f);
    if (rc != RN_OK) return rc;
    const Tune saved = ctx().tune;
    for (auto& e : kv)
        if (!getenv(find_tune_key(e.first.c_str())->env) && tune_assign(e.first.c_str(), e.second, st) != RN_OK) {
            ctx().tune = saved;
            return st ? st->code : RN_ERR_INVALID;
        }
    return ok(st);
}

int rn_init(rn_status* st) {
    RN_TRY(ensure_ctx(st));
    return ok(st);
}

int rn_set_stream(void* stream, rn_status* st) {
    RN_TRY(ensure_ctx(st));
    Context& c = ctx();
    c.stream = stream ? (cudaStream_t)stream : c.own_stream;
    return ok(st);
}

int rn_synchronize(rn_status* st) {
    RN_TRY(ensure_ctx(st));
    RN_CUDA(cudaStreamSynchronize(ctx().stream), st);
    RN_TRY(check_device_error(st, "rn_synchronize"));
    return ok(st);
}

int rn_device_info(rn_device_desc* out, rn_status* st) {
    if (!out) return fail(st, RN_ERR_INVALID, "null output");
    RN_TRY(ensure_ctx(st));
    cudaDeviceProp p;
    RN_CUDA(cudaGetDeviceProperties(&p, ctx().device), st);
    std::memset(out, 0, sizeof *out);
    std::snprintf(out->name, sizeof out->name, "%s", p.name);
    out->cc_major = p.major;
    out->cc_minor = p.minor;
    out->sm_count = p.multiProcessorCount;
    out->total_bytes = (uint64_t)p.totalGlobalMem;
    RN_CUDA(cudaDriverGetVersion(&out->driver_version), st);
    RN_CUDA(cudaRuntimeGetVersion(&out->runtime_version), st);
    return ok(st);
}

int rn_accel_build(const float* tris, uint32_t ntri, int flags, rn_accel** out, rn_status* st) {
    if (!out) return fail(st, RN_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (ntri > 0 && !tris) return fail(st, RN_ERR_INVALID, "null triangles");
    if (ntri >= (1u << 28)) return fail(st, RN_ERR_INVALID, "%u triangles: at most 2^28 - 1", ntri);
    RN_TRY(ensure_ctx(st));
    Context& c = ctx();
    const bool dev = (flags & RN_DEVICE_PTRS) != 0;
    const float* d_tris = nullptr;
    RN_TRY(stage_in(tris, (size_t)ntri * 9, dev, WS_TRIS_IN, &d_tris, st));
    rn_accel* acc = new rn_accel();
    acc->device = c.device;
    PlocTree tree;
    // the tree only prunes (every hit is the triangle test's): its shape is a tuning choice
    int rc = ploc_build(d_tris, ntri, c.tune.accel_radius, &tree, c.stream, st);
    if (rc == RN_OK)
        rc = collapse_bvh4(tree, d_tris, acc, ntri < kSmallScene ? c.tune.accel_leaf_small : c.tune.accel_leaf,
                           c.stream, st);
    if (rc == RN_OK) {
        cudaError_t e = cudaStreamSynchronize(c.stream);
        if (e != cudaSuccess) rc = cuda_fail(st, e, "rn_accel_build");
    }
    ploc_free(&tree);
    if (rc == RN_OK && acc->depth * 3 + 2 > 96)
        rc = fail(st, RN_ERR_OVERFLOW, "BVH depth %u needs more than the traversal's 96-entry stack", acc->depth);
    if (rc != RN_OK) { rn_accel_free(acc); return rc; }
    *out = acc;
    return ok(st);
}

void rn_accel_free(rn_accel* accel) {
    if (!accel) return;
    if (accel->d_nodes) {
        // d_tris lies in the same block. Any stream may still be reading it: wait for the
        // device (as cudaFree would), then hand the block back to the library's pool.
        cudaDeviceSynchronize();
        cudaFreeAsync(accel->d_nodes, ctx().stream);
    }
    delete accel;
}

int rn_accel_info(const rn_accel* accel, uint32_t* wide_nodes, uint32_t* leaf_tris, uint32_t* ploc_rounds, rn_status* st) {
    if (!accel) return fail(st, RN_ERR_INVALID, "null accelerator");
    if (wide_nodes) *wide_nodes = accel->nodes;
    if (leaf_tris) *leaf_tris = accel->ntri;
    if (ploc_rounds) *ploc_rounds = accel->rounds;
    return ok(st);
}

int rn_ao_visibility(const rn_gbuf* g, const rn_accel* accel, int spp, float radius, const float* to_light, int flags,
                     float* ao, float* sky, float* sun, rn_status* st) {
    RN_TRY(ensure_ctx(st));
    RN_TRY(check_vis_args(g, accel, spp, to_light, flags, ao, sky, sun, st));
    const bool dev = (flags & RN_DEVICE_PTRS) != 0;
    const size_t np = (size_t)g->w * g->h;
    StagedGbuf sg;
    RN_TRY(stage_gbuf(g, dev, &sg, st));
    float *d_ao, *d_sky = nullptr, *d_sun = nullptr;
    float tl[3] = {0.0f, 1.0f, 0.0f};
    if (flags & RN_SKY) { tl[0] = to_light[0]; tl[1] = to_light[1]; tl[2] = to_light[2]; }
    RN_TRY(stage_out(ao, np, dev, WS_AO, &d_ao, st));
    if (flags & RN_SKY) {
        RN_TRY(stage_out(sky, np, dev, WS_SKY, &d_sky, st));
        RN_TRY(stage_out(sun, np, dev, WS_SUN, &d_sun, st));
    }
    RN_TRY(do_visibility(sg, g->w, g->h, accel, spp, radius, tl, flags, d_ao, d_sky, d_sun, st));
    if (dev) return ok(st);
    RN_TRY(copy_back(ao, d_ao, np, st));
    if (flags & RN_SKY) { RN_TRY(copy_back(sky, d_sky, np, st)); RN_TRY(copy_back(sun, d_sun, np, st)); }
    RN_TRY(check_device_error(st, "rn_ao_visibility"));
    return ok(st);
}

int rn_ssao(const rn_gbuf* g, int samples, float radius, int flags, float* ao_ss, rn_status* st) {
    RN_TRY(ensure_ctx(st));
    RN_TRY(check_gbuf(g, st));
    if (!ao_ss) return fail(st, RN_ERR_INVALID, "null output");
    if (samples < 0) return fail(st, RN_ERR_INVALID, "samples %d < 0", samples);
    Context& c = ctx();
    const bool dev = (flags & RN_DEVICE_PTRS) != 0;
    const size_t np = (size_t)g->w * g->h;
    StagedGbuf sg;
    RN_TRY(stage_gbuf(g, dev, &sg, st));
    float* d_ss;
    RN_TRY(stage_out(ao_ss, np, dev, WS_SS, &d_ss, st));
    const uint8_t* corr = (flags & RN_DEVICE_TRIG) ? nullptr : c.trig_corr;
    if (launch_ssao(g->w, g->h, sg.pos, sg.nrm, sg.mask, samples, radius, corr, d_ss, nullptr, nullptr, nullptr,
                    nullptr, c.stream) != RN_OK)
        return cuda_fail(st, cudaGetLastError(), "ssao_kernel");
    if (dev) return ok(st);
    RN_TRY(copy_back(ao_ss, d_ss, np, st));
    RN_CUDA(cudaStreamSynchronize(c.stream), st);
    return ok(st);
}

int rn_gtao(const rn_gbuf* g, const float* camera, float radius, int slices, int steps, int flags, float* ao,
            rn_status* st) {
    RN_TRY(ensure_ctx(st));
    RN_TRY(check_gbuf(g, st));
    if (!ao || !camera) return fail(st, RN_ERR_INVALID, "null argument");
    if (!(radius > 0.0f) || slices <= 0 || steps <= 0 || slices > 1024 || steps > 1024)
        return fail(st, RN_ERR_INVALID, "radius %g slices %d steps %d", radius, slices, steps);
    Context& c = ctx();
    const bool dev = (flags & RN_DEVICE_PTRS) != 0;
    const size_t np = (size_t)g->w * g->h;
    StagedGbuf sg;
    RN_TRY(stage_gbuf(g, dev, &sg, st));
    void *vp, *vn, *vd;
    RN_TRY(ws_get(WS_VPOS, np * 12, &vp, st));
    RN_TRY(ws_get(WS_VNRM, np * 12, &vn, st));
    RN_TRY(ws_get(WS_VDEPTH, np * 4, &vd, st));
    float* d_ao;
    RN_TRY(stage_out(ao, np, dev, WS_GTAO, &d_ao, st));
    const M4 view = view_matrix(camera);
    if (launch_gtao(g->w, g->h, sg.pos, sg.nrm, sg.mask, view.m, camera[9], radius, slices, steps, (float*)vp,
                    (float*)vn, (float*)vd, d_ao, c.stream) != RN_OK)
        return cuda_fail(st, cudaGetLastError(), "gtao_kernel");
    if (dev) return ok(st);
    RN_TRY(copy_back(ao, d_ao, np, st));
    RN_CUDA(cudaStreamSynchronize(c.stream), st);
    return ok(st);
}

int rn_reconcile(const float* approx, const float* truth, const uint8_t* mask, int w, int h, float tolerance, int flags,
                 float* err, rn_reconcile_result* out, rn_status* st) {
    if (!approx || !truth || !mask || !out) return fail(st, RN_ERR_INVALID, "null argument");
    if (w < 0 || h < 0) return fail(st, RN_ERR_INVALID, "size %dx%d", w, h);
    RN_TRY(ensure_ctx(st));
    Context& c = ctx();
    const bool dev = (flags & RN_DEVICE_PTRS) != 0;
    const size_t np = (size_t)w * h;
    if (np == 0) {
        *out = rn_reconcile_result{0.0f, 0.0f, 0, 1, 0.0};
        out->within_tolerance = 0.0f <= tolerance;
        return ok(st);
    }
    const float *d_a, *d_t;
    const uint8_t* d_m;
    float* d_e = nullptr;
    RN_TRY(stage_in(approx, np, dev, WS_APPROX, &d_a, st));
    RN_TRY(stage_in(truth, np, dev, WS_TRUTH, &d_t, st));
    RN_TRY(stage_in(mask, np, dev, WS_MASK, &d_m, st));
    if (err) RN_TRY(stage_out(err, np, dev, WS_ERR, &d_e, st));
    const int nb = reconcile_blocks(np);
    void *parts = nullptr, *ro = nullptr;
    RN_TRY(ws_get(WS_PARTIALS, (size_t)nb * sizeof(RecPartial), &parts, st));
    RN_TRY(ws_get(WS_COUNTERS, sizeof(RecOut), &ro, st));
    const cudaError_t le = launch_reconcile(d_a, d_t, d_m, np, d_e, (RecPartial*)parts, nb, (RecOut*)ro, c.stream);
    if (le != cudaSuccess) return cuda_fail(st, le, "reconcile_kernel");
    RecOut r;
    RN_CUDA(cudaMemcpyAsync(&r, ro, sizeof r, cudaMemcpyDeviceToHost, c.stream), st);
    if (!dev) RN_TRY(copy_back(err, d_e, np, st));
    RN_CUDA(cudaStreamSynchronize(c.stream), st);
    fill_result(r, tolerance, out);
    return ok(st);
}

int rn_ao_frame(const rn_gbuf* g, const rn_accel* accel, int spp, float radius, int ss_samples, float tolerance,
                const float* to_light, int flags, float* ao, float* sky, float* sun, float* ao_ss, float* err,
                rn_reconcile_result* out, rn_status* st) {
    RN_TRY(ensure_ctx(st));
    RN_TRY(check_vis_args(g, accel, spp, to_light, flags, ao, sky, sun, st));
    if (!ao_ss || !out) return fail(st, RN_ERR_INVALID, "null ao_ss or result");
    if (ss_samples < 0) return fail(st, RN_ERR_INVALID, "ss_samples %d < 0", ss_samples);
    Context& c = ctx();
    const bool dev = (flags & RN_DEVICE_PTRS) != 0;
    const size_t np = (size_t)g->w * g->h;
    float tl[3] = {0.0f, 1.0f, 0.0f};
    if (flags & RN_SKY) { tl[0] = to_light[0]; tl[1] = to_light[1]; tl[2] = to_light[2]; }
    // host frames of 256k pixels and more, every buffer pinned and mapped: no copies
    if (!dev && c.tune.frame_direct && np >= ((size_t)1 << 18) && mapped(g->position) && mapped(g->normal) &&
        mapped(g->mask) && mapped(ao) && mapped(ao_ss) && (!err || mapped(err)) &&
        (!(flags & RN_SKY) || (mapped(sky) && mapped(sun))))
        return direct_frame(g, accel, spp, radius, ss_samples, tolerance, tl, flags, ao, sky, sun, ao_ss, err, out, st);
    StagedGbuf sg;
    RN_TRY(stage_gbuf(g, dev, &sg, st));
    float *d_ao, *d_sky = nullptr, *d_sun = nullptr, *d_ss, *d_err = nullptr;
    RN_TRY(stage_out(ao, np, dev, WS_AO, &d_ao, st));
    if (flags & RN_SKY) {
        RN_TRY(stage_out(sky, np, dev, WS_SKY, &d_sky, st));
        RN_TRY(stage_out(sun, np, dev, WS_SUN, &d_sun, st));
    }
    RN_TRY(stage_out(ao_ss, np, dev, WS_SS, &d_ss, st));
    if (err) RN_TRY(stage_out(err, np, dev, WS_ERR, &d_err, st));
    RN_TRY(do_visibility(sg, g->w, g->h, accel, spp, radius, tl, flags, d_ao, d_sky, d_sun, st));
    const int nb = ssao_blocks(g->w, g->h);
    void *parts = nullptr, *ro = nullptr;
    RN_TRY(ws_get(WS_PARTIALS, (size_t)nb * sizeof(RecPartial), &parts, st));
    RN_TRY(ws_get(WS_COUNTERS, sizeof(RecOut), &ro, st));
    const uint8_t* corr = (flags & RN_DEVICE_TRIG) ? nullptr : c.trig_corr;
    if (launch_ssao(g->w, g->h, sg.pos, sg.nrm, sg.mask, ss_samples, radius, corr, d_ss, d_ao, d_err,
                    (RecPartial*)parts, (RecOut*)ro, c.stream) != RN_OK)
        return cuda_fail(st, cudaGetLastError(), "ssao_kernel (fused reconcile)");
    RecOut r;
    RN_CUDA(cudaMemcpyAsync(&r, ro, sizeof r, cudaMemcpyDeviceToHost, c.stream), st);
    if (!dev) {
        RN_TRY(copy_back(ao, d_ao, np, st));
        if (flags & RN_SKY) { RN_TRY(copy_back(sky, d_sky, np, st)); RN_TRY(copy_back(sun, d_sun, np, st)); }
        RN_TRY(copy_back(ao_ss, d_ss, np, st));
        if (err) RN_TRY(copy_back(err, d_err, np, st));
    }
    RN_TRY(check_device_error(st, "rn_ao_frame"));
    fill_result(r, tolerance, out);
    return ok(st);
}


// raw::renderWithParams (src/renderer/render.cpp:99-137) on the GPU: the G-buffer with its
// albedo plane, the ray-traced AO (lighting model 2: with sky and sun), SSAO and the
// reconcile, the shaded frame and its HDR view, the motion plane. Every plane is the CPU
// path's bit for bit.
int rn_render_frame(const rn_frame_scene* sc, const float* camera, const float* prev_view_proj, int w, int h,
                    const rn_frame_options* opt, int flags, rn_frame_out* out, rn_status* st) {
    if (!sc || !camera || !out) return fail(st, RN_ERR_INVALID, "null argument");
    if (sc->ntri > 0 && (!sc->tris || !sc->normals || !sc->albedo)) return fail(st, RN_ERR_INVALID, "null scene arrays");
    if (w <= 0 || h <= 0 || (size_t)w * (size_t)h > ((size_t)1 << 31)) return fail(st, RN_ERR_INVALID, "size %dx%d", w, h);
    if (sc->ntri >= (1u << 28)) return fail(st, RN_ERR_INVALID, "%u triangles: too many", sc->ntri);
    rn_frame_options o{0.12f, 1, 2, 64, 2.0f, 24};
    if (opt) o = *opt;
    if (o.spp <= 0 || o.ss_samples < 0 || !(o.radius > 0.0f)) return fail(st, RN_ERR_INVALID, "spp %d ss %d radius %g", o.spp, o.ss_samples, o.radius);
    RN_TRY(ensure_ctx(st));
    Context& c = ctx();
    const bool dev = (flags & RN_DEVICE_PTRS) != 0;
    const size_t np = (size_t)w * h;
    const int model = !o.rtao ? 1 : (o.lighting == 1 ? 1 : 2);
    // scene in
    const float *d_tris = nullptr, *d_nin = nullptr, *d_alb_in = nullptr;
    RN_TRY(stage_in(sc->tris, (size_t)sc->ntri * 9, dev, WS_TRIS_IN, &d_tris, st));
    RN_TRY(stage_in(sc->normals, (size_t)sc->ntri * 9, dev, WS_NRM_IN, &d_nin, st));
    RN_TRY(stage_in(sc->albedo, (size_t)sc->ntri * 3, dev, WS_ALB_IN, &d_alb_in, st));
    // G-buffer
    float *d_depth, *d_pos, *d_nrm, *d_alb, *d_mot, *d_ao = nullptr, *d_sky = nullptr, *d_sun = nullptr, *d_ss, *d_err;
    float *d_frame, *d_hdr;
    uint8_t* d_mask;
    RN_TRY(frame_buf(out->depth, np, dev, WS_DEPTH, &d_depth, st));
    RN_TRY(frame_buf(out->position, np * 3, dev, WS_POS, &d_pos, st));
    RN_TRY(frame_buf(out->normal, np * 3, dev, WS_NRM, &d_nrm, st));
    RN_TRY(frame_buf(out->albedo, np * 3, dev, WS_ALB, &d_alb, st));
    RN_TRY(frame_buf(out->mask, np, dev, WS_MASK, &d_mask, st));
    RN_TRY(frame_buf(out->motion, np * 2, dev, WS_MOTION, &d_mot, st));
    RN_TRY(frame_buf(out->ao_ss, np, dev, WS_SS, &d_ss, st));
    RN_TRY(frame_buf(out->error_map, np, dev, WS_ERR, &d_err, st));
    RN_TRY(frame_buf(out->frame, np * 3, dev, WS_FRAME, &d_frame, st));
    RN_TRY(frame_buf(out->hdr, np * 3, dev, WS_HDR, &d_hdr, st));
    if (o.rtao) {
        RN_TRY(frame_buf(out->ao_rt, np, dev, WS_AO, &d_ao, st));
        if (model == 2) {
            RN_TRY(frame_buf(out->sky, np, dev, WS_SKY, &d_sky, st));
            RN_TRY(frame_buf(out->sun, np, dev, WS_SUN, &d_sun, st));
        }
    }
    const M4 vp = view_proj(camera, w, h, 0.1f, 100.0f);
    void* small = nullptr;
    RN_TRY(ws_get(WS_FRAME_SMALL, 256, &small, st));
    float* d_vp = (float*)small;
    unsigned* d_valid = (unsigned*)((char*)small + 128);
    RN_CUDA(cudaMemcpyAsync(d_vp, vp.m, 64, cudaMemcpyHostToDevice, c.stream), st);
    RN_CUDA(cudaMemsetAsync(d_valid, 0, 8, c.stream), st);
    size_t pairs = (size_t)8 * sc->ntri + 1024;
    for (int attempt = 0; attempt < 2; ++attempt) {
        const size_t bytes = raster_scratch_bytes(sc->ntri, np, pairs);
        void* scratch = nullptr;
        RN_TRY(ws_get(WS_RASTER, bytes, &scratch, st));
        size_t needed = 0;
        const int rc = launch_raster(d_tris, d_nin, sc->ntri, d_vp, 0.1f, w, h, (char*)scratch, ctx().ws[WS_RASTER].cap,
                                     d_depth, d_pos, d_nrm, d_mask, c.stream, &needed, d_alb_in, d_alb);
        if (rc == RN_OK) break;
        if (rc == RN_ERR_NO_MEMORY && attempt == 0) { pairs = needed + needed / 8 + 1024; continue; }
        return rc == RN_ERR_NO_MEMORY ? fail(st, rc, "raster: %zu bin pairs", needed)
                                      : cuda_fail(st, cudaGetLastError(), "raster kernels");
    }
    const float ldir[3] = {sc->has_light ? sc->light_dir[0] : 0.0f, sc->has_light ? sc->light_dir[1] : -1.0f,
                           sc->has_light ? sc->light_dir[2] : 0.0f};
    const float li = sc->has_light ? sc->light_intensity : 1.0f;
    StagedGbuf sg{d_pos, d_nrm, d_mask};
    rn_accel* acc = nullptr;
    RecOut r{};
    if (o.rtao) {
        // the accelerator is built per frame from the scene's triangles, as the rtao pass does
        RN_TRY(rn_accel_build(d_tris, sc->ntri, RN_DEVICE_PTRS, &acc, st));
        const float tl[3] = {-ldir[0], -ldir[1], -ldir[2]};
        int rc = do_visibility(sg, w, h, acc, o.spp, o.radius, tl, model == 2 ? RN_SKY : 0, d_ao, d_sky, d_sun, st);
        if (rc == RN_OK) {
            const int nb = ssao_blocks(w, h);
            void *parts = nullptr, *ro = nullptr;
            rc = ws_get(WS_PARTIALS, (size_t)nb * sizeof(RecPartial), &parts, st);
            if (rc == RN_OK) rc = ws_get(WS_COUNTERS, sizeof(RecOut), &ro, st);
            if (rc == RN_OK && launch_ssao(w, h, d_pos, d_nrm, d_mask, o.ss_samples, o.radius, c.trig_corr, d_ss, d_ao,
                                           d_err, (RecPartial*)parts, (RecOut*)ro, c.stream) != RN_OK)
                rc = cuda_fail(st, cudaGetLastError(), "ssao_kernel (fused reconcile)");
            if (rc == RN_OK && cudaMemcpyAsync(&r, ro, sizeof r, cudaMemcpyDeviceToHost, c.stream) != cudaSuccess)
                rc = cuda_fail(st, cudaGetLastError(), "reconcile read-back");
        }
        if (rc != RN_OK) { cudaStreamSynchronize(c.stream); rn_accel_free(acc); return rc; }
    } else {
        if (launch_ssao(w, h, d_pos, d_nrm, d_mask, o.ss_samples, o.radius, c.trig_corr, d_ss, nullptr, nullptr,
                        nullptr, nullptr, c.stream) != RN_OK)
            return cuda_fail(st, cudaGetLastError(), "ssao_kernel");
        RN_CUDA(cudaMemsetAsync(d_err, 0, np * 4, c.stream), st);   // no reference: an empty reconcile
    }
    const float* light_ao = model == 2 ? d_sky : (o.rtao ? d_ao : d_ss);
    int rc = launch_shade(w, h, d_nrm, d_alb, d_mask, model, light_ao, d_sun, ldir, li, d_frame, d_hdr, c.stream);
    if (rc == RN_OK)
        rc = launch_motion(w, h, d_pos, d_mask, vp.m, prev_view_proj ? prev_view_proj : vp.m, d_mot, d_valid, c.stream);
    unsigned counts[2] = {0, 0};
    if (rc == RN_OK && cudaMemcpyAsync(counts, d_valid, 8, cudaMemcpyDeviceToHost, c.stream) != cudaSuccess)
        rc = cuda_fail(st, cudaGetLastError(), "motion counts");
    if (rc == RN_OK && !dev) {
        const struct { void* h; const void* d; size_t bytes; } outs[] = {
            {out->depth, d_depth, np * 4}, {out->position, d_pos, np * 12}, {out->normal, d_nrm, np * 12},
            {out->albedo, d_alb, np * 12}, {out->mask, d_mask, np}, {out->motion, d_mot, np * 8},
            {out->ao_rt, d_ao, np * 4}, {o.rtao && model == 2 ? out->sky : nullptr, d_sky, np * 4},
            {o.rtao && model == 2 ? out->sun : nullptr, d_sun, np * 4},
            {out->ao_ss, d_ss, np * 4}, {out->error_map, d_err, np * 4}, {out->frame, d_frame, np * 12},
            {out->hdr, d_hdr, np * 12}};
        for (const auto& x : outs)
            if (rc == RN_OK && x.h && x.d && cudaMemcpyAsync(x.h, x.d, x.bytes, cudaMemcpyDeviceToHost, c.stream) != cudaSuccess)
                rc = cuda_fail(st, cudaGetLastError(), "frame read-back");
    }
    const cudaError_t e = cudaStreamSynchronize(c.stream);
    if (acc) rn_accel_free(acc);
    if (rc != RN_OK) return rc;
    if (e != cudaSuccess) return cuda_fail(st, e, "rn_render_frame");
    RN_TRY(check_device_error(st, "rn_render_frame"));
    if (o.rtao) fill_result(r, o.tolerance, &out->rec);
    else out->rec = rn_reconcile_result{0.0f, 0.0f, 0, 0, 0.0};
    out->motion_valid = (int)counts[0];
    out->motion_total = (int)counts[1];
    for (int k = 0; k < 16; ++k) out->view_proj[k] = vp.m[k];
    return ok(st);
}

int rn_ploc_build(const float* tris, uint32_t ntri, int radius, int flags, int32_t* nodes_out, int32_t* root,
                  uint32_t* rounds, rn_status* st) {
    if ((ntri > 0 && (!tris || !nodes_out)) || !root || !rounds) return fail(st, RN_ERR_INVALID, "null argument");
    if (ntri >= (1u << 30)) return fail(st, RN_ERR_INVALID, "%u triangles: too many", ntri);
    RN_TRY(ensure_ctx(st));
    Context& c = ctx();
    const bool dev = (flags & RN_DEVICE_PTRS) != 0;
    *root = -1;
    *rounds = 0;
    if (ntri == 0) return ok(st);
    const float* d_tris = nullptr;
    RN_TRY(stage_in(tris, (size_t)ntri * 9, dev, WS_TRIS_IN, &d_tris, st));
    PlocTree tree;
    int rc = ploc_build(d_tris, ntri, radius, &tree, c.stream, st);
    const size_t count = 2 * (size_t)ntri - 1;
    int32_t* d_out = nodes_out;
    if (rc == RN_OK && !dev) {
        void* p = nullptr;
        rc = ws_get(WS_HITS, count * 9 * 4, &p, st);
        d_out = (int32_t*)p;
    }
    if (rc == RN_OK) rc = ploc_export(tree, d_out, c.stream, st);
    if (rc == RN_OK && !dev) rc = copy_back(nodes_out, d_out, count * 9, st);
    if (rc == RN_OK) {
        cudaError_t e = cudaStreamSynchronize(c.stream);
        if (e != cudaSuccess) rc = cuda_fail(st, e, "rn_ploc_build");
    }
    *root = tree.root;
    *rounds = tree.rounds;
    ploc_free(&tree);
    return rc == RN_OK ? ok(st) : rc;
}

int rn_raster_gbuffer(const float* tris, const float* nrm, uint32_t ntri, const float* cam, int w, int h, int flags,
                      float* depth, float* position, float* normal, uint8_t* mask, rn_status* st) {
    if ((ntri > 0 && (!tris || !nrm)) || !cam || !position || !normal || !mask)
        return fail(st, RN_ERR_INVALID, "null argument");
    if (w <= 0 || h <= 0 || (size_t)w * (size_t)h > ((size_t)1 << 31)) return fail(st, RN_ERR_INVALID, "size %dx%d", w, h);
    if (ntri >= (1u << 28)) return fail(st, RN_ERR_INVALID, "%u triangles: too many", ntri);
    RN_TRY(ensure_ctx(st));
    Context& c = ctx();
    const bool dev = (flags & RN_DEVICE_PTRS) != 0;
    const size_t np = (size_t)w * h;
    const float *d_tris = nullptr, *d_nin = nullptr;
    RN_TRY(stage_in(tris, (size_t)ntri * 9, dev, WS_TRIS_IN, &d_tris, st));
    RN_TRY(stage_in(nrm, (size_t)ntri * 9, dev, WS_NRM_IN, &d_nin, st));
    float *d_depth = nullptr, *d_pos, *d_nrm;
    uint8_t* d_mask;
    if (depth) RN_TRY(stage_out(depth, np, dev, WS_DEPTH, &d_depth, st));
    RN_TRY(stage_out(position, np * 3, dev, WS_POS, &d_pos, st));
    RN_TRY(stage_out(normal, np * 3, dev, WS_NRM, &d_nrm, st));
    RN_TRY(stage_out(mask, np, dev, WS_MASK, &d_mask, st));
    const float nearZ = 0.1f, farZ = 100.0f;
    const M4 vp = view_proj(cam, w, h, nearZ, farZ);
    void* vpbuf = nullptr;
    RN_TRY(ws_get(WS_STATS, 256, &vpbuf, st));
    RN_CUDA(cudaMemcpyAsync(vpbuf, vp.m, sizeof vp.m, cudaMemcpyHostToDevice, c.stream), st);
    // first guess: four bins per triangle record; grown once if the scene needs more
    size_t pairs = (size_t)8 * ntri + 1024;
    for (int attempt = 0; attempt < 2; ++attempt) {
        const size_t bytes = raster_scratch_bytes(ntri, np, pairs);
        void* scratch = nullptr;
        RN_TRY(ws_get(WS_RASTER, bytes, &scratch, st));
        size_t needed = 0;
        const int rc = launch_raster(d_tris, d_nin, ntri, (const float*)vpbuf, nearZ, w, h, (char*)scratch,
                                     ctx().ws[WS_RASTER].cap, d_depth, d_pos, d_nrm, d_mask, c.stream, &needed);
        if (rc == RN_OK) break;
        if (rc == RN_ERR_NO_MEMORY && attempt == 0) { pairs = needed + needed / 8 + 1024; continue; }
        return rc == RN_ERR_NO_MEMORY ? fail(st, rc, "raster: %zu bin pairs", needed)
                                      : cuda_fail(st, cudaGetLastError(), "raster kernels");
    }
    if (dev) return ok(st);
    if (depth) RN_TRY(copy_back(depth, d_depth, np, st));
    RN_TRY(copy_back(position, d_pos, np * 3, st));
    RN_TRY(copy_back(normal, d_nrm, np * 3, st));
    RN_TRY(copy_back(mask, d_mask, np, st));
    RN_CUDA(cudaStreamSynchronize(c.stream), st);
    return ok(st);
}

int rn_ao_trace_stats(const rn_gbuf* g, const rn_accel* accel, int spp, float radius, const float* to_light, int flags,
                      uint32_t tile_stride, uint64_t* counts, rn_status* st) {
    RN_TRY(ensure_ctx(st));
    void* scratch[3];
    if (!counts) return fail(st, RN_ERR_INVALID, "null counts");
    const size_t np = g ? (size_t)g->w * g->h : 0;
    RN_TRY(ws_get(WS_AO, np * 4, &scratch[0], st));
    RN_TRY(check_vis_args(g, accel, spp, to_light, flags, (float*)scratch[0], (float*)scratch[0], (float*)scratch[0], st));
    Context& c = ctx();
    const bool dev = (flags & RN_DEVICE_PTRS) != 0;
    StagedGbuf sg;
    RN_TRY(stage_gbuf(g, dev, &sg, st));
    RN_TRY(ws_get(WS_SKY, np * 4, &scratch[1], st));
    RN_TRY(ws_get(WS_SUN, np * 4, &scratch[2], st));
    void* cnt = nullptr;
    RN_TRY(ws_get(WS_STATS, 4 * sizeof(unsigned long long), &cnt, st));
    RN_CUDA(cudaMemsetAsync(cnt, 0, 4 * sizeof(unsigned long long), c.stream), st);
    TraceParams p{};
    p.w = g->w; p.h = g->h;
    p.pos = sg.pos; p.nrm = sg.nrm; p.mask = sg.mask;
    p.nodes = accel->d_nodes; p.tris = accel->d_tris;
    p.has_geometry = accel->ntri > 0;
    p.spp = spp; p.radius = radius;
    p.want_sky = (flags & RN_SKY) != 0;
    p.sun_forced = (flags & RN_SUN_FORCED) != 0;
    if (p.want_sky) { p.lx = to_light[0]; p.ly = to_light[1]; p.lz = to_light[2]; } else { p.lx = 0; p.ly = 1; p.lz = 0; }
    p.corr = (flags & RN_DEVICE_TRIG) ? nullptr : c.trig_corr;
    p.ao = (float*)scratch[0]; p.sky = (float*)scratch[1]; p.sun = (float*)scratch[2];
    p.err_word = c.dev_error;
    apply_tune(p, accel);
    if (launch_trace(p, c.sm_count, c.stream, (unsigned long long*)cnt, tile_stride) != RN_OK)
        return cuda_fail(st, cudaGetLastError(), "trace_kernel (counting)");
    unsigned long long h[4];
    RN_CUDA(cudaMemcpyAsync(h, cnt, sizeof h, cudaMemcpyDeviceToHost, c.stream), st);
    RN_TRY(check_device_error(st, "rn_ao_trace_stats"));
    for (int k = 0; k < 4; ++k) counts[k] = h[k];
    return ok(st);
}

int rn_occluded(const rn_accel* accel, const float* rays, const float* t_max, uint32_t nrays, int flags, uint8_t* hit,
                rn_status* st) {
    if (!accel || (nrays > 0 && (!rays || !t_max || !hit))) return fail(st, RN_ERR_INVALID, "null argument");
    RN_TRY(ensure_ctx(st));
    Context& c = ctx();
    if (accel->device != c.device) return fail(st, RN_ERR_STATE, "accelerator belongs to device %d", accel->device);
    if (nrays == 0) return ok(st);
    const bool dev = (flags & RN_DEVICE_PTRS) != 0;
    const float *d_rays, *d_t;
    uint8_t* d_hit;
    RN_TRY(stage_in(rays, (size_t)nrays * 6, dev, WS_RAYS, &d_rays, st));
    RN_TRY(stage_in(t_max, (size_t)nrays, dev, WS_TMAX, &d_t, st));
    RN_TRY(stage_out(hit, (size_t)nrays, dev, WS_HITS, &d_hit, st));
    if (launch_occluded(accel->d_nodes, accel->d_tris, accel->ntri > 0, d_rays, d_t, nrays, d_hit, c.dev_error,
                        c.stream) != RN_OK)
        return cuda_fail(st, cudaGetLastError(), "occluded_kernel");
    if (dev) return ok(st);
    RN_TRY(copy_back(hit, d_hit, nrays, st));
    RN_TRY(check_device_error(st, "rn_occluded"));
    return ok(st);
}

// raw::rt::closest (src/renderer/rt_bvh.cpp:125-152) on the GPU: for each ray (origin,
// direction: 6 floats) the nearest hit below t_max, ties to the lowest triangle index.
int rn_closest(const rn_accel* accel, const float* rays, const float* t_max, uint32_t nrays, int flags, int32_t* tri,
               float* t, rn_status* st) {
    if (!accel || (nrays > 0 && (!rays || !t_max || !tri || !t))) return fail(st, RN_ERR_INVALID, "null argument");
    RN_TRY(ensure_ctx(st));
    Context& c = ctx();
    if (accel->device != c.device) return fail(st, RN_ERR_STATE, "accelerator belongs to device %d", accel->device);
    if (nrays == 0) return ok(st);
    const bool dev = (flags & RN_DEVICE_PTRS) != 0;
    const float *d_rays, *d_tm;
    int32_t* d_tri;
    float* d_t;
    RN_TRY(stage_in(rays, (size_t)nrays * 6, dev, WS_RAYS, &d_rays, st));
    RN_TRY(stage_in(t_max, (size_t)nrays, dev, WS_TMAX, &d_tm, st));
    RN_TRY(stage_out(tri, (size_t)nrays, dev, WS_CLOSEST_TRI, &d_tri, st));
    RN_TRY(stage_out(t, (size_t)nrays, dev, WS_CLOSEST_T, &d_t, st));
    if (launch_closest(accel->d_nodes, accel->d_tris, accel->ntri > 0, d_rays, d_tm, nrays, d_tri, d_t, c.dev_error,
                       c.stream) != RN_OK)
        return cuda_fail(st, cudaGetLastError(), "closest_kernel");
    if (dev) return ok(st);
    RN_TRY(copy_back(tri, d_tri, nrays, st));
    RN_TRY(copy_back(t, d_t, nrays, st));
    RN_TRY(check_device_error(st, "rn_closest"));
    return ok(st);
}

// The hybrid pass of raw::gpu_check::hybridGpu (src/renderer/gpu/rt_hybrid.cpp:43-83) over a
// G-buffer: per covered pixel a sun shadow ray and a mirror reflection ray (closest hit).
int rn_hybrid(const rn_gbuf* g, const float* geo_normal, const rn_accel* accel, const float* eye, const float* to_sun,
              int flags, float* lit, int32_t* refl_tri, float* refl_t, rn_status* st) {
    RN_TRY(ensure_ctx(st));
    RN_TRY(check_gbuf(g, st));
    if (!accel || !eye || !to_sun || !lit || !refl_tri || !refl_t) return fail(st, RN_ERR_INVALID, "null argument");
    Context& c = ctx();
    if (accel->device != c.device) return fail(st, RN_ERR_STATE, "accelerator belongs to device %d", accel->device);
    const bool dev = (flags & RN_DEVICE_PTRS) != 0;
    const size_t np = (size_t)g->w * g->h;
    StagedGbuf sg;
    RN_TRY(stage_gbuf(g, dev, &sg, st));
    const float* d_ng = nullptr;
    if (geo_normal) RN_TRY(stage_in(geo_normal, np * 3, dev, WS_HYB_NG, &d_ng, st));
    float *d_lit, *d_t;
    int32_t* d_tri;
    RN_TRY(stage_out(lit, np, dev, WS_HYB_LIT, &d_lit, st));
    RN_TRY(stage_out(refl_tri, np, dev, WS_HYB_TRI, &d_tri, st));
    RN_TRY(stage_out(refl_t, np, dev, WS_HYB_T, &d_t, st));
    if (launch_hybrid(g->w, g->h, sg.pos, sg.nrm, d_ng, sg.mask, accel, eye, to_sun, d_lit, d_tri, d_t, c.dev_error,
                      c.stream) != RN_OK)
        return cuda_fail(st, cudaGetLastError(), "hybrid_kernel");
    if (dev) return ok(st);
    RN_TRY(copy_back(lit, d_lit, np, st));
    RN_TRY(copy_back(refl_tri, d_tri, np, st));
    RN_TRY(copy_back(refl_t, d_t, np, st));
    RN_TRY(check_device_error(st, "rn_hybrid"));
    return ok(st);
}

}  // extern "C"
