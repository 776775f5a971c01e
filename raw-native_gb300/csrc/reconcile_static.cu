// reconcile_static.cu -- the reconcile with its scratch in a fixed device array, for callers
// that cannot let this library allocate GPU memory.
//
// Who needs it: a host that budgets every byte of device memory up front and refuses growth
// afterwards (raw-native's own renderer runs its frames in a fail-closed arena: an
// allocation over budget is refused, not grown), a frame loop that must not stall on
// cudaMalloc/cudaFree (both can synchronize the device), and code that owns the device's
// memory through its own pool. rn_reconcile gets its scratch (per-block partial sums and the
// completion counter) from the library's workspace, which cudaMallocs on first use and when
// an image grows; this entry point uses the array below instead and allocates nothing.
//
// The array: kScratchBytes (33 KiB) of file-scope device memory, held by every GPU that
// loads the library until the process exits. It holds one partial per reduction block (the
// reconcile never launches more than kMaxBlocks blocks, whatever the image size) and the
// completion counter. Host code cannot use the array's name as a device address, so each
// device's address comes from cudaGetSymbolAddress, once per device, on that device's first
// call, and is kept for the life of the process: it is not valid across a cudaDeviceReset of
// that device (the module and its array are loaded anew), so a process that resets a device
// must not call this entry point on it again. No call may be made on a stream under capture:
// it reads its result back into host memory and synchronizes the stream. Every call shares
// the array: the counter is cleared at each call, and calls that overlap on the GPU (two
// streams, or two host threads) race on it and must be serialized by the caller.
#include "rn_internal.h"
#include <cmath>
#include <mutex>

namespace rn {
namespace {

constexpr int kMaxBlocks = 2048;                              // reconcile_blocks() never exceeds this
constexpr size_t kPartialBytes = (size_t)kMaxBlocks * sizeof(RecPartial);
constexpr size_t kScratchBytes = kPartialBytes + 256;         // partials, then the RecOut counter block
static_assert(sizeof(RecOut) <= 256, "RecOut fits its slot");

static __device__ __align__(256) unsigned char g_reconcile_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_addr[kMaxDevices] = {};

// The scratch array's device address on the current device (set up once per device).
int scratch_address(int dev, void** out, rn_status* st) {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_reconcile_scratch);
        if (e != cudaSuccess) return cuda_fail(st, e, "cudaGetSymbolAddress(reconcile scratch)");
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return RN_OK;
}

}  // namespace
}  // namespace rn

using namespace rn;

extern "C" int rn_reconcile_noalloc(const float* approx, const float* truth, const uint8_t* mask, int w, int h,
                                    float tolerance, void* stream, float* err, rn_reconcile_result* out,
                                    rn_status* st) {
    if (!approx || !truth || !mask || !out) return fail(st, RN_ERR_INVALID, "null argument");
    if (w < 0 || h < 0) return fail(st, RN_ERR_INVALID, "size %dx%d", w, h);
    const size_t np = (size_t)w * (size_t)h;
    if (np > (size_t)0x7FFFFFFF)
        return fail(st, RN_ERR_INVALID, "%zu pixels: the allocation-free reconcile takes at most 2^31-1", np);
    if (np == 0) {
        *out = rn_reconcile_result{0.0f, 0.0f, 0, 0.0f <= tolerance ? 1 : 0, 0.0};
        return ok(st);
    }
    const int nb = reconcile_blocks(np);
    if (nb > kMaxBlocks) return fail(st, RN_ERR_INVALID, "%d reduction blocks exceed the scratch's %d", nb, kMaxBlocks);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(st, RN_ERR_NO_DEVICE, "no CUDA device");
    int dev = 0;
    RN_CUDA(cudaGetDevice(&dev), st);
    if (dev < 0 || dev >= kMaxDevices) return fail(st, RN_ERR_STATE, "device ordinal %d out of range", dev);
    void* base = nullptr;
    RN_TRY(scratch_address(dev, &base, st));
    RecPartial* parts = (RecPartial*)base;
    RecOut* ro = (RecOut*)((char*)base + kPartialBytes);
    const cudaStream_t s = (cudaStream_t)stream;
    RN_CUDA(cudaMemsetAsync(ro, 0, sizeof(RecOut), s), st);   // the completion counter starts at zero
    const cudaError_t le = launch_reconcile(approx, truth, mask, np, err, parts, nb, ro, s);
    if (le != cudaSuccess) return cuda_fail(st, le, "reconcile_kernel (allocation-free)");
    RecOut r;
    RN_CUDA(cudaMemcpyAsync(&r, ro, sizeof r, cudaMemcpyDeviceToHost, s), st);
    RN_CUDA(cudaStreamSynchronize(s), st);
    out->sum_sq = r.sum;
    out->pixels = r.n;
    out->max_error = r.max;
    out->rmse = r.n > 0 ? (float)std::sqrt(r.sum / (double)r.n) : 0.0f;
    out->within_tolerance = out->rmse <= tolerance ? 1 : 0;
    return ok(st);
}
