// reconcile.cu -- the reconcile pass (src/cert/reconcile.cpp:4-21) on the GPU: error map
// plus the FP64-grade sum of squares, max and count, in one HBM-bound sweep.
//
// Traffic per pixel: approx 4 B + truth 4 B + mask 1 B read, error 4 B written (13 B).
// Each thread moves 4 pixels per step with 16-byte loads and stores when the buffers allow.
#include "rn_internal.h"
#include "rn_device.cuh"
#include "rn_reduce.cuh"

namespace rn {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float rec_px(float a, float t, uint8_t m, RecAcc& acc) {
    if (!m) return 0.0f;
    const float e = fabsf(__fsub_rn(a, t));
    acc.add(e);
    return e;
}

template <bool kVec>
__global__ void __launch_bounds__(kThreads) reconcile_kernel(const float* __restrict__ approx, const float* __restrict__ truth,
                                                             const uint8_t* __restrict__ mask, size_t npx,
                                                             float* __restrict__ err, RecPartial* parts, RecOut* out) {
    RecAcc acc;
    const size_t stride = (size_t)gridDim.x * kThreads;
    size_t tail0 = 0;
    if (kVec) {
        const size_t nq = npx / 4;
        const float4* a4 = reinterpret_cast<const float4*>(approx);
        const float4* t4 = reinterpret_cast<const float4*>(truth);
        const uchar4* m4 = reinterpret_cast<const uchar4*>(mask);
        float4* e4 = reinterpret_cast<float4*>(err);
        for (size_t q = (size_t)blockIdx.x * kThreads + threadIdx.x; q < nq; q += stride) {
            const float4 a = __ldcs(a4 + q), t = __ldcs(t4 + q);
            const uchar4 m = __ldcs(m4 + q);
            float4 e;
            e.x = rec_px(a.x, t.x, m.x, acc);
            e.y = rec_px(a.y, t.y, m.y, acc);
            e.z = rec_px(a.z, t.z, m.z, acc);
            e.w = rec_px(a.w, t.w, m.w, acc);
            if (err) __stcs(e4 + q, e);
        }
        tail0 = nq * 4;
    }
    for (size_t i = tail0 + (size_t)blockIdx.x * kThreads + threadIdx.x; i < npx; i += stride) {
        const float e = rec_px(approx[i], truth[i], mask[i], acc);
        if (err) err[i] = e;
    }
    rec_block_finish<kThreads>(acc, parts, out, blockIdx.x, gridDim.x);
}

}  // namespace

// The block count depends on the pixel count alone, so the reduction order, and with it
// every bit of the result, is the same on every run and every GPU.
int reconcile_blocks(size_t npx) {
    const size_t per_block = (size_t)kThreads * 4 * 8;
    size_t nb = (npx + per_block - 1) / per_block;
    if (nb < 1) nb = 1;
    if (nb > 2048) nb = 2048;
    return (int)nb;
}

cudaError_t launch_reconcile(const float* approx, const float* truth, const uint8_t* mask, size_t npx, float* err,
                             RecPartial* partials, int nblocks, RecOut* out, cudaStream_t s) {
    const bool vec = ((uintptr_t)approx % 16 == 0) && ((uintptr_t)truth % 16 == 0) && ((uintptr_t)mask % 4 == 0) &&
                     (err == nullptr || (uintptr_t)err % 16 == 0);
    if (vec)
        reconcile_kernel<true><<<nblocks, kThreads, 0, s>>>(approx, truth, mask, npx, err, partials, out);
    else
        reconcile_kernel<false><<<nblocks, kThreads, 0, s>>>(approx, truth, mask, npx, err, partials, out);
    return cudaGetLastError();
}

}  // namespace rn
