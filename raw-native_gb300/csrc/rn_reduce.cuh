// rn_reduce.cuh -- the reconcile's reduction: sum of squared errors, max error, pixel count.
//
// src/cert/reconcile.cpp:10-20 sums (double)e * e in FP64 in row-major order. Here every e^2
// is formed exactly (float two-product: p = e*e plus its rounding error fma(e, e, -p)) and
// summed per thread with a compensated float pair (two-sum), then the threads' pairs are
// combined in FP64 in a fixed tree order, the blocks' FP64 partials by the last block in
// block order. The result is the same on every run, and it carries less rounding than the
// sequential FP64 sum it stands for. GB300 issues FP64 at a small fraction of its FP32 rate,
// so the per-pixel work stays in FP32 and FP64 is used once per thread.
#pragma once
#include "rn_internal.h"

namespace rn {

struct RecAcc {
    float hi = 0.0f, lo = 0.0f, mx = 0.0f;
    int n = 0;
    __device__ __forceinline__ void add(float e) {
        const float p = __fmul_rn(e, e);
        const float pe = __fmaf_rn(e, e, -p);          // exact: e*e = p + pe
        const float s = __fadd_rn(hi, p);
        const float bp = __fsub_rn(s, hi);
        const float d = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(p, bp));   // exact: hi + p = s + d
        hi = s;
        lo = __fadd_rn(lo, __fadd_rn(d, pe));
        mx = fmaxf(mx, e);                              // NaN never replaces a max, as `e > max` in the reference
        ++n;
    }
};

// Reduce one RecAcc per thread to one RecPartial for the block (fixed tree order), then let
// the last block to finish combine all blocks' partials in block order into *out.
// Every thread of the block must call it.
template <int kThreads>
__device__ void rec_block_finish(const RecAcc& a, RecPartial* __restrict__ parts, RecOut* out, uint32_t block,
                                 uint32_t nblocks) {
    __shared__ double s_sum[kThreads / 32];
    __shared__ float s_max[kThreads / 32];
    __shared__ int s_n[kThreads / 32];
    __shared__ bool s_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double sum = (double)a.hi + (double)a.lo;
    float mx = a.mx;
    int n = a.n;
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xffffffffu, sum, o);
        mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
        n += __shfl_down_sync(0xffffffffu, n, o);
    }
    if (lane == 0) { s_sum[warp] = sum; s_max[warp] = mx; s_n[warp] = n; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double bs = 0.0;
        float bm = 0.0f;
        int bn = 0;
        for (int w = 0; w < kThreads / 32; ++w) { bs += s_sum[w]; bm = fmaxf(bm, s_max[w]); bn += s_n[w]; }
        parts[block] = RecPartial{bs, bm, bn};
        __threadfence();
        const uint32_t ticket = atomicAdd(&out->done, 1u);
        s_last = ticket == nblocks - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // the last block: every thread sums a strided run of partials in order, then a fixed tree
    double ts = 0.0;
    float tm = 0.0f;
    int tn = 0;
    const volatile RecPartial* vp = parts;
    for (uint32_t b = threadIdx.x; b < nblocks; b += kThreads) {
        ts += vp[b].sum;
        tm = fmaxf(tm, vp[b].max);
        tn += vp[b].n;
    }
    for (int o = 16; o > 0; o >>= 1) {
        ts += __shfl_down_sync(0xffffffffu, ts, o);
        tm = fmaxf(tm, __shfl_down_sync(0xffffffffu, tm, o));
        tn += __shfl_down_sync(0xffffffffu, tn, o);
    }
    if (lane == 0) { s_sum[warp] = ts; s_max[warp] = tm; s_n[warp] = tn; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double bs = 0.0;
        float bm = 0.0f;
        int bn = 0;
        for (int w = 0; w < kThreads / 32; ++w) { bs += s_sum[w]; bm = fmaxf(bm, s_max[w]); bn += s_n[w]; }
        out->sum = bs;
        out->max = bm;
        out->n = bn;
        out->done = 0;     // ready for the next launch
    }
}

}  // namespace rn
