// ssao_device.cuh -- one 32 x 8 tile of the SSAO pass with the reconcile's per-thread share,
// shared by the single-frame kernel (ssao.cu) and the batched multi-view kernel (batch.cu).
// See ssao.cu for the design.
#pragma once
#include "rn_internal.h"
#include "rn_device.cuh"
#include "rn_reduce.cuh"

namespace rn {
namespace ssao_dev {

// A tile is kTX x TY pixels, one thread each (TY = 8 by default; 4 and 16 are the
// autotuner's alternatives), with a window of (TY + 2R) x (kTX + 2R) positions.
constexpr int kTX = 32, kTY = 8, kR = 6;
constexpr int kSW = kTX + 2 * kR, kSH = kTY + 2 * kR;
constexpr int kThreads = kTX * kTY;
template <int TY> struct Tile {
    static constexpr int kH = TY + 2 * kR;
    static constexpr int kThreads = kTX * TY;
};

__device__ __forceinline__ bool near_half(float v) {
    const float a = fabsf(v);
    return fabsf(a - floorf(a) - 0.5f) < 8e-6f;
}

// Tile (bx, by) of a w x h frame: SSAO into ao, and with kFused the error against `truth`
// into err (may be null) with this thread's share of the reconcile in `acc`. `win` is the
// block's shared window. Every thread of the block must call it.
template <bool kFused, int TY = kTY>
__device__ __forceinline__ void ssao_tile(float4 (&win)[Tile<TY>::kH][kSW], int bx, int by, int w, int h,
                                          const float* __restrict__ pos, const float* __restrict__ nrm,
                                          const uint8_t* __restrict__ mask, int samples, float radius,
                                          const uint8_t* __restrict__ corr, float* __restrict__ ao,
                                          const float* __restrict__ truth, float* __restrict__ err, RecAcc& acc) {
    const int x0 = bx * kTX, y0 = by * TY;
    for (int q = threadIdx.x; q < Tile<TY>::kH * kSW; q += Tile<TY>::kThreads) {
        const int wy = q / kSW, wx = q % kSW;
        const int gx = x0 - kR + wx, gy = y0 - kR + wy;
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (gx >= 0 && gy >= 0 && gx < w && gy < h) {
            const size_t j = (size_t)gy * w + gx;
            if (mask[j]) v = make_float4(pos[3 * j], pos[3 * j + 1], pos[3 * j + 2], 1.0f);
        }
        win[wy][wx] = v;
    }
    __syncthreads();
    const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
    const int x = x0 + tx, y = y0 + ty;
    if (x < w && y < h) {
        const size_t i = (size_t)y * w + x;
        const bool covered = mask[i] != 0;
        float a = 1.0f;
        if (covered) {
            const float4 Pw = win[ty + kR][tx + kR];
            const v3 P = mk(Pw.x, Pw.y, Pw.z);
            const v3 n = load3(nrm + 3 * i);
            int occ = 0, used = 0;
            for (int s = 0; s < samples; ++s) {
                const uint32_t k1 = hash24((uint32_t)x, (uint32_t)y, (uint32_t)s);
                const float rad = fmul(fadd(0.3f, fmul(0.7f, unit24(hash24((uint32_t)x, (uint32_t)y, (uint32_t)(s + 97))))), 6.0f);
                float c, sn;
                sample_sincos(k1, nullptr, c, sn);
                float vx = fmul(c, rad), vy = fmul(sn, rad);
                if (corr && (near_half(vx) || near_half(vy))) {
                    sample_sincos(k1, corr, c, sn);
                    vx = fmul(c, rad);
                    vy = fmul(sn, rad);
                }
                const int dx = (int)lroundf(vx), dy = (int)lroundf(vy);
                const float4 Q = win[ty + kR + dy][tx + kR + dx];
                if (Q.w == 0.0f) continue;            // out of the frame or not covered
                ++used;
                const v3 d = sub(mk(Q.x, Q.y, Q.z), P);
                const float dist = length(d);
                if (dist < 1e-4f || dist > radius) continue;
                const float ndl = dot(n, normalize(d));
                if (ndl > 0.15f) ++occ;
            }
            a = used > 0 ? fsub(1.0f, fdiv((float)occ, (float)used)) : 1.0f;
            a = a < 0.0f ? 0.0f : a;
        }
        ao[i] = a;
        if (kFused) {
            float e = 0.0f;
            if (covered) {
                e = fabsf(fsub(a, truth[i]));
                acc.add(e);
            }
            if (err) err[i] = e;
        }
    }
}

}  // namespace ssao_dev
}  // namespace rn
