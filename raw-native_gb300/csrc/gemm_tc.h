// gemm_tc.h -- the surrogate's tensor-core GEMM (gemm_tc.cu): C = P * Q^T, BF16 in,
// FP32 accumulation in TMEM.
#pragma once
#include "rn_internal.h"
#include <cuda_bf16.h>

namespace rn {
namespace tc {

constexpr int kBM = 128, kBK = 64;

struct Epilogue {
    int ldc;                         // row stride of C in elements
    float* c32;                      // FP32 output (split K: accumulated with atomics)
    __nv_bfloat16* c16;              // BF16 output
    const float* bias;               // [N] or null
    const __nv_bfloat16* gate;       // [M][ldc]: output zeroed where gate <= 0 (ReLU backward), or null
    int relu;
    int atomic;
    int k_per_split;                 // K range of one grid.z slice (a multiple of 64)
    uint32_t* err;
    uint32_t spin;                   // try_wait rounds before a wait gives up (0: the default)
    int withhold;                    // self-test only: the first K block's copies are never issued
    // convolutions with N = 32 in one slice: the U-Net head fused into the epilogue,
    // head_out[pixel] = sigmoid(head_b[0] + sum over c of bf16(out[c]) * head_w[c]), c in order
    const float* head_w;
    const float* head_b;
    float* head_out;
};

// One input of an implicit-GEMM 3x3 convolution: an NHWC BF16 tensor at the output's
// resolution with C channels (C a multiple of 32).
struct ConvSrc {
    const __nv_bfloat16* ptr;
    int C;
};

// Output tiling of the implicit convolution: 128 output pixels per CTA as a TH x TW block
// (TW = the largest power of two <= 128 dividing W, TH = 128 / TW; H % TH == 0).
struct ConvTiling {
    int tw_log2;
    bool ok;
};
ConvTiling conv_tiling(int H, int W);

}  // namespace tc

// Implicit-GEMM 3x3 convolution, stride 1, zero padding 1 (no im2col in memory):
//   out[b, y, x, n] = sum over taps (dy, dx) and input channels ci of
//                     in[b, y + dy - 1, x + dx - 1, ci] * w[n][tap * Cin + ci]
// with the inputs' channels concatenated (src[0] first), Cin = sum of src[i].C, w [N][ldw]
// BF16 (ldw >= 9 Cin, a multiple of 8). Per K step the producer loads, by TMA, the
// (channels x TW x TH) box of one source at the tap's offset (the border reads zeros) and
// the matching weight columns. The epilogue's ldc/c16/c32/bias/relu apply per pixel row;
// up16, when set, also receives the output upsampled 2x (nearest) at (2H, 2W).
int tc_conv3x3(const tc::ConvSrc* src, int nsrc, int B, int H, int W, const __nv_bfloat16* w, int ldw, int N,
               const tc::Epilogue& epi, __nv_bfloat16* up16, cudaStream_t s, rn_status* st);

// C (M x N, row stride ldc) = P (M x K, row stride ldp) * Q (N x K, row stride ldq)^T.
// M % 128 == 0, N in {32, 64, 128, 256} or a multiple of 128, K % (64 * splits) == 0;
// P, Q 16-byte aligned with ldp, ldq multiples of 8. splits > 1 requires c32 with atomic.
int tc_gemm(const __nv_bfloat16* P, int ldp, const __nv_bfloat16* Q, int ldq, int M, int N, int K, int splits,
            const tc::Epilogue& epi, cudaStream_t s, rn_status* st);

}  // namespace rn
