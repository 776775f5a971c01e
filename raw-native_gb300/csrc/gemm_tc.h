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
};

}  // namespace tc

// C (M x N, row stride ldc) = P (M x K, row stride ldp) * Q (N x K, row stride ldq)^T.
// M % 128 == 0, N in {32, 64, 128, 256} or a multiple of 128, K % (64 * splits) == 0;
// P, Q 16-byte aligned with ldp, ldq multiples of 8. splits > 1 requires c32 with atomic.
int tc_gemm(const __nv_bfloat16* P, int ldp, const __nv_bfloat16* Q, int ldq, int M, int N, int K, int splits,
            const tc::Epilogue& epi, cudaStream_t s, rn_status* st);

}  // namespace rn
