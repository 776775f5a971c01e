// gemm_tc.cu -- the tensor-core GEMM of the learned AO surrogate: C = P * Q^T with P (M x K)
// and Q (N x K) in BF16, both K-major, accumulated in FP32 on sm_103a's fifth-generation
// tensor cores.
//
// One CTA of 128 threads computes one 128 x BN tile of C (BN = 32..256):
//   - warp 0, lane 0: TMA producer. Each 64-wide K step loads a 128 x 64 tile of P and a
//     BN x 64 tile of Q (cp.async.bulk.tensor, 128-byte swizzle) into one of 4 shared-memory
//     stages and signals the stage's "full" mbarrier with the byte count;
//   - warp 1, lane 0: MMA issuer. Per stage, four tcgen05.mma.kind::f16 (M 128, N BN, K 16)
//     accumulate into a BN-column TMEM accumulator; tcgen05.commit releases the stage
//     ("empty" mbarrier) when its MMAs have read it, and a final commit signals "done";
//   - all four warps: epilogue. Each thread owns one row (its warp's TMEM lane quarter),
//     reads it with tcgen05.ld 16 columns at a time, adds the bias, applies ReLU or the
//     ReLU-backward gate, and stores BF16 or FP32 (or adds FP32 atomically for split K).
// Every mbarrier wait is bounded; on a timeout the kernel sets the error word, waits
// (bounded) for its own copies in flight, frees its TMEM and returns.
#include "gemm_tc.h"
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <mutex>

namespace rn {
namespace tc {

constexpr int kStages = 4, kThreads = 128;
constexpr uint32_t kSpin = 1u << 24;      // try_wait rounds before a wait gives up

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t i = 0; i < kSpin; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}
// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);          // start address
    d |= (uint64_t)((1024u >> 4) & 0x3FFFu) << 32;            // stride byte offset
    d |= (uint64_t)1 << 46;                                   // descriptor version
    d |= (uint64_t)2 << 61;                                   // 128-byte swizzle
    return d;
}
// Instruction descriptor of tcgen05.mma.kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t instr_desc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
}
__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

template <int BN>
__global__ void __launch_bounds__(kThreads, 1) tc_gemm_kernel(const __grid_constant__ CUtensorMap mapP,
                                                              const __grid_constant__ CUtensorMap mapQ,
                                                              const Epilogue e) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    constexpr uint32_t kABytes = kBM * kBK * 2, kBBytes = BN * kBK * 2;
    constexpr uint32_t kCols = BN < 32 ? 32 : BN;
    uint8_t* sA = smem;
    uint8_t* sB = smem + kStages * kABytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sB + kStages * kBBytes);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kStages + 1);
    __shared__ int s_abort;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
    const int kbeg = blockIdx.z * e.k_per_split, nkb = e.k_per_split / kBK;
    auto full = [&](int s) { return smem_u32(&bars[s]); };
    auto empty = [&](int s) { return smem_u32(&bars[kStages + s]); };
    const uint32_t done = smem_u32(&bars[2 * kStages]);

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) { mbar_init(full(s), 1); mbar_init(empty(s), 1); }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // producer
        int issued = 0;
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % kStages;
            const uint32_t ph = (uint32_t)(kb / kStages) & 1u;
            if (!mbar_wait(empty(s), ph ^ 1u)) { atomicOr(e.err, DEV_GUARD); s_abort = 1; break; }
            mbar_expect_tx(full(s), kABytes + kBBytes);
            tma_load_2d(smem_u32(sA + s * kABytes), &mapP, kbeg + kb * kBK, m0, full(s));
            tma_load_2d(smem_u32(sB + s * kBBytes), &mapQ, kbeg + kb * kBK, n0, full(s));
            ++issued;
        }
        // the copies this thread issued must land before the CTA can leave
        for (int kb = issued > kStages ? issued - kStages : 0; kb < issued; ++kb)
            mbar_wait(full(kb % kStages), (uint32_t)(kb / kStages) & 1u);
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        const uint32_t idesc = instr_desc(BN);
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % kStages;
            const uint32_t ph = (uint32_t)(kb / kStages) & 1u;
            if (!mbar_wait(full(s), ph)) { atomicOr(e.err, DEV_GUARD); s_abort = 1; break; }
            tc_fence_after();
            const uint32_t a0 = smem_u32(sA + s * kABytes), b0 = smem_u32(sB + s * kBBytes);
#pragma unroll
            for (int k = 0; k < kBK / 16; ++k)
                tc_mma(tmem, smem_desc(a0 + k * 32), smem_desc(b0 + k * 32), idesc, (kb | k) != 0 ? 1u : 0u);
            tc_commit(empty(s));
        }
        tc_commit(done);
    }
    // epilogue: thread t owns row m0 + t, TMEM lane t
    const bool ok = __all_sync(0xffffffffu, mbar_wait(done, 0));    // warp-uniform: the loads below are .sync.aligned
    tc_fence_after();
    if (!ok && lane == 0) atomicOr(e.err, DEV_GUARD);
    const int abort_warp = __shfl_sync(0xffffffffu, *(volatile int*)&s_abort, 0);
    if (ok && !abort_warp) {
        const int row = m0 + warp * 32 + lane;
        const uint32_t tbase = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            uint32_t v[16];
            tmem_ld16(tbase + (uint32_t)c0, v);
            float f[16];
            const int col = n0 + c0;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                float x = __uint_as_float(v[j]);
                if (e.bias) x += e.bias[col + j];
                if (e.relu) x = fmaxf(x, 0.0f);
                f[j] = x;
            }
            const size_t o = (size_t)row * e.ldc + col;
            if (e.gate) {
                const uint4* g4 = reinterpret_cast<const uint4*>(e.gate + o);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const uint4 gv = g4[h];
                    const __nv_bfloat16* gb = reinterpret_cast<const __nv_bfloat16*>(&gv);
#pragma unroll
                    for (int j = 0; j < 8; ++j)
                        if (!(__bfloat162float(gb[j]) > 0.0f)) f[h * 8 + j] = 0.0f;
                }
            }
            if (e.c16) {
                uint4 out[2];
                __nv_bfloat16* ob = reinterpret_cast<__nv_bfloat16*>(out);
#pragma unroll
                for (int j = 0; j < 16; ++j) ob[j] = __float2bfloat16_rn(f[j]);
                uint4* d4 = reinterpret_cast<uint4*>(e.c16 + o);
                d4[0] = out[0];
                d4[1] = out[1];
            }
            if (e.c32) {
                float4* d4 = reinterpret_cast<float4*>(e.c32 + o);
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    const float4 q = make_float4(f[4 * h], f[4 * h + 1], f[4 * h + 2], f[4 * h + 3]);
                    if (e.atomic) atomicAdd(d4 + h, q);
                    else d4[h] = q;
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
}

// ------------------------------------------------------------------ host side
PFN_cuTensorMapEncodeTiled_v12000 encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// A 2-D map of a row-major BF16 matrix [rows][ld] (ld elements, K-major rows of `cols`), read
// in boxes of 64 x box_rows with the 128-byte swizzle.
bool make_map(CUtensorMap* m, const void* base, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows) {
    auto fn = encoder();
    if (!fn) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kBK, box_rows};
    const cuuint32_t elem[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, elem,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
int launch_bn(const CUtensorMap& mp, const CUtensorMap& mq, const Epilogue& e, int M, int N, int splits,
              cudaStream_t s) {
    const size_t smem = 1024 + kStages * (kBM * kBK * 2 + BN * kBK * 2) + (2 * kStages + 1) * 8 + 16;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(tc_gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return RN_ERR_CUDA;
        attr = true;
    }
    const dim3 grid(M / kBM, N / BN, splits);
    tc_gemm_kernel<BN><<<grid, kThreads, smem, s>>>(mp, mq, e);
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}

}  // namespace tc

// C (M x N, row stride ldc) = P (M x K, row stride ldp) * Q (N x K, row stride ldq)^T.
// M % 128 == 0, N in {32, 64, 128, 256} or a multiple of 128, K % (64 * splits) == 0;
// P, Q 16-byte aligned with ldp, ldq multiples of 8. splits > 1 requires c32 with atomic.
int tc_gemm(const __nv_bfloat16* P, int ldp, const __nv_bfloat16* Q, int ldq, int M, int N, int K, int splits,
            const tc::Epilogue& epi, cudaStream_t s, rn_status* st) {
    if (M <= 0 || N <= 0 || K <= 0 || M % tc::kBM || splits < 1 || K % (tc::kBK * splits))
        return fail(st, RN_ERR_INVALID, "tc_gemm shape M %d N %d K %d splits %d", M, N, K, splits);
    if ((ldp % 8) || (ldq % 8) || ((uintptr_t)P % 16) || ((uintptr_t)Q % 16))
        return fail(st, RN_ERR_INVALID, "tc_gemm operands must be 16-byte aligned rows");
    if (splits > 1 && !(epi.c32 && epi.atomic)) return fail(st, RN_ERR_INVALID, "split K needs an atomic FP32 output");
    const int bn = (N == 32 || N == 64 || N == 128 || N == 256) ? N : 128;
    if (N % bn) return fail(st, RN_ERR_INVALID, "tc_gemm N %d", N);
    tc::Epilogue e = epi;
    e.k_per_split = K / splits;
    CUtensorMap mp, mq;
    if (!tc::make_map(&mp, P, (uint64_t)M, (uint64_t)K, (uint64_t)ldp, tc::kBM) ||
        !tc::make_map(&mq, Q, (uint64_t)N, (uint64_t)K, (uint64_t)ldq, (uint32_t)bn))
        return fail(st, RN_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    int rc;
    switch (bn) {
        case 32: rc = tc::launch_bn<32>(mp, mq, e, M, N, splits, s); break;
        case 64: rc = tc::launch_bn<64>(mp, mq, e, M, N, splits, s); break;
        case 256: rc = tc::launch_bn<256>(mp, mq, e, M, N, splits, s); break;
        default: rc = tc::launch_bn<128>(mp, mq, e, M, N, splits, s); break;
    }
    if (rc != RN_OK) return cuda_fail(st, cudaGetLastError(), "tc_gemm_kernel");
    return RN_OK;
}

}  // namespace rn

using namespace rn;

// Test and measurement entry of the GEMM (device pointers, the library's stream).
extern "C" int rn_tc_gemm(const void* P, int ldp, const void* Q, int ldq, int M, int N, int K, int splits, float* c32,
                          void* c16, int ldc, const float* bias, int relu, rn_status* st) {
    RN_TRY(ensure_ctx(st));
    tc::Epilogue e{};
    e.ldc = ldc;
    e.c32 = c32;
    e.c16 = (__nv_bfloat16*)c16;
    e.bias = bias;
    e.relu = relu;
    e.atomic = splits > 1;
    e.err = ctx().dev_error;
    RN_TRY(tc_gemm((const __nv_bfloat16*)P, ldp, (const __nv_bfloat16*)Q, ldq, M, N, K, splits, e, ctx().stream, st));
    return ok(st);
}
