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
#include <algorithm>
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
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t limit = kSpin) {
    for (uint32_t i = 0; i < limit; ++i) {
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
// The same for rows of 64 bytes (32 BF16): 64-byte swizzle, 8-row atoms 512 bytes apart.
__device__ __forceinline__ uint64_t smem_desc64(uint32_t addr) {
    uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((512u >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)4 << 61;                                   // 64-byte swizzle
    return d;
}
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c, int x, int y, int b,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c), "r"(x), "r"(y), "r"(b), "r"(bar)
        : "memory");
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

// 64 consecutive TMEM columns of this warp's 32 lanes in one load and one wait.
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, uint32_t (&v)[64]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, %48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%64];\n"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31]), "=r"(v[32]), "=r"(v[33]), "=r"(v[34]), "=r"(v[35]), "=r"(v[36]), "=r"(v[37]), "=r"(v[38]), "=r"(v[39]), "=r"(v[40]), "=r"(v[41]), "=r"(v[42]), "=r"(v[43]), "=r"(v[44]), "=r"(v[45]), "=r"(v[46]), "=r"(v[47]), "=r"(v[48]), "=r"(v[49]), "=r"(v[50]), "=r"(v[51]), "=r"(v[52]), "=r"(v[53]), "=r"(v[54]), "=r"(v[55]), "=r"(v[56]), "=r"(v[57]), "=r"(v[58]), "=r"(v[59]), "=r"(v[60]), "=r"(v[61]), "=r"(v[62]), "=r"(v[63])
        : "r"(taddr)
        : "memory");
}
// Zeros into 32 consecutive TMEM columns of this warp's 32 lanes (its wait is separate:
// tcgen05.wait::st before the columns are handed to the MMAs).
__device__ __forceinline__ void tmem_zero32(uint32_t taddr) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
        "%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1};" ::"r"(taddr), "r"(0u)
        : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// 32 consecutive TMEM columns of this warp's 32 lanes, the load and its wait in one
// statement (the registers are defined only once the wait has returned).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
          "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr)
        : "memory");
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

    const uint32_t spin = e.spin ? e.spin : kSpin;
    if (warp == 0 && lane == 0) {
        // producer
        int issued = 0;
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % kStages;
            const uint32_t ph = (uint32_t)(kb / kStages) & 1u;
            if (!mbar_wait(empty(s), ph ^ 1u, spin)) { atomicOr(e.err, DEV_GUARD); s_abort = 1; break; }
            mbar_expect_tx(full(s), kABytes + kBBytes);
            if (e.withhold && kb == 0) continue;      // the self-test's missing copy: its stage never fills
            tma_load_2d(smem_u32(sA + s * kABytes), &mapP, kbeg + kb * kBK, m0, full(s));
            tma_load_2d(smem_u32(sB + s * kBBytes), &mapQ, kbeg + kb * kBK, n0, full(s));
            ++issued;
        }
        // the copies this thread issued must land before the CTA can leave
        for (int kb = issued > kStages ? issued - kStages : 0; kb < issued; ++kb)
            mbar_wait(full(kb % kStages), (uint32_t)(kb / kStages) & 1u, spin);
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        const uint32_t idesc = instr_desc(BN);
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % kStages;
            const uint32_t ph = (uint32_t)(kb / kStages) & 1u;
            if (!mbar_wait(full(s), ph, spin)) { atomicOr(e.err, DEV_GUARD); s_abort = 1; break; }
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
    const bool ok = __all_sync(0xffffffffu, mbar_wait(done, 0, spin));    // warp-uniform: the loads below are .sync.aligned
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


// ------------------------------------------------------------------ implicit 3x3 convolution
// A persistent kernel: each CTA walks work items (128-pixel tile, BN-column slice) with a
// stride of the grid, keeping its barriers and TMEM across items. CB is the channel block of
// one K step (64: 128-byte rows and swizzle; 32: 64-byte rows and swizzle); a K step is
// (tap, source, channel block), taps outermost, matching the weights' column order
// tap * Cin + ci. Roles (6 warps):
//   - warp 0, lane 0: TMA producer over all items' K steps, through a ring of kSt stages;
//   - warp 1, lane 0: MMA issuer; item i accumulates into TMEM buffer i & 1 (2 x BN columns),
//     so the MMAs of item i + 1 run while the epilogue drains item i;
//   - warps 2..5: epilogue; warp w reads TMEM lanes 32 (w % 4) .. +31 (its row quarter),
//     then releases the buffer.
// Every wait is bounded and also gives up when another role has aborted.
constexpr int kConvThreads = 192;

struct ConvArgs {
    int nsrc;
    int C0, C1;                 // channels of the sources
    int B, H, W, tw_log2;       // output (= input) geometry and tiling
    int tiles_x, tiles_y;       // tiles per image row / column
    int cin;                    // C0 + C1
    int n_slices;               // N / BN
    int items;                  // tiles x slices
    __nv_bfloat16* up16;        // optional 2x nearest-upsampled copy of the BF16 output
};

__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t bar, uint32_t parity, volatile int* abort_flag) {
    for (uint32_t i = 0; i < kSpin; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if ((i & 255u) == 255u && *abort_flag) return false;
    }
    return false;
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// kT tiles per work item (1 or 2): with 2, every weight box feeds two 128-pixel tiles (two
// A boxes per stage, two TMEM accumulators per buffer), halving the weights' L2 traffic;
// each tile's MMAs are the same in the same order.
// Pipeline stages of tc_conv_kernel: 8 of 32 channels or 4 of 64; pairs of tiles with a
// 64-column or narrower slice take half as many, so that two CTAs still share an SM.
template <int BN, int CB, int kT>
__host__ __device__ constexpr int conv_stages() { return (CB == 32 ? 8 : 4) / (kT == 2 && BN <= 64 ? 2 : 1); }

template <int BN, int CB, int kT>
__global__ void __launch_bounds__(kConvThreads, 1) tc_conv_kernel(const __grid_constant__ CUtensorMap map0,
                                                                  const __grid_constant__ CUtensorMap map1,
                                                                  const __grid_constant__ CUtensorMap mapW,
                                                                  const ConvArgs a, const Epilogue e) {
    constexpr int kSt = conv_stages<BN, CB, kT>();
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    constexpr uint32_t kABytes = kBM * CB * 2, kBBytes = BN * CB * 2;
    constexpr uint32_t kCols = 2 * kT * BN;                  // two buffers of kT accumulators
    uint8_t* sA = smem;                                      // kSt stages of kT A boxes
    uint8_t* sB = smem + kSt * kT * kABytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sB + kSt * kBBytes);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kSt + 4);
    __shared__ int s_abort;
    __shared__ float s_bias[512];       // the bias of every output channel, staged once
    volatile int* abort_flag = &s_abort;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tw = 1 << a.tw_log2, th = kBM >> a.tw_log2;
    const int nb0 = a.C0 / CB, nb1 = a.nsrc > 1 ? a.C1 / CB : 0, per_tap = nb0 + nb1;
    const int nkb = 9 * per_tap;
    auto full = [&](int s) { return smem_u32(&bars[s]); };
    auto empty = [&](int s) { return smem_u32(&bars[kSt + s]); };
    auto acc_full = [&](int b) { return smem_u32(&bars[2 * kSt + b]); };
    auto acc_empty = [&](int b) { return smem_u32(&bars[2 * kSt + 2 + b]); };

    if (threadIdx.x == 0) {
        for (int s = 0; s < kSt; ++s) { mbar_init(full(s), 1); mbar_init(empty(s), 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(acc_full(b), 1); mbar_init(acc_empty(b), 4); }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    if (e.bias)
        for (int i = threadIdx.x; i < a.n_slices * BN; i += blockDim.x) s_bias[i] = e.bias[i];
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

    if (warp == 0) {
        // lane s < kSt owns stage s: it issues K steps kc = s, s + kSt, ... of this CTA's
        // sequence (items blockIdx.x, + gridDim.x, ...; nkb steps each), waiting for each
        // previous use of its stage in order, so the stages fill in parallel
        if (lane < kSt) {
            const int my_items = a.items > (int)blockIdx.x ? (a.items - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
            const uint32_t total = (uint32_t)my_items * (uint32_t)nkb;
            uint32_t last = 0xFFFFFFFFu;
            for (uint32_t kc = lane; kc < total; kc += kSt) {
                const uint32_t ph = (kc / kSt) & 1u;
                if (!mbar_wait_or_abort(empty(lane), ph ^ 1u, abort_flag)) {
                    atomicOr(e.err, DEV_GUARD);
                    s_abort = 1;
                    break;
                }
                const int item = (int)blockIdx.x + (int)(kc / nkb) * (int)gridDim.x, kb = (int)(kc % nkb);
                const int group = item / a.n_slices, n0 = (item % a.n_slices) * BN;
                const int tap = kb / per_tap, r = kb % per_tap;
                const bool second = r >= nb0;
                const int cb = second ? r - nb0 : r;
                mbar_expect_tx(full(lane), kT * kABytes + kBBytes);
                for (int t = 0; t < kT; ++t) {
                    const int tile = group * kT + t;
                    const int tx = tile % a.tiles_x, ty = (tile / a.tiles_x) % a.tiles_y, b = tile / (a.tiles_x * a.tiles_y);
                    tma_load_4d(smem_u32(sA + (lane * kT + t) * kABytes), second ? &map1 : &map0, cb * CB,
                                tx * tw + tap % 3 - 1, ty * th + tap / 3 - 1, b, full(lane));
                }
                tma_load_2d(smem_u32(sB + lane * kBBytes), &mapW, tap * a.cin + (second ? a.C0 : 0) + cb * CB, n0,
                            full(lane));
                last = kc;
            }
            // the copies this lane issued must land before the CTA can leave
            if (last != 0xFFFFFFFFu) mbar_wait(full(lane), (last / kSt) & 1u);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = instr_desc(BN);
            uint32_t kc = 0, i = 0;
            for (int item = blockIdx.x; item < a.items && !*abort_flag; item += gridDim.x, ++i) {
                const uint32_t buf = i & 1u, use = i >> 1;
                if (!mbar_wait_or_abort(acc_empty(buf), (use & 1u) ^ 1u, abort_flag)) {
                    atomicOr(e.err, DEV_GUARD);
                    s_abort = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t acc = tmem + buf * kT * BN;
                bool ok = true;
                for (int kb = 0; kb < nkb; ++kb, ++kc) {
                    const int s = kc % kSt;
                    const uint32_t ph = (kc / kSt) & 1u;
                    if (!mbar_wait_or_abort(full(s), ph, abort_flag)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t b0 = smem_u32(sB + s * kBBytes);
#pragma unroll
                    for (int k = 0; k < CB / 16; ++k) {
                        const uint64_t db = CB == 64 ? smem_desc(b0 + k * 32) : smem_desc64(b0 + k * 32);
#pragma unroll
                        for (int t = 0; t < kT; ++t) {
                            const uint32_t a0 = smem_u32(sA + (s * kT + t) * kABytes);
                            const uint64_t da = CB == 64 ? smem_desc(a0 + k * 32) : smem_desc64(a0 + k * 32);
                            tc_mma(acc + (uint32_t)(t * BN), da, db, idesc, (kb | k) != 0 ? 1u : 0u);
                        }
                    }
                    tc_commit(empty(s));
                }
                if (!ok) {
                    atomicOr(e.err, DEV_GUARD);
                    s_abort = 1;
                    break;
                }
                tc_commit(acc_full(buf));
            }
        }
    } else {
        // epilogue warps 2..5: TMEM lane quarter q = warp % 4 holds rows 32 q .. 32 q + 31
        const int q = warp & 3;
        const int r = q * 32 + lane;
        uint32_t i = 0;
        for (int item = blockIdx.x; item < a.items; item += gridDim.x, ++i) {
            const uint32_t buf = i & 1u, use = i >> 1;
            const bool ok = __all_sync(0xffffffffu, mbar_wait_or_abort(acc_full(buf), use & 1u, abort_flag));
            if (!ok) {
                if (lane == 0) { atomicOr(e.err, DEV_GUARD); s_abort = 1; }
                break;
            }
            tc_fence_after();
            const int group = item / a.n_slices, n0 = (item % a.n_slices) * BN;
#pragma unroll 1
            for (int t = 0; t < kT; ++t) {
            const int tile = group * kT + t;
            const int tx = tile % a.tiles_x, ty = (tile / a.tiles_x) % a.tiles_y, b = tile / (a.tiles_x * a.tiles_y);
            const int y = ty * th + (r >> a.tw_log2), x = tx * tw + (r & (tw - 1));
            const size_t pix = ((size_t)b * a.H + y) * a.W + x;
            const uint32_t tbase = tmem + buf * kT * BN + (uint32_t)(t * BN) + ((uint32_t)(q * 32) << 16);
            float hz = e.head_out ? e.head_b[0] : 0.0f;
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 16) {
                uint32_t v[16];
                tmem_ld16(tbase + (uint32_t)c0, v);
                float f[16];
                const int col = n0 + c0;
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    float t = __uint_as_float(v[j]);
                    if (e.bias) t += s_bias[col + j];
                    if (e.relu) t = fmaxf(t, 0.0f);
                    f[j] = t;
                }
                if (e.head_out)
#pragma unroll
                    for (int j = 0; j < 16; ++j) hz += __bfloat162float(__float2bfloat16_rn(f[j])) * e.head_w[col + j];
                const size_t o = pix * e.ldc + col;
                if (e.c16) {
                    uint4 out[2];
                    __nv_bfloat16* ob = reinterpret_cast<__nv_bfloat16*>(out);
#pragma unroll
                    for (int j = 0; j < 16; ++j) ob[j] = __float2bfloat16_rn(f[j]);
                    uint4* d4 = reinterpret_cast<uint4*>(e.c16 + o);
                    d4[0] = out[0];
                    d4[1] = out[1];
                    if (a.up16) {
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const size_t up = ((size_t)b * 2 * a.H + 2 * y + (u >> 1)) * (2 * a.W) + 2 * x + (u & 1);
                            uint4* d = reinterpret_cast<uint4*>(a.up16 + up * e.ldc + col);
                            d[0] = out[0];
                            d[1] = out[1];
                        }
                    }
                }
                if (e.c32) {
                    float4* d4 = reinterpret_cast<float4*>(e.c32 + o);
#pragma unroll
                    for (int h = 0; h < 4; ++h) d4[h] = make_float4(f[4 * h], f[4 * h + 1], f[4 * h + 2], f[4 * h + 3]);
                }
            }
            if (e.head_out) e.head_out[pix] = 1.0f / (1.0f + __expf(-hz));
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(acc_empty(buf));
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
}


// ------------------------------------------------------------------ implicit 3x3, row ring
// For 128-pixel tiles of one image row (W % 128 == 0) and a layer whose whole weight matrix
// fits in shared memory. A work item is a strip of 128 pixels (x0 .. x0 + 127) over a chunk
// of output rows [y0, y1); the CTA loads the chunk's input rows y0 - 1 .. y1 one at a time,
// each as ONE TMA box per source holding 136 pixels (x0 - 1 .. x0 + 134) of every input
// channel, into a ring of row slots. Output row y reads the slots of rows y - 1, y, y + 1
// in place, each tap's A operand starting 16 bytes (one pixel) further along its row: every
// input row crosses from L2 once per chunk instead of three times. Layouts are the
// no-swizzle K-major canonical form: 8 rows x 16 bytes (8 channels) per core matrix, core
// matrices 128 bytes apart along M (pixels) and one channel group apart along K (136 x 16
// bytes for A, N x 16 bytes for B). The weights are loaded once per CTA. K order (tap
// outermost, then channel) and the K16 steps are tc_conv_kernel's, so the two kernels give
// identical results.
constexpr int kHaloW = 136;                        // box width: 128 + 2 halo, rounded for alignment
constexpr uint32_t kHaloGroup = kHaloW * 16;       // bytes of one 8-channel group of a row slot

__device__ __forceinline__ uint64_t desc_plain(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;      // leading byte offset: next core matrix along K
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;      // stride byte offset: next 8 rows along M / N
    d |= (uint64_t)1 << 46;                           // descriptor version; layout 0: no swizzle
    return d;
}
__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, int c4,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}

// tcgen05.cp of a 128-row x 256-bit matrix (128 pixels x 16 BF16 channels, K-major, the
// descriptor's canonical layout) from shared memory into TMEM columns [taddr, taddr + 8).
__device__ __forceinline__ void tc_cp_128x256b(uint32_t taddr, uint64_t sdesc) {
    asm volatile("tcgen05.cp.cta_group::1.128x256b [%0], %1;" ::"r"(taddr), "l"(sdesc) : "memory");
}
// tcgen05.mma.kind::f16 with the A operand read from TMEM (128 lanes = M rows, K in columns).
__device__ __forceinline__ void tc_mma_ta(uint32_t tmem_d, uint32_t tmem_a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n" ::"r"(tmem_d),
        "r"(tmem_a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
// The A operands of one input row kept in TMEM (kTA): its three horizontal taps (the row
// shifted by -1, 0, +1 pixel) x the K steps of its channels, 8 columns each, in a ring of
// kTaSlots rows after the two accumulators. Each input row is copied from its shared-memory
// slot once and read by the three output rows that need it, so shared memory serves the A
// operand once per input row instead of once per tap of every output row; the MMAs then
// read only the weights (B) from shared memory.
constexpr int kTaSlots = 4;
constexpr uint32_t kTaRowCols = 3 * 2 * 8;         // taps x K steps (at most 32 channels) x 8 columns

struct HaloArgs {
    int nsrc, C0, C1, cin;
    int B, H, W;
    int chunk, chunks_y;        // output rows per work item; items per strip column
    int items;                  // n_slices x slice_items
    int n_slices, slice_items;  // output-channel slices of BN (fan-out; else 1) and items per slice,
                                // (W / 128) x chunks_y x B
    int stages;                 // row slots in the ring (>= 4; fan-out >= 2)
    uint32_t a_bytes, b_bytes;  // one row slot (all sources), the resident weights
    __nv_bfloat16* up16;
};

// Work item -> (output-channel slice, image, strip, first row, rows). The slices of one strip
// chunk are consecutive items: with a grid that is a multiple of the slice count every CTA
// keeps one slice (its weights load once), and the CTAs that hold a chunk's slices read its
// input rows at about the same time, so the second read finds them in L2.
struct HaloItem { int slice, b, tx, y0, rows; };
__device__ __forceinline__ HaloItem halo_item(const HaloArgs& a, int item) {
    const int tiles_x = a.W >> 7;
    HaloItem it;
    it.slice = item % a.n_slices;
    item /= a.n_slices;
    it.tx = item % tiles_x;
    const int c = (item / tiles_x) % a.chunks_y;
    it.b = item / (tiles_x * a.chunks_y);
    it.y0 = c * a.chunk;
    it.rows = min(a.chunk, a.H - it.y0);
    return it;
}

// Fan-out (kFan): the MMAs follow the input rows instead of the output rows. Input row r is
// read by output rows r + 1, r and r - 1 (vertical taps 0, 1, 2), so one MMA of N = 3 x BN
// (A: the row shifted by dx, K16 channels; B: the three vertical taps' weights stacked along
// N) adds its products to all three rows' accumulators at once. An output row's accumulator
// lives in a ring of kAcc = 256 / BN TMEM slots, ring index i at columns (kAcc - 1 - i % kAcc)
// x BN: ascending columns hold descending rows, so the three rows r + 1, r, r - 1 sit in
// ascending columns and their taps 0, 1, 2 in ascending B rows (where the ring wraps, the MMA
// splits in two). The weights are staged as [dx][channel group][dy][n][8 channels] by a 5-D
// box. Per output row the K16 steps still run tap by tap (dy, then dx) and channel by channel
// within a tap, as in the row-by-row MMAs; the accumulators start at zero (the epilogue warps
// clear each one after reading it, and the whole ring at the start) and every MMA adds, so
// both forms give the same values (0 + x = x; at most the sign of an all-zero sum differs).
// Each row slot in shared memory is read by the MMAs of its own input row only; the row's A
// operand crosses from shared memory three times (dx) instead of nine.
constexpr int kFanMaxAcc = 8;   // accumulator slots (BN 32: 8; BN 64: 4)
constexpr int kFanCases = 6;    // which of a load's three output rows exist
// Fan-out accumulator ring and residency: 256 TMEM columns (eight rows' accumulators at BN
// 32, four at BN 64) and two CTAs per SM. Three CTAs of a four-row ring at BN 32 (128
// columns, 96 registers) measured slower on every layer (32 -> 32 at 1088 x 1920: 94.0 us
// against 88.7).
__host__ __device__ constexpr int fan_acc(int bn) { return 256 / bn; }
__host__ __device__ constexpr int fan_ctas(int bn) { return 2; }
// The MMAs of one K16 step of one load in fan-out form: n pieces (two where the accumulator
// ring wraps), each (accumulator address, instruction descriptor, B offset in 16-byte units).
struct FanPlan { uint4 p[2]; int n, pad0, pad1, pad2; };
// Static shared memory of tc_conv_halo_kernel<BN>, rounded up: the bias (512 floats), the
// abort flag, the epilogue's stage (4 warps x 32 pixels x BN BF16 channels) and the fan-out
// MMA plans.
__host__ __device__ constexpr size_t halo_static_smem(int bn) {
    return 2048 + 64 + (size_t)4 * 32 * bn * 2 + sizeof(FanPlan) * kFanCases * kFanMaxAcc;
}

template <int BN, bool kTA, bool kFan>
__global__ void __launch_bounds__(kConvThreads, kFan ? fan_ctas(BN) : 1) tc_conv_halo_kernel(const __grid_constant__ CUtensorMap map0,
                                                                       const __grid_constant__ CUtensorMap map1,
                                                                       const __grid_constant__ CUtensorMap mapW,
                                                                       const HaloArgs a, const Epilogue e) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    // TMEM: kAcc accumulators (the MMAs of a row run while the previous row is in the
    // epilogue; four measured no faster), then (kTA) the ring of input rows' A operands; a
    // power of two. Fan-out: a ring of 256 / BN accumulators.
    static_assert(!(kTA && kFan), "one form at a time");
    static_assert(!kFan || (3 * BN <= 256 && 256 / BN <= kFanMaxAcc), "three rows' accumulators in one MMA");
    constexpr uint32_t kAcc = kFan ? (uint32_t)fan_acc(BN) : 2u;
    constexpr uint32_t kCols = (kTA || kFan) ? 256u : kAcc * BN;
    static_assert(!kTA || 2 * BN + kTaSlots * kTaRowCols <= 256, "the TMEM ring fits");
    const int kSt = a.stages;
    uint8_t* sB = smem;
    uint8_t* sA = smem + ((a.b_bytes + 1023) & ~1023u);
    const uint32_t a_stride = (a.a_bytes + 1023) & ~1023u;
    // full[kSt], empty[kSt], acc_full[8], acc_empty[8], w (weights landed), wfree (the weights'
    // last MMAs done: a slice's weights may be replaced)
    uint64_t* bars = reinterpret_cast<uint64_t*>(sA + kSt * a_stride);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kSt + 2 * kFanMaxAcc + 2);
    __shared__ int s_abort;
    __shared__ float s_bias[512];       // the bias of every output channel, staged once
    __shared__ FanPlan s_fan[kFanCases][kFanMaxAcc];
    volatile int* abort_flag = &s_abort;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    auto full = [&](int s) { return smem_u32(&bars[s]); };
    auto empty = [&](int s) { return smem_u32(&bars[kSt + s]); };
    auto acc_full = [&](int b) { return smem_u32(&bars[2 * kSt + b]); };
    auto acc_empty = [&](int b) { return smem_u32(&bars[2 * kSt + kFanMaxAcc + b]); };
    const uint32_t wbar = smem_u32(&bars[2 * kSt + 2 * kFanMaxAcc]);
    const uint32_t wfree = smem_u32(&bars[2 * kSt + 2 * kFanMaxAcc + 1]);
    // first TMEM column of the accumulator of output row i (counted over the CTA's items)
    auto acc_col = [&](uint32_t i) -> uint32_t { return kFan ? (kAcc - 1u - i % kAcc) * BN : (i % kAcc) * BN; };

    if (threadIdx.x == 0) {
        for (int s = 0; s < kSt; ++s) { mbar_init(full(s), 1); mbar_init(empty(s), 1); }
        for (int b = 0; b < (int)kAcc; ++b) { mbar_init(acc_full(b), 1); mbar_init(acc_empty(b), 4); }
        mbar_init(wbar, 1);
        mbar_init(wfree, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    if (e.bias)
        for (int i = threadIdx.x; i < a.n_slices * BN; i += blockDim.x) s_bias[i] = e.bias[i];
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
    const uint32_t src1_off = (uint32_t)(a.C0 / 8) * kHaloGroup;
    if (kFan) {
        // fan-out accumulators start at zero and every MMA adds to them: each epilogue warp
        // clears its lane quarter of the ring now and of each row again once it has read it
        if (warp >= 2)
            for (uint32_t c = 0; c < kCols; c += 32) tmem_zero32(tmem + c + ((uint32_t)((warp & 3) * 32) << 16));
        tmem_wait_st();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    }

    if (warp == 0) {
        if (lane == 0) {
            // loads in ring order: item by item, input rows y0 - 1 .. y0 + rows
            // the weights of the first item's slice; a later slice's replace them once the MMA
            // thread reports the last MMAs that read them done (wfree)
            int wslice = (int)blockIdx.x % a.n_slices;
            uint32_t wfree_ph = 0;
            mbar_expect_tx(wbar, a.b_bytes);
            if (kFan) tma_load_5d(smem_u32(sB), &mapW, 0, wslice * BN, 0, 0, 0, wbar);
            else tma_load_3d(smem_u32(sB), &mapW, 0, 0, 0, wbar);
            // kc counts loads; s and ph are its ring slot and the slot's phase (kc % kSt and
            // kc / kSt mod 2, kept by increment: kSt is a launch argument, and a division per
            // load would sit on this thread's path)
            uint32_t kc = 0, ph = 0;
            int s = 0;
            for (int item = blockIdx.x; item < a.items && !*abort_flag; item += gridDim.x) {
                const HaloItem it = halo_item(a, item);
                if (kFan && it.slice != wslice) {
                    if (!mbar_wait_or_abort(wfree, wfree_ph, abort_flag)) {
                        atomicOr(e.err, DEV_GUARD);
                        s_abort = 1;
                        break;
                    }
                    wfree_ph ^= 1u;
                    wslice = it.slice;
                    mbar_expect_tx(wbar, a.b_bytes);
                    tma_load_5d(smem_u32(sB), &mapW, 0, wslice * BN, 0, 0, 0, wbar);
                }
                for (int r = -1; r <= it.rows && !*abort_flag; ++r, ++kc) {
                    if (!mbar_wait_or_abort(empty(s), ph ^ 1u, abort_flag)) {
                        atomicOr(e.err, DEV_GUARD);
                        s_abort = 1;
                        break;
                    }
                    mbar_expect_tx(full(s), a.a_bytes);
                    const uint32_t dst = smem_u32(sA + s * a_stride);
                    tma_load_5d(dst, &map0, 0, it.tx * 128 - 1, it.y0 + r, it.b, 0, full(s));
                    if (a.nsrc > 1) tma_load_5d(dst + src1_off, &map1, 0, it.tx * 128 - 1, it.y0 + r, it.b, 0, full(s));
                    if (++s == kSt) { s = 0; ph ^= 1u; }
                }
            }
            // the copies this lane issued must land before the CTA can leave
            for (uint32_t k = kc > (uint32_t)kSt ? kc - kSt : 0; k < kc; ++k) mbar_wait(full(k % kSt), (k / kSt) & 1u);
            mbar_wait(wbar, wfree_ph);      // the last weights load (one more than the reloads)
        }
    } else if (warp == 1 && kFan) {
        // The MMAs of a load depend only on which of its three output rows exist (the load's
        // case: lo = max(0, k - 2) - k and hi = min(rows - 1, k) - k, six cases) and on the
        // ring residue of its row k, so the warp tabulates them once: per case and residue the
        // one or two pieces (two where the ring wraps) of every K16 step, each an accumulator
        // address, an instruction descriptor (N) and the offset of its first B row (vertical
        // tap k - h for its top row h, in 16-byte units). The issuing thread then spends two
        // shared loads per load instead of forming pieces: it is blocked while the tensor
        // pipe takes each MMA, so its other work adds directly to the layer's time.
        for (int e_ = lane; e_ < kFanCases * (int)kAcc; e_ += 32) {
            const int cs = e_ / (int)kAcc, r = e_ % (int)kAcc;
            const int lo = cs == 0 ? 0 : cs <= 2 ? -1 : -2;                       // relative to k
            const int hi = cs == 0 || cs == 1 || cs == 3 ? 0 : cs == 2 || cs == 4 ? -1 : -2;
            // ring index of row k + x is r + x (mod kAcc); the piece holding the top row first
            FanPlan& pl = s_fan[cs][r];
            int n = 0;
            for (int h = hi; h >= lo;) {
                const uint32_t ih = (uint32_t)(r + h + (int)kAcc) % kAcc;
                const int b = max(lo, h - (int)ih);
                pl.p[n++] = make_uint4(tmem + (kAcc - 1u - ih) * BN, instr_desc((h - b + 1) * BN), (uint32_t)(-h * BN), 0u);
                h = b - 1;
            }
            pl.n = n;
        }
        __syncwarp();
        if (lane == 0) {
            const int q16 = a.cin / 16, G = a.cin / 8;
            const uint32_t b_grp = 3u * BN * 16u;                         // next channel group of B (LBO)
            const uint64_t db0 = desc_plain(smem_u32(sB), b_grp, 128);
            const uint64_t dq_a = (2u * kHaloGroup) >> 4;                 // the next 16 channels of A
            const uint64_t dq_b = (2u * b_grp) >> 4;                      // ... of B
            const uint64_t dx_b = ((uint32_t)G * b_grp) >> 4;             // the next horizontal tap of B
            bool ok = mbar_wait_or_abort(wbar, 0, abort_flag);
            int wslice = (int)blockIdx.x % a.n_slices;
            uint32_t w_ph = 0;
            uint32_t i0 = 0;            // output rows of earlier items
            // the current load's ring slot, its phase and its shared-memory row (kept by increment)
            int slot = 0;
            uint32_t phase = 0, row_smem = smem_u32(sA);
            // Descriptors are affine in their address (the 14-bit field holds address / 16, and
            // no offset here carries out of it): every MMA is a base descriptor plus a constant.
            for (int item = blockIdx.x; ok && item < a.items && !*abort_flag; item += gridDim.x) {
                const HaloItem it = halo_item(a, item);
                if (it.slice != wslice) {
                    // the next slice's weights: once this slice's MMAs have read theirs
                    tc_commit(wfree);
                    w_ph ^= 1u;
                    if (!mbar_wait_or_abort(wbar, w_ph, abort_flag)) { ok = false; break; }
                    wslice = it.slice;
                }
                // load k is input row y0 - 1 + k; it feeds output rows k - 2 .. k of the item
                for (int k = 0; ok && k <= it.rows + 1; ++k) {
                    const int lo = max(0, k - 2) - k, hi = min(it.rows - 1, k) - k;
                    const int cs = -lo * (1 - lo) / 2 - hi;               // (0,0) 0; (-1,0) 1; (-1,-1) 2; (-2,0) 3; ...
                    const FanPlan& pl = s_fan[cs][(i0 + (uint32_t)k) % kAcc];
                    const uint4 c0 = pl.p[0], c1 = pl.p[1];
                    const int nc = pl.n;
                    if (hi == 0) {
                        // output row k's first load: its accumulator must be free
                        const uint32_t i = i0 + (uint32_t)k;
                        if (!mbar_wait_or_abort(acc_empty(i % kAcc), ((i / kAcc) & 1u) ^ 1u, abort_flag)) {
                            ok = false;
                            break;
                        }
                    }
                    if (!mbar_wait_or_abort(full(slot), phase, abort_flag)) { ok = false; break; }
                    tc_fence_after();
                    const uint64_t da_row = desc_plain(row_smem, kHaloGroup, 128);
#pragma unroll
                    for (int dx = 0; dx < 3; ++dx) {
                        uint64_t da = da_row + (uint64_t)dx;                      // one pixel: 16 bytes
                        uint64_t db = db0 + (uint64_t)dx * dx_b;
                        for (int q = 0; q < q16; ++q) {
                            tc_mma(c0.x, da, db + c0.z, c0.y, 1u);
                            if (nc > 1) tc_mma(c1.x, da, db + c1.z, c1.y, 1u);
                            da += dq_a;
                            db += dq_b;
                        }
                    }
                    // the row slot is free once its MMAs have read it; output row k - 2 is complete
                    tc_commit(empty(slot));
                    if (k >= 2) tc_commit(acc_full((i0 + (uint32_t)(k - 2)) % kAcc));
                    if (++slot == kSt) {
                        slot = 0;
                        phase ^= 1u;
                        row_smem = smem_u32(sA);
                    } else {
                        row_smem += a_stride;
                    }
                }
                if (!ok) break;
                i0 += (uint32_t)it.rows;
            }
            if (!ok) {
                atomicOr(e.err, DEV_GUARD);
                s_abort = 1;
            }
        }
    } else if (warp == 1 && kTA) {
        if (lane == 0) {
            const uint32_t idesc = instr_desc(BN);
            const uint32_t b0 = smem_u32(sB);
            const int q16 = a.cin / 16, g_tap = a.cin / 8;
            const uint32_t ta0 = tmem + 2u * BN;
            bool ok = mbar_wait_or_abort(wbar, 0, abort_flag);
            uint32_t base = 0, i = 0;   // ring index of the item's first load; output rows so far
            for (int item = blockIdx.x; ok && item < a.items && !*abort_flag; item += gridDim.x) {
                const HaloItem it = halo_item(a, item);
                for (int j = 0; ok && j < it.rows; ++j, ++i) {
                    // output row y0 + j reads loads j, j + 1, j + 2 of the item
                    const uint32_t buf = i % kAcc, use = i / kAcc;
                    // row i - 2's MMAs are done once its accumulator is free again: the TMEM
                    // slots they read may be overwritten
                    if (!mbar_wait_or_abort(acc_empty(buf), (use & 1u) ^ 1u, abort_flag)) { ok = false; break; }
                    if (j == 0 && i > 0) {
                        // a new item reloads three rows: the previous row's MMAs must be done too
                        const uint32_t pi = i - 1;
                        if (!mbar_wait_or_abort(acc_full(pi % kAcc), (pi / kAcc) & 1u, abort_flag)) { ok = false; break; }
                    }
                    for (int d = (j == 0 ? 0 : 2); d < 3 && ok; ++d) {
                        const uint32_t k = base + (uint32_t)(j + d);
                        ok = mbar_wait_or_abort(full(k % kSt), (k / kSt) & 1u, abort_flag);
                        if (!ok) break;
                        tc_fence_after();
                        const uint32_t row = smem_u32(sA + (k % kSt) * a_stride);
                        const uint32_t slot = ta0 + (k % kTaSlots) * kTaRowCols;
                        for (int dx = 0; dx < 3; ++dx)
                            for (int q = 0; q < q16; ++q)
                                tc_cp_128x256b(slot + (uint32_t)(dx * q16 + q) * 8u,
                                               desc_plain(row + (uint32_t)dx * 16u + (uint32_t)(2 * q) * kHaloGroup,
                                                          kHaloGroup, 128));
                        // the shared-memory slot is free once its copies have run
                        tc_commit(empty(k % kSt));
                    }
                    if (!ok) break;
                    const uint32_t acc = tmem + buf * BN;
                    for (int t = 0; t < 9; ++t) {
                        const uint32_t k = base + (uint32_t)(j + t / 3);
                        const uint32_t slot = ta0 + (k % kTaSlots) * kTaRowCols + (uint32_t)((t % 3) * q16) * 8u;
                        for (int q = 0; q < q16; ++q) {
                            const uint64_t db = desc_plain(b0 + (uint32_t)(t * g_tap + 2 * q) * (BN * 16), BN * 16, 128);
                            tc_mma_ta(acc, slot + (uint32_t)q * 8u, db, idesc, (t | q) != 0 ? 1u : 0u);
                        }
                    }
                    tc_commit(acc_full(buf));
                }
                if (!ok) break;
                base += (uint32_t)it.rows + 2;
            }
            if (!ok) {
                atomicOr(e.err, DEV_GUARD);
                s_abort = 1;
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = instr_desc(BN);
            const int q16 = a.cin / 16, g_tap = a.cin / 8;
            const uint64_t db0 = desc_plain(smem_u32(sB), BN * 16, 128);
            const uint64_t dq_a = (2u * kHaloGroup) >> 4;                 // the next 16 channels of A
            const uint64_t dq_b = (2u * BN * 16u) >> 4;                   // ... of B
            const uint64_t dtap_b = ((uint32_t)g_tap * BN * 16u) >> 4;    // the next tap of B
            bool ok = mbar_wait_or_abort(wbar, 0, abort_flag);
            uint32_t base = 0, i = 0;   // ring index of the item's first load; output rows so far
            for (int item = blockIdx.x; ok && item < a.items && !*abort_flag; item += gridDim.x) {
                const HaloItem it = halo_item(a, item);
                for (int j = 0; ok && j < it.rows; ++j, ++i) {
                    // output row y0 + j reads loads j, j + 1, j + 2 of the item
                    const uint32_t buf = i % kAcc, use = i / kAcc;
                    if (!mbar_wait_or_abort(acc_empty(buf), (use & 1u) ^ 1u, abort_flag)) { ok = false; break; }
                    uint32_t row_addr[3];
                    for (int d = 0; d < 3 && ok; ++d) {
                        const uint32_t k = base + (uint32_t)(j + d);
                        ok = mbar_wait_or_abort(full(k % kSt), (k / kSt) & 1u, abort_flag);
                        row_addr[d] = smem_u32(sA + (k % kSt) * a_stride);
                    }
                    if (!ok) break;
                    tc_fence_after();
                    const uint32_t acc = tmem + buf * BN;
                    // a descriptor is affine in its address (the 14-bit field holds address / 16
                    // and no offset here carries out of it): each MMA's operands are the row's or
                    // the weights' base descriptor plus a constant, so the issuing thread spends
                    // a few instructions per MMA instead of forming two descriptors
                    const uint64_t da_row[3] = {desc_plain(row_addr[0], kHaloGroup, 128),
                                                desc_plain(row_addr[1], kHaloGroup, 128),
                                                desc_plain(row_addr[2], kHaloGroup, 128)};
                    uint64_t db_tap = db0;
#pragma unroll
                    for (int t = 0; t < 9; ++t) {
                        uint64_t da = da_row[t / 3] + (uint64_t)(t % 3);        // one pixel: 16 bytes
                        uint64_t db = db_tap;
                        for (int q = 0; q < q16; ++q) {
                            tc_mma(acc, da, db, idesc, (t | q) != 0 ? 1u : 0u);
                            da += dq_a;
                            db += dq_b;
                        }
                        db_tap += dtap_b;
                    }
                    tc_commit(acc_full(buf));
                    // load j (input row y0 + j - 1) has no later reader
                    tc_commit(empty((base + (uint32_t)j) % kSt));
                }
                if (!ok) break;
                // the item's last two loads
                tc_commit(empty((base + (uint32_t)it.rows) % kSt));
                tc_commit(empty((base + (uint32_t)it.rows + 1) % kSt));
                base += (uint32_t)it.rows + 2;
            }
            if (!ok) {
                atomicOr(e.err, DEV_GUARD);
                s_abort = 1;
            }
        }
    } else {
        const int q = warp & 3;
        const int r = q * 32 + lane;
        // BF16 outputs pass through shared memory: a lane converts its pixel's BN channels
        // into 16-byte chunks of its warp's stage, then the warp stores the stage's 32 pixels
        // as whole 512-byte runs (16 contiguous bytes a lane) instead of one 16-byte piece a
        // lane 2 x BN bytes apart. Chunk c of pixel p sits at slot p kCh + (c ^ swz(p)): a
        // quarter-warp's eight 16-byte accesses then fall in eight different bank groups
        // both when lanes write their own pixels and when they read consecutive chunks.
        constexpr int kCh = BN / 8;
        __shared__ __align__(16) uint4 s_stage[4][32 * kCh];
        uint4* stage = s_stage[q];
        auto slot = [](int p, int c) { return p * kCh + (c ^ ((kCh == 4 ? (p >> 1) : p) & (kCh - 1))); };
        uint32_t i = 0;
        bool ok = true;
        for (int item = blockIdx.x; ok && item < a.items; item += gridDim.x) {
            const HaloItem it = halo_item(a, item);
            for (int j = 0; j < it.rows; ++j, ++i) {
                const uint32_t buf = i % kAcc, use = i / kAcc;
                ok = __all_sync(0xffffffffu, mbar_wait_or_abort(acc_full(buf), use & 1u, abort_flag));
                if (!ok) {
                    if (lane == 0) { atomicOr(e.err, DEV_GUARD); s_abort = 1; }
                    break;
                }
                tc_fence_after();
                const int y = it.y0 + j, x = it.tx * 128 + r;
                const size_t pix = ((size_t)it.b * a.H + y) * a.W + x;
                const uint32_t tbase = tmem + acc_col(i) + ((uint32_t)(q * 32) << 16);
                const int n0 = it.slice * BN;                  // the item's first output channel
                float hz = e.head_out ? e.head_b[0] : 0.0f;
                // the row's BN columns in one TMEM load and one wait
                uint32_t vv[BN];
                if constexpr (BN == 64) tmem_ld64(tbase, vv);
                else tmem_ld32(tbase, vv);
                if (kFan)                                      // the row's next use starts from zero
#pragma unroll
                    for (int c32 = 0; c32 < BN; c32 += 32) tmem_zero32(tbase + (uint32_t)c32);
#pragma unroll
                for (int c0 = 0; c0 < BN; c0 += 16) {
                    const uint32_t* v = vv + c0;
                    float f[16];
#pragma unroll
                    for (int jj = 0; jj < 16; ++jj) {
                        float t = __uint_as_float(v[jj]);
                        if (e.bias) t += s_bias[n0 + c0 + jj];
                        if (e.relu) t = fmaxf(t, 0.0f);
                        f[jj] = t;
                    }
                    if (e.head_out)
#pragma unroll
                        for (int jj = 0; jj < 16; ++jj)
                            hz += __bfloat162float(__float2bfloat16_rn(f[jj])) * e.head_w[c0 + jj];
                    const size_t o = pix * e.ldc + n0 + c0;
                    if (e.c16) {
                        uint4 out[2];
                        __nv_bfloat16* ob = reinterpret_cast<__nv_bfloat16*>(out);
#pragma unroll
                        for (int jj = 0; jj < 16; ++jj) ob[jj] = __float2bfloat16_rn(f[jj]);
                        stage[slot(lane, c0 / 8)] = out[0];
                        stage[slot(lane, c0 / 8 + 1)] = out[1];
                    }
                    if (e.c32) {
                        float4* d4 = reinterpret_cast<float4*>(e.c32 + o);
#pragma unroll
                        for (int h = 0; h < 4; ++h) d4[h] = make_float4(f[4 * h], f[4 * h + 1], f[4 * h + 2], f[4 * h + 3]);
                    }
                }
                if (e.head_out) e.head_out[pix] = 1.0f / (1.0f + __expf(-hz));
                if (kFan) tmem_wait_st();
                tc_fence_before();
                __syncwarp();
                // the accumulator is read (and, fan-out, cleared): the MMAs may refill it while
                // the warp stores
                if (lane == 0) mbar_arrive(acc_empty(buf));
                if (e.c16) {
                    const size_t pix0 = pix - lane;                       // the warp's first pixel
#pragma unroll 1
                    for (int k = 0; k < kCh; ++k) {
                        const int idx = k * 32 + lane, p = idx / kCh, c = idx % kCh;
                        *reinterpret_cast<uint4*>(e.c16 + (pix0 + p) * e.ldc + n0 + c * 8) = stage[slot(p, c)];
                    }
                    if (a.up16) {
                        // rows 2y and 2y + 1 of the 2x copy: 64 pixels, each source pixel twice
                        const size_t up0 = ((size_t)it.b * 2 * a.H + 2 * y) * (2 * a.W) + 2 * (x - lane);
#pragma unroll 1
                        for (int k = 0; k < 2 * kCh; ++k) {
                            const int idx = k * 32 + lane, P = idx / kCh, c = idx % kCh;
                            const uint4 v = stage[slot(P >> 1, c)];
                            *reinterpret_cast<uint4*>(a.up16 + (up0 + P) * e.ldc + n0 + c * 8) = v;
                            *reinterpret_cast<uint4*>(a.up16 + (up0 + 2 * a.W + P) * e.ldc + n0 + c * 8) = v;
                        }
                    }
                    __syncwarp();                                         // the stage is free again
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


// A 2-D weight map [rows][ld] read in boxes of cb x box_rows (128- or 64-byte swizzle).
bool make_map_cb(CUtensorMap* m, const void* base, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows, int cb) {
    auto fn = encoder();
    if (!fn) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)cb, box_rows};
    const cuuint32_t elem[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, elem,
              CU_TENSOR_MAP_INTERLEAVE_NONE, cb == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// A 4-D map of an NHWC BF16 tensor [B][H][W][C], boxes of cb x tw x th x 1; coordinates
// outside the tensor read zeros (the convolution's padding).
bool make_map_nhwc(CUtensorMap* m, const void* base, int B, int H, int W, int C, int tw, int th, int cb) {
    auto fn = encoder();
    if (!fn) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
    const cuuint32_t box[4] = {(cuuint32_t)cb, (cuuint32_t)tw, (cuuint32_t)th, 1};
    const cuuint32_t elem[4] = {1, 1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, elem,
              CU_TENSOR_MAP_INTERLEAVE_NONE, cb == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN, int CB, int kT>
int launch_conv(const CUtensorMap& m0, const CUtensorMap& m1, const CUtensorMap& mw, const ConvArgs& a,
                const Epilogue& e, cudaStream_t s) {
    constexpr int kSt = conv_stages<BN, CB, kT>();
    const size_t smem = 1024 + kSt * (kT * kBM * CB * 2 + BN * CB * 2) + (2 * kSt + 4) * 8 + 16;
    static int per_sm = 0;
    if (!per_sm) {
        if (cudaFuncSetAttribute(tc_conv_kernel<BN, CB, kT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
                cudaSuccess ||
            cudaFuncSetAttribute(tc_conv_kernel<BN, CB, kT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared) != cudaSuccess)
            return RN_ERR_CUDA;
        // residency: shared memory (228 KB per SM, 1 KB reserved per CTA), TMEM (512 columns per
        // SM, 2 x BN per CTA) and at most 3 CTAs of 192 threads and 88 registers
        int smem_sm = 0;
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx().device);
        const int by_smem = smem_sm / (int)(smem + 1024);
        per_sm = std::max(1, std::min(std::min(by_smem, 512 / (2 * kT * BN)), 3));
    }
    const int ctas = std::min(a.items, per_sm * ctx().sm_count);
    tc_conv_kernel<BN, CB, kT><<<ctas, kConvThreads, smem, s>>>(m0, m1, mw, a, e);
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}


// The row box of one source: a 5-D view of the NHWC tensor, (8 channels, W, H, B, C / 8
// groups), read in boxes of 8 x 136 x 1 x 1 x C/8 without swizzle (the channel groups
// outermost in shared memory).
bool make_map_halo(CUtensorMap* m, const void* base, int B, int H, int W, int C) {
    auto fn = encoder();
    if (!fn) return false;
    const cuuint64_t dims[5] = {8, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B, (cuuint64_t)(C / 8)};
    const cuuint64_t strides[4] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2, 16};
    const cuuint32_t box[5] = {8, (cuuint32_t)kHaloW, 1, 1, (cuuint32_t)(C / 8)};
    const cuuint32_t elem[5] = {1, 1, 1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(base), dims, strides, box, elem,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
// The resident weights: (8 columns, N rows, K / 8 groups), one box of 8 x N x kgroups.
bool make_map_wgroups(CUtensorMap* m, const void* base, int N, int ldw, int kgroups) {
    auto fn = encoder();
    if (!fn) return false;
    const cuuint64_t dims[3] = {8, (cuuint64_t)N, (cuuint64_t)(ldw / 8)};
    const cuuint64_t strides[2] = {(cuuint64_t)ldw * 2, 16};
    const cuuint32_t box[3] = {8, (cuuint32_t)N, (cuuint32_t)kgroups};
    const cuuint32_t elem[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, elem,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The resident weights in the fan-out order: a 5-D view (8 columns, N rows, vertical tap dy,
// channel group, horizontal tap dx) of the [N][ldw] matrix whose column is
// (3 dy + dx) cin + channel, one box of a slice of bn rows: shared memory [dx][group][dy][n][8].
bool make_map_wfan(CUtensorMap* m, const void* base, int N, int ldw, int cin, int bn) {
    auto fn = encoder();
    if (!fn) return false;
    const cuuint64_t dims[5] = {8, (cuuint64_t)N, 3, (cuuint64_t)(cin / 8), 3};
    const cuuint64_t strides[4] = {(cuuint64_t)ldw * 2, (cuuint64_t)cin * 6, 16, (cuuint64_t)cin * 2};
    const cuuint32_t box[5] = {8, (cuuint32_t)bn, 3, (cuuint32_t)(cin / 8), 3};
    const cuuint32_t elem[5] = {1, 1, 1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(base), dims, strides, box, elem,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN, bool kTA, bool kFan>
int launch_conv_halo(const CUtensorMap& m0, const CUtensorMap& m1, const CUtensorMap& mw, const HaloArgs& a,
                     const Epilogue& e, size_t smem, cudaStream_t s) {
    static size_t attr = 0;
    if (attr < smem) {
        if (cudaFuncSetAttribute(tc_conv_halo_kernel<BN, kTA, kFan>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess ||
            cudaFuncSetAttribute(tc_conv_halo_kernel<BN, kTA, kFan>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared) != cudaSuccess)
            return RN_ERR_CUDA;
        attr = smem;
    }
    int smem_sm = 0;
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx().device);
    // co-resident CTAs: shared memory (dynamic, static and 1 KB reserved) and TMEM (512
    // columns an SM) both have to fit
    const int tmem_cols = kTA ? 256 : kFan ? fan_acc(BN) * BN : 2 * BN;
    const int per_cta = (int)(smem + halo_static_smem(BN) + 1024);
    const int per_sm = std::max(1, std::min(std::min(smem_sm / per_cta, 512 / tmem_cols), 3));
    const int ctas = std::min(a.items, per_sm * ctx().sm_count);
    tc_conv_halo_kernel<BN, kTA, kFan><<<ctas, kConvThreads, smem, s>>>(m0, m1, mw, a, e);
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}

ConvTiling conv_tiling(int H, int W) {
    ConvTiling t{0, false};
    if (H <= 0 || W <= 0) return t;
    int lg = 0;
    while (lg < 7 && (W % (2 << lg)) == 0) ++lg;            // TW = 2^lg <= 128 divides W
    const int th = kBM >> lg;
    t.tw_log2 = lg;
    t.ok = (H % th) == 0;
    return t;
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
    int bn = (N == 32 || N == 64 || N == 128 || N == 256) ? N : 128;
    if (N % bn) return fail(st, RN_ERR_INVALID, "tc_gemm N %d", N);
    while (bn > ctx().tune.conv_bn_max && bn > 32) bn /= 2;     // the tuned tile width (divides N)
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


int tc_conv3x3(const tc::ConvSrc* src, int nsrc, int B, int H, int W, const __nv_bfloat16* w, int ldw, int N,
               const tc::Epilogue& epi, __nv_bfloat16* up16, cudaStream_t s, rn_status* st) {
    if (nsrc < 1 || nsrc > 2 || !src) return fail(st, RN_ERR_INVALID, "tc_conv3x3: %d sources", nsrc);
    const tc::ConvTiling t = tc::conv_tiling(H, W);
    if (!t.ok || B <= 0) return fail(st, RN_ERR_INVALID, "tc_conv3x3: %dx%d cannot be tiled", H, W);
    int cin = 0;
    bool all64 = true, all32 = true;
    for (int i = 0; i < nsrc; ++i) {
        if (!src[i].ptr || src[i].C <= 0 || src[i].C % 16 || ((uintptr_t)src[i].ptr % 16))
            return fail(st, RN_ERR_INVALID, "tc_conv3x3: source %d (C %d)", i, src[i].C);
        all64 = all64 && src[i].C % 64 == 0;
        all32 = all32 && src[i].C % 32 == 0;
        cin += src[i].C;
    }
    if (ldw < 9 * cin || ldw % 8 || ((uintptr_t)w % 16)) return fail(st, RN_ERR_INVALID, "tc_conv3x3: weight stride %d", ldw);
    if (epi.atomic || epi.gate) return fail(st, RN_ERR_INVALID, "tc_conv3x3: no atomic or gated epilogue");
    if (epi.head_out && (N != 32 || !epi.head_w || !epi.head_b || up16))
        return fail(st, RN_ERR_INVALID, "tc_conv3x3: the fused head needs N 32, its weights and no upsampled copy");
    int bn = (N == 32 || N == 64 || N == 128 || N == 256) ? N : 128;
    if (N % bn || N > 512) return fail(st, RN_ERR_INVALID, "tc_conv3x3 N %d", N);
    while (bn > ctx().tune.conv_bn_max && bn > 32) bn /= 2;
    if (up16 && !epi.c16) return fail(st, RN_ERR_INVALID, "tc_conv3x3: the upsampled copy needs a BF16 output");
    // row-ring tiles: rows of 128 pixels, channels in groups of 16, the weights resident in
    // shared memory. Row by row (conv_fan 0, conv_tmem_a): N 32 or 64 in one slice and a ring of
    // at least four row slots. Fan-out (conv_fan 1): N 32 or 64 in one slice where that fits,
    // else slices of 32 output channels (N a multiple of 32 up to 512), at least two slots, and
    // two CTAs per SM where shared memory allows, one otherwise. Sources of 16 channels have
    // only this kernel (the per-tap boxes take 32 or 64 channels).
    const bool ta = ctx().tune.conv_tmem_a && N == 32 && cin <= 32;
    const bool fan = !ta && ctx().tune.conv_fan;
    const bool ring_shape = t.tw_log2 == 7 && (9 * cin) / 8 <= 256 && cin % 16 == 0;
    const bool one_slice = N == 32 || N == 64;
    if ((ctx().tune.conv_halo || !all32) && ring_shape && (one_slice || (fan && N % 32 == 0 && N <= 512))) {
        const uint32_t a_bytes = (uint32_t)cin / 8 * tc::kHaloGroup;
        const uint32_t a_stride = (a_bytes + 1023) & ~1023u;
        const size_t bars = (size_t)(2 * 8 + 2 * tc::kFanMaxAcc + 2) * 8 + 16;
        int bn = one_slice && (N == 32 || !fan || ctx().tune.conv_fan_bn == 64) ? N : 32, stages = 0;
        uint32_t b_bytes = 0, b_pad = 0;
        auto fit = [&](int bnf) {
            b_bytes = (uint32_t)bnf * 9 * cin * 2;
            b_pad = (b_bytes + 1023) & ~1023u;
            const size_t stat = tc::halo_static_smem(bnf);
            if (!fan) {
                // dynamic shared memory: 227 KB a block less the kernel's static arrays (the
                // bias, the abort flag and the epilogue's BF16 stage of 4 x 32 pixels x N)
                const size_t budget = 220 * 1024 - stat;
                return (int)std::min<size_t>(8, (budget - std::min<size_t>(budget, b_pad + 2048)) / a_stride);
            }
            // fan-out: a slot is busy only until its own MMAs have run: four at most (4, 6 and 8
            // measured alike); two CTAs per SM (228 KB less 1 KB reserved each) where two slots
            // fit, else one CTA with the whole 227 KB of a block
            const size_t fixed = stat + 1024 + bars + b_pad;
            for (const size_t cta : {(size_t)228 * 1024 / 2 - 1024, (size_t)227 * 1024}) {
                const size_t room = cta > fixed ? (cta - fixed) / a_stride : 0;
                if (room >= 2) return (int)std::min<size_t>(4, room);
            }
            return 0;
        };
        stages = fit(bn);
        if (fan && bn == 64 && stages < 2) {
            bn = 32;
            stages = fit(bn);
        }
        CUtensorMap hm[2], hw;
        bool maps = stages >= (fan ? 2 : 4) && (fan || one_slice);
        for (int i = 0; maps && i < nsrc; ++i) maps = tc::make_map_halo(&hm[i], src[i].ptr, B, H, W, src[i].C);
        if (maps && nsrc == 1) hm[1] = hm[0];
        maps = maps && (fan ? tc::make_map_wfan(&hw, w, N, ldw, cin, bn) : tc::make_map_wgroups(&hw, w, N, ldw, 9 * cin / 8));
        if (maps) {
            tc::HaloArgs h{};
            h.nsrc = nsrc; h.C0 = src[0].C; h.C1 = nsrc > 1 ? src[1].C : 0; h.cin = cin;
            h.B = B; h.H = H; h.W = W;
            // chunks of 16 output rows (2 halo rows re-read per chunk), fewer where that leaves
            // less than two items per SM
            h.chunk = 16;
            while (h.chunk > 4 && (long)(W / 128) * B * ((H + h.chunk - 1) / h.chunk) < 2L * ctx().sm_count) h.chunk /= 2;
            h.chunks_y = (H + h.chunk - 1) / h.chunk;
            h.n_slices = N / bn;
            h.slice_items = (W / 128) * h.chunks_y * B;
            h.items = h.n_slices * h.slice_items;
            h.stages = stages;
            h.a_bytes = a_bytes; h.b_bytes = b_bytes;
            h.up16 = up16;
            const size_t smem = 1024 + b_pad + (size_t)stages * a_stride + bars;
            const int rc = ta    ? tc::launch_conv_halo<32, true, false>(hm[0], hm[1], hw, h, epi, smem, s)
                         : fan   ? (bn == 32 ? tc::launch_conv_halo<32, false, true>(hm[0], hm[1], hw, h, epi, smem, s)
                                             : tc::launch_conv_halo<64, false, true>(hm[0], hm[1], hw, h, epi, smem, s))
                         : N == 32 ? tc::launch_conv_halo<32, false, false>(hm[0], hm[1], hw, h, epi, smem, s)
                                   : tc::launch_conv_halo<64, false, false>(hm[0], hm[1], hw, h, epi, smem, s);
            if (rc != RN_OK) return cuda_fail(st, cudaGetLastError(), "tc_conv_halo_kernel");
            return RN_OK;
        }
    }
    if (!all32)
        return fail(st, RN_ERR_INVALID, "tc_conv3x3: 16-channel sources need 128-pixel rows, N 32 or 64 and resident weights");
    const int cb = all64 ? 64 : 32;
    const int tw = 1 << t.tw_log2, th = tc::kBM >> t.tw_log2;
    CUtensorMap m[2], mw;
    for (int i = 0; i < nsrc; ++i)
        if (!tc::make_map_nhwc(&m[i], src[i].ptr, B, H, W, src[i].C, tw, th, cb))
            return fail(st, RN_ERR_CUDA, "cuTensorMapEncodeTiled (activation) failed");
    if (nsrc == 1) m[1] = m[0];
    if (!tc::make_map_cb(&mw, w, (uint64_t)N, (uint64_t)ldw, (uint64_t)ldw, (uint32_t)bn, cb))
        return fail(st, RN_ERR_CUDA, "cuTensorMapEncodeTiled (weights) failed");
    tc::ConvArgs a{};
    a.nsrc = nsrc;
    a.C0 = src[0].C;
    a.C1 = nsrc > 1 ? src[1].C : 0;
    a.B = B; a.H = H; a.W = W; a.tw_log2 = t.tw_log2;
    a.tiles_x = W / tw; a.tiles_y = H / th;
    a.cin = cin;
    a.n_slices = N / bn;
    // two tiles per item where the tile count is even, both accumulator pairs fit in TMEM and
    // the doubled A stages keep as many CTAs per SM as single tiles do
    const long tiles = (long)a.tiles_x * a.tiles_y * B;
    auto resident = [&](int kt) {
        const int st_n = (cb == 32 ? 8 : 4) / (kt == 2 && bn <= 64 ? 2 : 1);
        const int smem = 1024 + st_n * (kt * tc::kBM * cb * 2 + bn * cb * 2) + (2 * st_n + 4) * 8 + 16;
        int smem_sm = 0;
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx().device);
        return std::min(std::min(smem_sm / (smem + 1024), 512 / (2 * kt * bn)), 3);
    };
    const bool pair = ctx().tune.conv_pair && tiles % 2 == 0 && bn <= 128 && resident(2) >= std::max(1, resident(1));
    a.items = (int)(tiles / (pair ? 2 : 1)) * a.n_slices;
    a.up16 = up16;
    int rc;
#define RN_CONV_CASE(BNV, KT)                                                                         \
    case BNV:                                                                                         \
        rc = cb == 64 ? tc::launch_conv<BNV, 64, KT>(m[0], m[1], mw, a, epi, s)                       \
                      : tc::launch_conv<BNV, 32, KT>(m[0], m[1], mw, a, epi, s);                      \
        break;
    if (pair) {
        switch (bn) {
            RN_CONV_CASE(32, 2)
            RN_CONV_CASE(64, 2)
            default: RN_CONV_CASE(128, 2)
        }
    } else {
        switch (bn) {
            RN_CONV_CASE(32, 1)
            RN_CONV_CASE(64, 1)
            RN_CONV_CASE(256, 1)
            default: RN_CONV_CASE(128, 1)
        }
    }
#undef RN_CONV_CASE
    if (rc != RN_OK) return cuda_fail(st, cudaGetLastError(), "tc_conv_kernel");
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

// Test and measurement entry of the implicit 3x3 convolution (device pointers, NHWC BF16
// sources, the library's stream).
extern "C" int rn_tc_conv3x3(const void* src0, int c0, const void* src1, int c1, int B, int H, int W, const void* w,
                             int ldw, int N, float* c32, void* c16, void* up16, const float* bias, int relu,
                             rn_status* st) {
    RN_TRY(ensure_ctx(st));
    tc::ConvSrc src[2] = {{(const __nv_bfloat16*)src0, c0}, {(const __nv_bfloat16*)src1, c1}};
    tc::Epilogue e{};
    e.ldc = N;
    e.c32 = c32;
    e.c16 = (__nv_bfloat16*)c16;
    e.bias = bias;
    e.relu = relu;
    e.err = ctx().dev_error;
    RN_TRY(tc_conv3x3(src, src1 ? 2 : 1, B, H, W, (const __nv_bfloat16*)w, ldw, N, e, (__nv_bfloat16*)up16,
                      ctx().stream, st));
    return ok(st);
}

// Self-test of the device-side wait budget (no counterpart in the reference): a 128 x 32 x 64
// GEMM whose only K block's copies are withheld, so its stage never fills. The MMA thread's
// bounded wait gives up after `spin_limit` rounds, sets the error word and the CTA frees its
// TMEM and returns: the call must come back with RN_ERR_BUDGET and leave the context usable.
extern "C" int rn_selftest_wait_budget(uint32_t spin_limit, rn_status* st) {
    RN_TRY(ensure_ctx(st));
    if (spin_limit == 0 || spin_limit > (1u << 24)) return fail(st, RN_ERR_INVALID, "spin limit %u", spin_limit);
    ScopedDev pb, qb, cb;
    RN_CUDA(cudaMalloc(&pb.p, 128 * 64 * 2), st);
    RN_CUDA(cudaMalloc(&qb.p, 32 * 64 * 2), st);
    RN_CUDA(cudaMalloc(&cb.p, 128 * 32 * 4), st);
    void *p = pb.p, *q = qb.p, *c = cb.p;
    RN_CUDA(cudaMemsetAsync(p, 0, 128 * 64 * 2, ctx().stream), st);
    RN_CUDA(cudaMemsetAsync(q, 0, 32 * 64 * 2, ctx().stream), st);
    tc::Epilogue e{};
    e.ldc = 32;
    e.c32 = (float*)c;
    e.err = ctx().dev_error;
    e.spin = spin_limit;
    e.withhold = 1;
    int rc = tc_gemm((const __nv_bfloat16*)p, 64, (const __nv_bfloat16*)q, 64, 128, 32, 64, 1, e, ctx().stream, st);
    if (rc == RN_OK) rc = check_device_error(st, "rn_selftest_wait_budget");
    cudaStreamSynchronize(ctx().stream);
    return rc;
}
