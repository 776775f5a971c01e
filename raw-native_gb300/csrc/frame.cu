// frame.cu -- the rest of raw-native's frame on the GPU: the shaded frame and its HDR view
// (src/renderer/composite.cpp:8-42) and the motion plane (src/renderer/motion.cpp:7-32), in
// the reference's float operation order, one IEEE rounding each (bit-identical).
#include "rn_internal.h"
#include "rn_device.cuh"

namespace rn {
namespace {

struct Light3 { float x, y, z; };

// radianceV2 / radianceAt: ndl = max(0, n . (l * -1)) * li; model 2: lit = 0.2 sky + ndl sun,
// model 1: lit = (0.2 + ndl) ao; rgb = albedo * lit; the frame clamps it to [0, 1].
__global__ void shade_kernel(int w, int h, const float* __restrict__ nrm, const float* __restrict__ albedo,
                             const uint8_t* __restrict__ mask, int model, const float* __restrict__ a_or_sky,
                             const float* __restrict__ sun, Light3 nl, float li, float* __restrict__ frame,
                             float* __restrict__ hdr) {
    const size_t n = (size_t)w * h;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float r[3] = {0.0f, 0.0f, 0.0f};
        if (mask[i]) {
            const float d = fadd(fadd(fmul(nrm[3 * i], nl.x), fmul(nrm[3 * i + 1], nl.y)), fmul(nrm[3 * i + 2], nl.z));
            const float ndl = fmul(d > 0.0f ? d : 0.0f, li);
            const float lit = model == 2 ? fadd(fmul(0.2f, a_or_sky[i]), fmul(ndl, sun[i]))
                                         : fmul(fadd(0.2f, ndl), a_or_sky[i]);
            for (int k = 0; k < 3; ++k) r[k] = fmul(albedo[3 * i + k], lit);
        }
        for (int k = 0; k < 3; ++k) {
            if (hdr) hdr[3 * i + k] = r[k];
            if (frame) frame[3 * i + k] = r[k] < 0.0f ? 0.0f : r[k] > 1.0f ? 1.0f : r[k];
        }
    }
}

struct M16 { float m[16]; };

__device__ __forceinline__ bool project_uv(const M16& vp, float x, float y, float z, float& u, float& v) {
    float cs[4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
        cs[r] = fadd(fadd(fadd(fmul(vp.m[4 * r], x), fmul(vp.m[4 * r + 1], y)), fmul(vp.m[4 * r + 2], z)),
                     fmul(vp.m[4 * r + 3], 1.0f));
    if (cs[3] <= 1e-6f) return false;
    const float invw = frcp(cs[3]);
    const float nx = fmul(cs[0], invw), ny = fmul(cs[1], invw);
    u = fadd(fmul(nx, 0.5f), 0.5f);
    v = fsub(1.0f, fadd(fmul(ny, 0.5f), 0.5f));
    return true;
}

__global__ void motion_kernel(int w, int h, const float* __restrict__ pos, const uint8_t* __restrict__ mask, M16 cur,
                              M16 prev, float* __restrict__ motion, unsigned* __restrict__ valid) {
    const size_t n = (size_t)w * h;
    unsigned mine = 0, covered = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float mx = 0.0f, my = 0.0f;
        if (mask[i]) {
            ++covered;
            float au, av, bu, bv;
            const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
            if (project_uv(cur, x, y, z, au, av) && project_uv(prev, x, y, z, bu, bv)) {
                const float dx = fsub(au, bu), dy = fsub(av, bv);
                if (isfinite(dx) && isfinite(dy)) { mx = dx; my = dy; ++mine; }
            }
        }
        motion[2 * i] = mx;
        motion[2 * i + 1] = my;
    }
    for (int o = 16; o; o >>= 1) {
        mine += __shfl_xor_sync(0xffffffffu, mine, o);
        covered += __shfl_xor_sync(0xffffffffu, covered, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (mine) atomicAdd(valid, mine);
        if (covered) atomicAdd(valid + 1, covered);
    }
}

unsigned grid_of(size_t n) {
    const size_t g = (n + 255) / 256;
    return (unsigned)(g > 65535 * 8 ? 65535 * 8 : (g ? g : 1));
}

}  // namespace

int launch_shade(int w, int h, const float* nrm, const float* albedo, const uint8_t* mask, int model,
                 const float* a_or_sky, const float* sun, const float ldir[3], float li, float* frame, float* hdr,
                 cudaStream_t s) {
    // ldir * -1.0f: an exact negation
    const Light3 nl{-ldir[0], -ldir[1], -ldir[2]};
    shade_kernel<<<grid_of((size_t)w * h), 256, 0, s>>>(w, h, nrm, albedo, mask, model, a_or_sky, sun, nl, li, frame,
                                                         hdr);
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}

int launch_motion(int w, int h, const float* pos, const uint8_t* mask, const float* vp16, const float* prev16,
                  float* motion, unsigned* valid, cudaStream_t s) {
    M16 a, b;
    for (int k = 0; k < 16; ++k) { a.m[k] = vp16[k]; b.m[k] = prev16[k]; }
    motion_kernel<<<grid_of((size_t)w * h), 256, 0, s>>>(w, h, pos, mask, a, b, motion, valid);
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}

}  // namespace rn
