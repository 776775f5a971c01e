// ssao.cu -- the screen-space AO pass (src/renderer/ssao.cpp:11-39) on the GPU, with the
// reconcile against the ray-traced truth optionally fused into its epilogue.
//
// Every sample lands within R = 6 pixels of its pixel (radius (0.3 + 0.7 u) * 6, rounded), so
// a 32 x 8 tile needs a 44 x 20 window of positions and coverage. The block stages that window
// in shared memory once (position.xyz and a validity flag: in the frame and covered), and the
// 24 taps of each pixel read it from there: per pixel the pass moves 12 B of position, 12 B
// of normal, 1 B of mask and 4 B of output through HBM, the halo's re-reads hit L2.
//
// Sample angle: std::lround(std::cos(a) * rad) only changes when the host's cos differs from
// the device's by enough to cross a half-integer. With |cos_host - cos_dev| <= 8 ulp and
// rad <= 6 the product moves by < 3.5e-6, so only taps within 8e-6 of a half-integer consult
// the host-libm correction table (about 2e-5 of them).
#include "ssao_device.cuh"

namespace rn {
namespace {

using namespace ssao_dev;

template <bool kFused, int TY>
__global__ void __launch_bounds__(Tile<TY>::kThreads) ssao_kernel(int w, int h, const float* __restrict__ pos,
                                                                  const float* __restrict__ nrm,
                                                                  const uint8_t* __restrict__ mask, int samples,
                                                                  float radius, const uint8_t* __restrict__ corr,
                                                                  float* __restrict__ ao, const float* __restrict__ truth,
                                                                  float* __restrict__ err, RecPartial* parts, RecOut* out) {
    __shared__ float4 win[Tile<TY>::kH][kSW];
    RecAcc acc;
    ssao_tile<kFused, TY>(win, blockIdx.x, blockIdx.y, w, h, pos, nrm, mask, samples, radius, corr, ao, truth, err, acc);
    if (kFused)
        rec_block_finish<Tile<TY>::kThreads>(acc, parts, out, blockIdx.y * gridDim.x + blockIdx.x, gridDim.x * gridDim.y);
}

template <int TY>
void launch_tile(int w, int h, const float* pos, const float* nrm, const uint8_t* mask, int samples, float radius,
                 const uint8_t* corr, float* ao, const float* truth, float* err, RecPartial* partials, RecOut* out,
                 cudaStream_t s) {
    const dim3 grid((w + kTX - 1) / kTX, (h + TY - 1) / TY);
    if (truth)
        ssao_kernel<true, TY><<<grid, Tile<TY>::kThreads, 0, s>>>(w, h, pos, nrm, mask, samples, radius, corr, ao, truth,
                                                                   err, partials, out);
    else
        ssao_kernel<false, TY><<<grid, Tile<TY>::kThreads, 0, s>>>(w, h, pos, nrm, mask, samples, radius, corr, ao,
                                                                    nullptr, nullptr, nullptr, nullptr);
}

int tile_h() {
    const int t = ctx().tune.ssao_tile_h;
    return t == 4 || t == 16 ? t : 8;
}

}  // namespace

// Blocks of one SSAO launch (the fused reconcile keeps one partial per block).
int ssao_blocks(int w, int h) { return ((w + kTX - 1) / kTX) * ((h + tile_h() - 1) / tile_h()); }

int launch_ssao(int w, int h, const float* pos, const float* nrm, const uint8_t* mask, int samples, float radius,
                const uint8_t* corr, float* ao, const float* truth, float* err, RecPartial* partials, RecOut* out,
                cudaStream_t s) {
    switch (tile_h()) {
        case 4: launch_tile<4>(w, h, pos, nrm, mask, samples, radius, corr, ao, truth, err, partials, out, s); break;
        case 16: launch_tile<16>(w, h, pos, nrm, mask, samples, radius, corr, ao, truth, err, partials, out, s); break;
        default: launch_tile<8>(w, h, pos, nrm, mask, samples, radius, corr, ao, truth, err, partials, out, s); break;
    }
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}

}  // namespace rn
