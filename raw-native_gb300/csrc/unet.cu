// unet.cu -- the learned AO surrogate: a BF16 U-Net run and trained by this project's own
// kernels, every 3x3 convolution on the tcgen05 GEMM (gemm_tc.cu), FP32 accumulation.
//
// Network (inputs: depth / radius, world normal xyz, 4-spp traced AO; output: converged AO):
//   level 0 (H x W)    e0a = conv(x; 8->32)        e0 = conv(e0a; 32->32)
//   level 1 (H/2)      e1a = conv(pool e0; 32->64) e1 = conv(e1a; 64->64)
//   level 2 (H/4)      e2a = conv(pool e1; 64->128) e2 = conv(e2a; 128->128)
//   level 3 (H/8)      b3a = conv(pool e2; 128->256) b3 = conv(b3a; 256->256)
//   level 2            d2a = conv([e2, up b3]; 384->128) d2 = conv(d2a; 128->128)
//   level 1            d1a = conv([e1, up d2]; 192->64)  d1 = conv(d1a; 64->64)
//   level 0            d0a = conv([e0, up d1]; 96->32)   d0 = conv(d0a; 32->32)
//   head               out = sigmoid(1x1 conv(d0; 32->1))
// Every 3x3 convolution is followed by ReLU; pooling is a 2x2 average, upsampling nearest.
// Activations are NHWC BF16. A convolution is a GEMM of its im2col rows (the concat and the
// upsample are read in place, never materialized) with the weights [Cout][9 Cin]:
//   forward  Y = im2col(X) W^T (+ bias, ReLU in the epilogue);
//   wgrad    dW^T = im2col(X)^T dZ (split over pixels, FP32 atomics);
//   dgrad    dX = im2col(dZ) W'^T with W'[ci][tap', co] = W[co][8 - tap', ci] (the flipped,
//            transposed kernel), routed back to the sources (2x2 sums for an upsampled one).
// Loss: mean squared error of the sigmoid output; optimizer: Adam on FP32 master weights,
// which refreshes the BF16 copies the GEMMs read.
#include "gemm_tc.h"
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

namespace rn {
namespace {

using bf16 = __nv_bfloat16;
constexpr int kInC = 8;          // input channels as stored (5 used)
constexpr int kLayers = 14;

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

struct Src { int tensor; int up; };      // tensor index; up: read nearest from the half-size level

struct LayerSpec { int level, cin, cout; Src s0, s1; int nsrc; };

// tensors: 0 input, 1..14 layer outputs (layer L writes tensor L+1), 15..17 pooled p0, p1, p2
enum { T_IN = 0, T_P0 = 15, T_P1 = 16, T_P2 = 17, T_COUNT = 18 };
const LayerSpec kSpec[kLayers] = {
    {0, 8, 32, {T_IN, 0}, {0, 0}, 1},    {0, 32, 32, {1, 0}, {0, 0}, 1},      // e0a, e0
    {1, 32, 64, {T_P0, 0}, {0, 0}, 1},   {1, 64, 64, {3, 0}, {0, 0}, 1},      // e1a, e1
    {2, 64, 128, {T_P1, 0}, {0, 0}, 1},  {2, 128, 128, {5, 0}, {0, 0}, 1},    // e2a, e2
    {3, 128, 256, {T_P2, 0}, {0, 0}, 1}, {3, 256, 256, {7, 0}, {0, 0}, 1},    // b3a, b3
    {2, 384, 128, {6, 0}, {8, 1}, 2},    {2, 128, 128, {9, 0}, {0, 0}, 1},    // d2a, d2
    {1, 192, 64, {4, 0}, {10, 1}, 2},    {1, 64, 64, {11, 0}, {0, 0}, 1},     // d1a, d1
    {0, 96, 32, {2, 0}, {12, 1}, 2},     {0, 32, 32, {13, 0}, {0, 0}, 1},     // d0a, d0
};

// ------------------------------------------------------------------ kernels
struct Im2col {
    const bf16* s0; int c0; int up0;
    const bf16* s1; int c1; int up1;
    int B, H, W, kpad;
    bf16* out;
    int ld0;                    // channels stored per pixel of s0 (0: c0)
};
// One thread per (row, 8 consecutive columns): a group never straddles a tap or a source
// because every channel count is a multiple of 8.
__global__ void im2col_kernel(const Im2col a) {
    const int G = a.kpad / 8;
    const size_t total = (size_t)a.B * a.H * a.W * G;
    const int cin = a.c0 + a.c1;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        const size_t m = idx / G;
        const int k = (int)(idx % G) * 8;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (k < 9 * cin) {
            const int tap = k / cin, ci = k % cin;
            const int x = (int)(m % a.W), y = (int)((m / a.W) % a.H), b = (int)(m / ((size_t)a.W * a.H));
            const int yy = y + tap / 3 - 1, xx = x + tap % 3 - 1;
            if (yy >= 0 && yy < a.H && xx >= 0 && xx < a.W) {
                const bool first = ci < a.c0;
                const bf16* s = first ? a.s0 : a.s1;
                const int C = first ? (a.ld0 ? a.ld0 : a.c0) : a.c1, c = first ? ci : ci - a.c0,
                          up = first ? a.up0 : a.up1;
                const int h = up ? a.H / 2 : a.H, w = up ? a.W / 2 : a.W;
                const int sy = up ? yy >> 1 : yy, sx = up ? xx >> 1 : xx;
                v = *reinterpret_cast<const uint4*>(s + (((size_t)b * h + sy) * w + sx) * C + c);
            }
        }
        *reinterpret_cast<uint4*>(a.out + m * a.kpad + k) = v;
    }
}

// out[c][r] = in[r][c] for an R x C BF16 matrix (R, C multiples of 32).
__global__ void transpose_kernel(const bf16* __restrict__ in, int R, int Cc, bf16* __restrict__ out) {
    __shared__ bf16 tile[32][33];
    const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    for (int j = threadIdx.y; j < 32; j += 8) tile[j][threadIdx.x] = in[(size_t)(r0 + j) * Cc + c0 + threadIdx.x];
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) out[(size_t)(c0 + j) * R + r0 + threadIdx.x] = tile[threadIdx.x][j];
}

// 2x2 average pool, 8 channels (16 bytes) per thread; the sum order (top-left, top-right,
// bottom-left, bottom-right) is fixed.
__global__ void pool_kernel(const bf16* __restrict__ in, int B, int H, int W, int C, bf16* __restrict__ out) {
    const int h = H / 2, w = W / 2, G = C / 8;
    const size_t total = (size_t)B * h * w * G;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % G) * 8;
        const size_t p = i / G;
        const int x = (int)(p % w), y = (int)((p / w) % h), b = (int)(p / ((size_t)w * h));
        const size_t base = (((size_t)b * H + 2 * y) * W + 2 * x) * C + c;
        uint4 q[4] = {*reinterpret_cast<const uint4*>(in + base), *reinterpret_cast<const uint4*>(in + base + C),
                      *reinterpret_cast<const uint4*>(in + base + (size_t)W * C),
                      *reinterpret_cast<const uint4*>(in + base + (size_t)W * C + C)};
        uint4 o;
        bf16* ob = reinterpret_cast<bf16*>(&o);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float s = __bfloat162float(reinterpret_cast<const bf16*>(&q[0])[j]) +
                            __bfloat162float(reinterpret_cast<const bf16*>(&q[1])[j]) +
                            __bfloat162float(reinterpret_cast<const bf16*>(&q[2])[j]) +
                            __bfloat162float(reinterpret_cast<const bf16*>(&q[3])[j]);
            ob[j] = __float2bfloat16_rn(0.25f * s);
        }
        *reinterpret_cast<uint4*>(out + p * C + c) = o;
    }
}

// dHi[b, 2y+dy, 2x+dx, c] += 0.25 dLo[b, y, x, c]
__global__ void pool_back_kernel(const float* __restrict__ dlo, int B, int H, int W, int C, float* __restrict__ dhi) {
    const size_t total = (size_t)B * H * W * C;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const size_t p = i / C;
        const int x = (int)(p % W), y = (int)((p / W) % H), b = (int)(p / ((size_t)W * H));
        dhi[i] += 0.25f * dlo[(((size_t)b * (H / 2) + y / 2) * (W / 2) + x / 2) * C + c];
    }
}

// Route a convolution's input gradient dX [M][ldx] (columns off..off+C) to a source's FP32
// accumulator: directly, or summed over 2 x 2 blocks for a nearest-upsampled source.
__global__ void route_kernel(const float* __restrict__ dx, int ldx, int off, int C, int up, int B, int H, int W,
                             float* __restrict__ dsrc) {
    const int h = up ? H / 2 : H, w = up ? W / 2 : W;
    const size_t total = (size_t)B * h * w * C;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const size_t p = i / C;
        const int x = (int)(p % w), y = (int)((p / w) % h), b = (int)(p / ((size_t)w * h));
        float s;
        if (!up) {
            s = dx[p * ldx + off + c];
        } else {
            const size_t m00 = ((size_t)b * H + 2 * y) * W + 2 * x;
            s = dx[m00 * ldx + off + c] + dx[(m00 + 1) * ldx + off + c] + dx[(m00 + W) * ldx + off + c] +
                dx[(m00 + W + 1) * ldx + off + c];
        }
        dsrc[i] += s;
    }
}

// dZ = bf16(dOut where out > 0): the gradient at the pre-activation of a ReLU layer.
__global__ void gate_kernel(const float* __restrict__ dout, const bf16* __restrict__ out, size_t n, bf16* __restrict__ dz) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dz[i] = __float2bfloat16_rn(__bfloat162float(out[i]) > 0.0f ? dout[i] : 0.0f);
}

// db[c] += sum over rows of dZ[m][c] (C <= 256; blocks of 256 threads over row chunks).
__global__ void colsum_kernel(const bf16* __restrict__ dz, size_t M, int C, float* __restrict__ db) {
    const int c = threadIdx.x;
    if (c >= C) return;
    float s = 0.0f;
    for (size_t m = blockIdx.x; m < M; m += gridDim.x) s += __bfloat162float(dz[m * C + c]);
    atomicAdd(db + c, s);
}

// The head: out = sigmoid(d0 . wh + bh); with a target also the loss, dOut(d0) and the head's
// gradients. C = 32 channels, one thread per pixel.
__global__ void head_kernel(const bf16* __restrict__ d0, const float* __restrict__ wh, const float* __restrict__ bh,
                            size_t M, float* __restrict__ out, const float* __restrict__ target, float inv_m,
                            float* __restrict__ dd0, float* __restrict__ gwh, float* __restrict__ gbh,
                            float* __restrict__ loss) {
    __shared__ float s_gw[32], s_gb, s_loss;
    if (threadIdx.x < 32) s_gw[threadIdx.x] = 0.0f;
    if (threadIdx.x == 0) { s_gb = 0.0f; s_loss = 0.0f; }
    __syncthreads();
    const size_t m = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m < M) {
        float f[32];
        const uint4* p = reinterpret_cast<const uint4*>(d0 + m * 32);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint4 v = p[q];
            const bf16* h = reinterpret_cast<const bf16*>(&v);
#pragma unroll
            for (int j = 0; j < 8; ++j) f[q * 8 + j] = __bfloat162float(h[j]);
        }
        float z = bh[0];
#pragma unroll
        for (int c = 0; c < 32; ++c) z += f[c] * wh[c];
        const float s = 1.0f / (1.0f + __expf(-z));
        if (out) out[m] = s;
        if (target) {
            const float diff = s - target[m];
            const float dz = 2.0f * diff * s * (1.0f - s) * inv_m;
            atomicAdd(&s_loss, diff * diff);
            atomicAdd(&s_gb, dz);
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                dd0[m * 32 + c] = dz * wh[c];
                atomicAdd(&s_gw[c], dz * f[c]);
            }
        }
    }
    __syncthreads();
    if (target) {
        if (threadIdx.x < 32) atomicAdd(gwh + threadIdx.x, s_gw[threadIdx.x]);
        if (threadIdx.x == 0) { atomicAdd(gbh, s_gb); atomicAdd(loss, s_loss); }
    }
}

// fp32 features [M][5] -> bf16 [M][C] (C = 8, 16 or 32; channels 5.. zero)
__global__ void input_kernel(const float* __restrict__ in, size_t M, int C, bf16* __restrict__ out) {
    for (size_t m = (size_t)blockIdx.x * blockDim.x + threadIdx.x; m < M; m += (size_t)gridDim.x * blockDim.x) {
        uint4 v;
        bf16* h = reinterpret_cast<bf16*>(&v);
        for (int c = 0; c < 8; ++c) h[c] = __float2bfloat16_rn(c < 5 ? in[m * 5 + c] : 0.0f);
        uint4* o = reinterpret_cast<uint4*>(out + m * C);
        o[0] = v;
        for (int q = 1; q < C / 8; ++q) o[q] = make_uint4(0, 0, 0, 0);
    }
}

// The first convolution's weights in the cin-channel input layout of the implicit path
// (cin 16 or 32): w0[co][tap * cin + ci] = wq[co][tap * 8 + ci] (ci < 8; the other columns
// stay zero, so the zero input channels add exact zeros).
__global__ void expand_w0_kernel(const bf16* __restrict__ wq, int kpad, bf16* __restrict__ w0, int kpad0, int cout,
                                 int cin) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cout * 72) return;
    const int co = i / 72, k = i % 72, tap = k / 8, ci = k % 8;
    w0[(size_t)co * kpad0 + tap * cin + ci] = wq[(size_t)co * kpad + k];
}

struct AdamArgs { float lr, b1, b2, eps, c1, c2; const float* scale; };

// Adam on one convolution's weights (master [cout][kpad], gradient stored [kpad][cout],
// multiplied by the clip factor *a.scale), then its BF16 copies: wq [cout][kpad] and the
// flipped, transposed wt [cin_pad][kpad_t].
__global__ void adam_conv_kernel(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                                 const float* __restrict__ g, int cout, int cin, int kpad, int kpad_t, AdamArgs a,
                                 bf16* __restrict__ wq, bf16* __restrict__ wt) {
    const int total = cout * 9 * cin;
    const float sc = g ? *a.scale : 0.0f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int co = i / (9 * cin), k = i % (9 * cin);
        const size_t wi = (size_t)co * kpad + k;
        if (g) {
            const float gr = g[(size_t)k * cout + co] * sc;
            const float mm = a.b1 * m[wi] + (1.0f - a.b1) * gr;
            const float vv = a.b2 * v[wi] + (1.0f - a.b2) * gr * gr;
            m[wi] = mm;
            v[wi] = vv;
            w[wi] -= a.lr * (mm * a.c1) / (sqrtf(vv * a.c2) + a.eps);
        }
        const bf16 q = __float2bfloat16_rn(w[wi]);
        wq[wi] = q;
        const int tap = k / cin, ci = k % cin;
        wt[(size_t)ci * kpad_t + (size_t)(8 - tap) * cout + co] = q;
    }
}
__global__ void adam_vec_kernel(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                                const float* __restrict__ g, int n, AdamArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gr = g[i] * *a.scale;
    const float mm = a.b1 * m[i] + (1.0f - a.b1) * gr;
    const float vv = a.b2 * v[i] + (1.0f - a.b2) * gr * gr;
    m[i] = mm;
    v[i] = vv;
    w[i] -= a.lr * (mm * a.c1) / (sqrtf(vv * a.c2) + a.eps);
}

// The squared global gradient norm: blockIdx.y picks one gradient array of the table.
struct GradSeg { const float* p; unsigned n; };
__global__ void grad_sumsq_kernel(const GradSeg* __restrict__ segs, float* __restrict__ sumsq) {
    const GradSeg sg = segs[blockIdx.y];
    float s = 0.0f;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < sg.n; i += gridDim.x * blockDim.x) s += sg.p[i] * sg.p[i];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ float part[8];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += part[k];
        atomicAdd(sumsq, t);
    }
}

// Adaptive clipping: the norm is limited to ratio x a running mean of the (clipped) norms.
// stats: [0] sum of squares (input), [1] norm, [2] scale applied, [3] running mean.
__global__ void clip_kernel(float* __restrict__ stats, float ratio) {
    const float norm = sqrtf(stats[0]);
    float ema = stats[3];
    float scale = 1.0f;
    if (ratio > 0.0f && isfinite(norm)) {
        if (ema <= 0.0f) ema = norm;
        const float thr = ratio * ema;
        if (norm > thr) scale = thr / norm;
        ema = 0.99f * ema + 0.01f * fminf(norm, thr);
    }
    if (!isfinite(norm)) scale = 0.0f;             // a non-finite gradient skips the step's update
    stats[1] = norm;
    stats[2] = scale;
    stats[3] = ema;
}


// ------------------------------------------------------------------ the surrogate's frame
constexpr int kSppIn = 4;                 // samples of the traced input
constexpr int kTile = 16;                 // fallback tiles: 16 x 16 pixels
constexpr int kDepthBlocks = 512;

// Per-block sums of the covered pixels' depth (FP64) and count, in a fixed order.
__global__ void depth_partial_kernel(const float* __restrict__ depth, const uint8_t* __restrict__ mask, size_t n,
                                     double* __restrict__ part_sum, unsigned* __restrict__ part_cnt) {
    double s = 0.0;
    unsigned c = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        if (mask[i]) { s += (double)depth[i]; ++c; }
    for (int o = 16; o; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    __shared__ double ss[8];
    __shared__ unsigned sc[8];
    if ((threadIdx.x & 31) == 0) { ss[threadIdx.x >> 5] = s; sc[threadIdx.x >> 5] = c; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        unsigned tc = 0;
        for (int k = 0; k < 8; ++k) { t += ss[k]; tc += sc[k]; }
        part_sum[blockIdx.x] = t;
        part_cnt[blockIdx.x] = tc;
    }
}
// mean = (float)(sum / count) over the partials in block order (0 without covered pixels).
__global__ void depth_mean_kernel(const double* __restrict__ part_sum, const unsigned* __restrict__ part_cnt, int nb,
                                  float* __restrict__ mean) {
    if (threadIdx.x != 0) return;
    double t = 0.0;
    unsigned long long c = 0;
    for (int k = 0; k < nb; ++k) { t += part_sum[k]; c += part_cnt[k]; }
    *mean = c ? (float)(t / (double)c) : 0.0f;
}

// The network's BF16 input for a w x h frame inside its H x W shape: clamp((depth - mean) /
// radius, -32, 32) / 8, the world normal and the 4-spp AO on covered pixels; 0, 0 and AO 1 on
// uncovered and padding pixels (channels 5..7 zero).
__global__ void features_kernel(const float* __restrict__ depth, const float* __restrict__ nrm,
                                const uint8_t* __restrict__ mask, const float* __restrict__ ao4, int w, int h, int W,
                                int H, const float* __restrict__ mean, float radius, int C, bf16* __restrict__ out) {
    const size_t total = (size_t)W * H;
    const float mu = *mean;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % W), y = (int)(i / W);
        float f[5] = {0.0f, 0.0f, 0.0f, 0.0f, 1.0f};
        if (x < w && y < h) {
            const size_t p = (size_t)y * w + x;
            if (mask[p]) {
                f[0] = fminf(fmaxf((depth[p] - mu) / radius, -32.0f), 32.0f) * 0.125f;
                f[1] = nrm[3 * p];
                f[2] = nrm[3 * p + 1];
                f[3] = nrm[3 * p + 2];
                f[4] = ao4[p];
            }
        }
        uint4 v = make_uint4(0, 0, 0, 0);
        bf16* hb = reinterpret_cast<bf16*>(&v);
#pragma unroll
        for (int c = 0; c < 5; ++c) hb[c] = __float2bfloat16_rn(f[c]);
        uint4* o = reinterpret_cast<uint4*>(out + i * C);
        o[0] = v;
        for (int q = 1; q < C / 8; ++q) o[q] = make_uint4(0, 0, 0, 0);
    }
}

// One 16 x 16 tile per block: the confidence band test of the prediction's tile mean against
// the 4-spp tile mean (sigma = max(sqrt(sum p (1 - p) / 4) / n, 0.5 / sqrt(4 n)) over the n
// covered pixels), the tile's flag, and the fallback mask of its pixels.
__global__ void __launch_bounds__(kTile * kTile) band_kernel(const float* __restrict__ pred, int W,
                                                              const float* __restrict__ ao4,
                                                              const uint8_t* __restrict__ mask, int w, int h, float k,
                                                              uint8_t* __restrict__ tile_flag,
                                                              uint8_t* __restrict__ fb_mask,
                                                              unsigned* __restrict__ counts,
                                                              uint32_t* __restrict__ fb_list) {
    const int x = blockIdx.x * kTile + (threadIdx.x % kTile), y = blockIdx.y * kTile + (threadIdx.x / kTile);
    const bool in = x < w && y < h;
    const size_t p = (size_t)y * w + x;
    const bool cov = in && mask[p];
    float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (cov) {
        const float a = ao4[p];
        v[0] = 1.0f;
        v[1] = pred[(size_t)y * W + x];
        v[2] = a;
        v[3] = a * (1.0f - a);
    }
    __shared__ float red[4][kTile * kTile / 32];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        float t = v[q];
        for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = t;
    }
    __syncthreads();
    __shared__ int s_flag;
    if (threadIdx.x == 0) {
        float t[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int q = 0; q < 4; ++q)
            for (int j = 0; j < kTile * kTile / 32; ++j) t[q] += red[q][j];
        const float n = fmaxf(t[0], 1.0f);
        const float sigma = fmaxf(sqrtf(fmaxf(t[3], 0.0f) / (float)kSppIn) / n, 0.5f / sqrtf((float)kSppIn * n));
        const int flag = t[0] > 0.0f && fabsf(t[1] / n - t[2] / n) > k * sigma;
        tile_flag[blockIdx.y * gridDim.x + blockIdx.x] = (uint8_t)flag;
        if (t[0] > 0.0f) atomicAdd(counts, 1u);
        if (flag) atomicAdd(counts + 1, 1u);
        s_flag = flag;
    }
    __syncthreads();
    if (in) fb_mask[p] = (uint8_t)(cov && s_flag);
    if (cov && s_flag) fb_list[atomicAdd(counts + 2, 1u)] = (uint32_t)p;
}

// ao = 1 off the coverage, the traced AO (open rays / spp, as the trace divides) on fallback
// pixels, the prediction elsewhere.
__global__ void composite_kernel(const float* __restrict__ pred, int W, const uint32_t* __restrict__ open, int spp,
                                 const uint8_t* __restrict__ mask, const uint8_t* __restrict__ fb, int w, int h,
                                 float* __restrict__ ao) {
    const size_t total = (size_t)w * h;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % w), y = (int)(i / w);
        ao[i] = !mask[i] ? 1.0f : fb[i] ? __fdiv_rn((float)open[i], (float)spp) : pred[(size_t)y * W + x];
    }
}

inline unsigned grid_for(size_t n, int block = 256) {
    size_t g = (n + block - 1) / block;
    return (unsigned)(g > 65535 * 8 ? 65535 * 8 : (g ? g : 1));
}

}  // namespace
}  // namespace rn

using namespace rn;

struct rn_unet {
    int B = 0, H = 0, W = 0;
    int step = 0;
    bool inference = false;       // forward only: one shared im2col buffer, no gradient storage
    bool implicit = false;        // 3x3 convolutions of >= 32 input channels on the implicit GEMM
    bf16* UT[T_COUNT] = {};       // implicit: 2x upsampled copies of the tensors read upsampled
    bf16* wq0 = nullptr;          // implicit: the first convolution's weights for the 16/32-channel input
    int kpad0 = 0;
    // per layer
    struct Layer {
        int level, cin, cout, kpad, kpad_t, cin_pad;
        float *w, *m, *v, *b, *bm, *bv, *gw, *gb;
        bf16 *wq, *wt;
        bf16* A;          // im2col rows [M][kpad], kept for wgrad
    } L[kLayers];
    float *wh, *mh, *vh, *bh, *mbh, *vbh, *gwh, *gbh;
    bf16* T[T_COUNT];     // activations
    float* dT[T_COUNT];   // FP32 gradient accumulators
    size_t Tn[T_COUNT];   // elements
    int Tlevel[T_COUNT], TC[T_COUNT];
    bf16 *at, *dzt, *dz, *bcol;   // scratch: A^T, dZ^T, dZ, im2col(dZ)
    float* dx;                    // scratch: dgrad output [M][cin_pad]
    float* loss;                  // device scalar
    float* host_loss;             // pinned: loss, gradient norm, clip scale
    float* gstats;                // device: see clip_kernel
    GradSeg* segs;                // device table of the gradient arrays
    int nsegs = 0;
    std::vector<GradSeg> hsegs;   // the same table on the host (flat gradient copies)
    float clip_ratio = 0.0f;
    std::vector<void*> allocs;
    size_t param_count = 0;
};

namespace {

int ualloc(rn_unet* u, void** p, size_t bytes, rn_status* st) {
    RN_CUDA(cudaMalloc(p, bytes ? bytes : 16), st);
    RN_CUDA(cudaMemset(*p, 0, bytes ? bytes : 16), st);
    u->allocs.push_back(*p);
    return RN_OK;
}
size_t pixels(const rn_unet* u, int level) { return (size_t)u->B * (u->H >> level) * (u->W >> level); }

// The upsampled copy a layer's output feeds (implicit path), or null.
bf16* up_target(rn_unet* u, int l) { return u->implicit ? u->UT[l + 1] : nullptr; }

// head_out (implicit path, the last layer): the head's sigmoid output straight from the
// layer's epilogue; the layer's own activation is then not stored.
int conv_forward(rn_unet* u, int l, cudaStream_t s, rn_status* st, float* head_out = nullptr) {
    auto& Ly = u->L[l];
    const LayerSpec& sp = kSpec[l];
    const int H = u->H >> Ly.level, W = u->W >> Ly.level;
    const size_t M = pixels(u, Ly.level);
    if (u->implicit && l == 0) {          // the input is stored with 16 or 32 channels (5 used)
        const tc::ConvSrc src{u->T[T_IN], u->TC[T_IN]};
        tc::Epilogue e{};
        e.ldc = Ly.cout;
        e.c16 = u->T[1];
        e.bias = Ly.b;
        e.relu = 1;
        e.err = ctx().dev_error;
        return tc_conv3x3(&src, 1, u->B, H, W, u->wq0, u->kpad0, Ly.cout, e, nullptr, s, st);
    }
    if (u->implicit) {
        tc::ConvSrc src[2] = {{u->T[sp.s0.tensor], u->TC[sp.s0.tensor]}, {nullptr, 0}};
        if (sp.nsrc == 2) src[1] = {sp.s1.up ? u->UT[sp.s1.tensor] : u->T[sp.s1.tensor], u->TC[sp.s1.tensor]};
        tc::Epilogue e{};
        e.ldc = Ly.cout;
        e.c16 = u->T[l + 1];
        e.bias = Ly.b;
        e.relu = 1;
        e.err = ctx().dev_error;
        if (head_out) {
            e.c16 = nullptr;
            e.head_w = u->wh;
            e.head_b = u->bh;
            e.head_out = head_out;
        }
        return tc_conv3x3(src, sp.nsrc, u->B, H, W, Ly.wq, Ly.kpad, Ly.cout, e, up_target(u, l), s, st);
    }
    Im2col a{u->T[sp.s0.tensor], u->TC[sp.s0.tensor], sp.s0.up, nullptr, 0, 0, u->B, H, W, Ly.kpad, Ly.A};
    if (sp.nsrc == 2) { a.s1 = u->T[sp.s1.tensor]; a.c1 = u->TC[sp.s1.tensor]; a.up1 = sp.s1.up; }
    im2col_kernel<<<grid_for(M * (Ly.kpad / 8)), 256, 0, s>>>(a);
    tc::Epilogue e{};
    e.ldc = Ly.cout;
    e.c16 = u->T[l + 1];
    e.bias = Ly.b;
    e.relu = 1;
    e.err = ctx().dev_error;
    return tc_gemm(Ly.A, Ly.kpad, Ly.wq, Ly.kpad, (int)M, Ly.cout, Ly.kpad, 1, e, s, st);
}

// The forward pass; with head_out (implicit path only) the head's sigmoid output is written
// by the last layer's epilogue, else the caller runs head_kernel on T[14].
int forward_all(rn_unet* u, cudaStream_t s, rn_status* st, float* head_out = nullptr) {
    for (int l = 0; l < kLayers; ++l) {
        if (l == 2) pool_kernel<<<grid_for(pixels(u, 1) * 4), 256, 0, s>>>(u->T[2], u->B, u->H, u->W, 32, u->T[T_P0]);
        if (l == 4) pool_kernel<<<grid_for(pixels(u, 2) * 8), 256, 0, s>>>(u->T[4], u->B, u->H >> 1, u->W >> 1, 64, u->T[T_P1]);
        if (l == 6) pool_kernel<<<grid_for(pixels(u, 3) * 16), 256, 0, s>>>(u->T[6], u->B, u->H >> 2, u->W >> 2, 128, u->T[T_P2]);
        RN_TRY(conv_forward(u, l, s, st, l == kLayers - 1 && u->implicit ? head_out : nullptr));
    }
    return RN_OK;
}

int conv_backward(rn_unet* u, int l, cudaStream_t s, rn_status* st) {
    auto& Ly = u->L[l];
    const LayerSpec& sp = kSpec[l];
    const int H = u->H >> Ly.level, W = u->W >> Ly.level;
    const size_t M = pixels(u, Ly.level);
    // dZ: the gradient at the pre-activation
    gate_kernel<<<grid_for(M * Ly.cout), 256, 0, s>>>(u->dT[l + 1], u->T[l + 1], M * Ly.cout, u->dz);
    colsum_kernel<<<256, 256, 0, s>>>(u->dz, M, Ly.cout, Ly.gb);
    if (u->implicit) {
        // the forward left no im2col rows: form this layer's now (one shared buffer)
        Im2col a{u->T[sp.s0.tensor], u->TC[sp.s0.tensor], sp.s0.up, nullptr, 0, 0, u->B, H, W, Ly.kpad, Ly.A};
        if (sp.nsrc == 2) { a.s1 = u->T[sp.s1.tensor]; a.c1 = u->TC[sp.s1.tensor]; a.up1 = sp.s1.up; }
        if (l == 0) { a.c0 = kInC; a.ld0 = u->TC[T_IN]; }
        im2col_kernel<<<grid_for(M * (Ly.kpad / 8)), 256, 0, s>>>(a);
    }
    // wgrad: dW^T [kpad][cout] = A^T (kpad x M) * (dZ^T (cout x M))^T
    transpose_kernel<<<dim3(Ly.kpad / 32, (unsigned)(M / 32)), dim3(32, 8), 0, s>>>(Ly.A, (int)M, Ly.kpad, u->at);
    transpose_kernel<<<dim3(Ly.cout / 32, (unsigned)(M / 32)), dim3(32, 8), 0, s>>>(u->dz, (int)M, Ly.cout, u->dzt);
    int splits = 1;
    while (splits < 64 && (M / 64) % (size_t)(splits * 2) == 0 && M / (size_t)(splits * 2) >= 4096) splits *= 2;
    tc::Epilogue ew{};
    ew.ldc = Ly.cout;
    ew.c32 = Ly.gw;
    ew.atomic = 1;
    ew.err = ctx().dev_error;
    RN_TRY(tc_gemm(u->at, (int)M, u->dzt, (int)M, Ly.kpad, Ly.cout, (int)M, splits, ew, s, st));
    if (l == 0) return RN_OK;                          // the input needs no gradient
    // dgrad: dX [M][cin_pad] = conv(dZ, W') with W'[ci][tap'][co] = W[co][8 - tap'][ci]
    tc::Epilogue ed{};
    ed.ldc = Ly.cin_pad;
    ed.c32 = u->dx;
    ed.err = ctx().dev_error;
    if (u->implicit) {
        const tc::ConvSrc src{u->dz, Ly.cout};
        RN_TRY(tc_conv3x3(&src, 1, u->B, H, W, Ly.wt, Ly.kpad_t, Ly.cin_pad, ed, nullptr, s, st));
    } else {
        Im2col a{u->dz, Ly.cout, 0, nullptr, 0, 0, u->B, H, W, Ly.kpad_t, u->bcol};
        im2col_kernel<<<grid_for(M * (Ly.kpad_t / 8)), 256, 0, s>>>(a);
        RN_TRY(tc_gemm(u->bcol, Ly.kpad_t, Ly.wt, Ly.kpad_t, (int)M, Ly.cin_pad, Ly.kpad_t, 1, ed, s, st));
    }
    const int c0 = u->TC[sp.s0.tensor];
    route_kernel<<<grid_for(M * c0), 256, 0, s>>>(u->dx, Ly.cin_pad, 0, c0, sp.s0.up, u->B, H, W, u->dT[sp.s0.tensor]);
    if (sp.nsrc == 2)
        route_kernel<<<grid_for(M * u->TC[sp.s1.tensor]), 256, 0, s>>>(u->dx, Ly.cin_pad, c0, u->TC[sp.s1.tensor],
                                                                         sp.s1.up, u->B, H, W, u->dT[sp.s1.tensor]);
    return RN_OK;
}

void refresh_weights(rn_unet* u, const AdamArgs* a, cudaStream_t s) {
    for (int l = 0; l < kLayers; ++l) {
        auto& Ly = u->L[l];
        const int n = Ly.cout * 9 * Ly.cin;
        adam_conv_kernel<<<(n + 255) / 256, 256, 0, s>>>(Ly.w, Ly.m, Ly.v, a ? Ly.gw : nullptr, Ly.cout, Ly.cin,
                                                        Ly.kpad, Ly.kpad_t, a ? *a : AdamArgs{}, Ly.wq, Ly.wt);
        if (a) adam_vec_kernel<<<(Ly.cout + 255) / 256, 256, 0, s>>>(Ly.b, Ly.bm, Ly.bv, Ly.gb, Ly.cout, *a);
    }
    if (u->wq0)
        expand_w0_kernel<<<(u->L[0].cout * 72 + 255) / 256, 256, 0, s>>>(u->L[0].wq, u->L[0].kpad, u->wq0, u->kpad0,
                                                                          u->L[0].cout, u->TC[T_IN]);
    if (a) {
        adam_vec_kernel<<<1, 32, 0, s>>>(u->wh, u->mh, u->vh, u->gwh, 32, *a);
        adam_vec_kernel<<<1, 32, 0, s>>>(u->bh, u->mbh, u->vbh, u->gbh, 1, *a);
    }
}

int check_shape(const rn_unet* u, int batch, rn_status* st) {
    if (batch != u->B) return fail(st, RN_ERR_INVALID, "batch %d: this network was created for %d", batch, u->B);
    return RN_OK;
}

// Parameter order for get/set: per layer w[cout][9 cin] then b[cout]; then head wh[32], bh.
template <typename F>
void for_params(rn_unet* u, F f) {
    for (int l = 0; l < kLayers; ++l) {
        auto& Ly = u->L[l];
        for (int co = 0; co < Ly.cout; ++co) f(Ly.w + (size_t)co * Ly.kpad, (size_t)9 * Ly.cin);
        f(Ly.b, (size_t)Ly.cout);
    }
    f(u->wh, 32);
    f(u->bh, 1);
}

// Adam's moments in the parameters' order: which 0 = first moment, 1 = second.
template <typename F>
void for_moments(rn_unet* u, int which, F f) {
    for (int l = 0; l < kLayers; ++l) {
        auto& Ly = u->L[l];
        float* m = which ? Ly.v : Ly.m;
        for (int co = 0; co < Ly.cout; ++co) f(m + (size_t)co * Ly.kpad, (size_t)9 * Ly.cin);
        f(which ? Ly.bv : Ly.bm, (size_t)Ly.cout);
    }
    f(which ? u->vh : u->mh, 32);
    f(which ? u->vbh : u->mbh, 1);
}

}  // namespace

extern "C" {

int rn_unet_create(int batch, int height, int width, uint64_t seed, uint32_t flags, rn_unet** out, rn_status* st) {
    if (!out) return fail(st, RN_ERR_INVALID, "null output");
    *out = nullptr;
    if (batch <= 0 || height <= 0 || width <= 0 || height % 16 || width % 16)
        return fail(st, RN_ERR_INVALID, "shape %dx%dx%d: sizes must be multiples of 16", batch, height, width);
    if (((size_t)batch * (height / 8) * (width / 8)) % 128)
        return fail(st, RN_ERR_INVALID, "batch x (H/8) x (W/8) must be a multiple of 128");
    RN_TRY(ensure_ctx(st));
    rn_unet* u = new rn_unet();
    u->B = batch; u->H = height; u->W = width;
    u->inference = (flags & RN_UNET_INFERENCE) != 0;
    u->implicit = !(flags & RN_UNET_EXPLICIT);
    for (int lv = 0; lv < 4; ++lv) u->implicit = u->implicit && tc::conv_tiling(height >> lv, width >> lv).ok;
    auto bail = [&](int rc) { rn_unet_free(u); return rc; };
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.0f, 1.0f);
    size_t max_a = 0, max_at = 0, max_dz = 0, max_bcol = 0, max_dx = 0;
    for (int l = 0; l < kLayers; ++l) {
        auto& Ly = u->L[l];
        Ly.level = kSpec[l].level; Ly.cin = kSpec[l].cin; Ly.cout = kSpec[l].cout;
        Ly.kpad = round_up(9 * Ly.cin, 128);
        Ly.kpad_t = round_up(9 * Ly.cout, 128);
        Ly.cin_pad = Ly.cin <= 32 ? 32 : Ly.cin <= 64 ? 64 : Ly.cin <= 128 ? 128 : round_up(Ly.cin, 128);
        const size_t M = pixels(u, Ly.level);
        const size_t nw = (size_t)Ly.cout * Ly.kpad;
        int rc = RN_OK;
        for (float** p : {&Ly.w, &Ly.m, &Ly.v}) if (rc == RN_OK) rc = ualloc(u, (void**)p, nw * 4, st);
        for (float** p : {&Ly.b, &Ly.bm, &Ly.bv, &Ly.gb}) if (rc == RN_OK) rc = ualloc(u, (void**)p, (size_t)Ly.cout * 4, st);
        if (rc == RN_OK) rc = ualloc(u, (void**)&Ly.gw, (size_t)Ly.kpad * Ly.cout * 4, st);
        if (rc == RN_OK) rc = ualloc(u, (void**)&Ly.wq, nw * 2, st);
        if (rc == RN_OK) rc = ualloc(u, (void**)&Ly.wt, (size_t)Ly.cin_pad * Ly.kpad_t * 2, st);
        if (rc == RN_OK && !u->inference && !u->implicit) rc = ualloc(u, (void**)&Ly.A, M * Ly.kpad * 2, st);
        if (rc != RN_OK) return bail(rc);
        // He initialization of the real taps; padded columns stay zero
        std::vector<float> w(nw, 0.0f);
        const float sd = std::sqrt(2.0f / (9.0f * Ly.cin));
        for (int co = 0; co < Ly.cout; ++co)
            for (int k = 0; k < 9 * Ly.cin; ++k) w[(size_t)co * Ly.kpad + k] = nd(rng) * sd;
        if (cudaMemcpy(Ly.w, w.data(), nw * 4, cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(fail(st, RN_ERR_CUDA, "weight upload"));
        u->param_count += (size_t)Ly.cout * 9 * Ly.cin + Ly.cout;
        max_a = std::max(max_a, M * Ly.kpad);
        max_dz = std::max(max_dz, M * Ly.cout);
        max_bcol = std::max(max_bcol, M * Ly.kpad_t);
        max_dx = std::max(max_dx, M * Ly.cin_pad);
    }
    max_at = max_a;
    if (u->inference || u->implicit) {   // the layers run in order: one im2col buffer serves all
        // (implicit inference forms no im2col rows at all)
        const size_t need = (u->implicit && u->inference) ? 8 : max_a;
        bf16* shared = nullptr;
        if (ualloc(u, (void**)&shared, need * 2, st)) return bail(RN_ERR_NO_MEMORY);
        for (auto& Ly : u->L) Ly.A = shared;
    }
    for (float** p : {&u->wh, &u->mh, &u->vh, &u->gwh}) if (ualloc(u, (void**)p, 32 * 4, st)) return bail(RN_ERR_CUDA);
    for (float** p : {&u->bh, &u->mbh, &u->vbh, &u->gbh, &u->loss}) if (ualloc(u, (void**)p, 4, st)) return bail(RN_ERR_CUDA);
    {
        std::vector<float> wh(32);
        for (auto& x : wh) x = nd(rng) * std::sqrt(1.0f / 32.0f);
        const cudaError_t e = cudaMemcpy(u->wh, wh.data(), 32 * 4, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return bail(cuda_fail(st, e, "unet head weights"));
    }
    u->param_count += 33;
    // tensors
    const int tlevel[T_COUNT] = {0, 0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0, 1, 2, 3};
    const int tch[T_COUNT] = {kInC, 32, 32, 64, 64, 128, 128, 256, 256, 128, 128, 64, 64, 32, 32, 32, 64, 128};
    for (int t = 0; t < T_COUNT; ++t) {
        u->Tlevel[t] = tlevel[t];
        // the implicit path's input: 16 channels where the row-ring kernel takes level 0
        // (128-pixel rows), else 32 (5 used)
        u->TC[t] = (t == T_IN && u->implicit) ? (u->W % 128 == 0 ? 16 : 32) : tch[t];
        u->Tn[t] = pixels(u, tlevel[t]) * u->TC[t];
        if (ualloc(u, (void**)&u->T[t], u->Tn[t] * 2, st) ||
            (!u->inference && ualloc(u, (void**)&u->dT[t], u->Tn[t] * 4, st)))
            return bail(RN_ERR_NO_MEMORY);
    }
    if (u->implicit) {
        u->kpad0 = round_up(9 * u->TC[T_IN], 128);
        if (ualloc(u, (void**)&u->wq0, (size_t)u->L[0].cout * u->kpad0 * 2, st)) return bail(RN_ERR_NO_MEMORY);
    }
    if (u->implicit)
        for (int t : {8, 10, 12})            // b3, d2, d1: read upsampled by d2a, d1a, d0a
            if (ualloc(u, (void**)&u->UT[t], pixels(u, u->Tlevel[t] - 1) * u->TC[t] * 2, st))
                return bail(RN_ERR_NO_MEMORY);
    if (!u->inference &&
        (ualloc(u, (void**)&u->at, max_at * 2, st) || ualloc(u, (void**)&u->dzt, max_dz * 2, st) ||
         ualloc(u, (void**)&u->dz, max_dz * 2, st) || ualloc(u, (void**)&u->bcol, (u->implicit ? 8 : max_bcol) * 2, st) ||
         ualloc(u, (void**)&u->dx, max_dx * 4, st)))
        return bail(RN_ERR_NO_MEMORY);
    if (cudaMallocHost((void**)&u->host_loss, 16) != cudaSuccess) return bail(fail(st, RN_ERR_NO_MEMORY, "pinned loss"));
    std::memset(u->host_loss, 0, 16);
    if (ualloc(u, (void**)&u->gstats, 16, st)) return bail(RN_ERR_NO_MEMORY);
    {
        std::vector<GradSeg> segs;
        for (auto& Ly : u->L) {
            segs.push_back({Ly.gw, (unsigned)((size_t)Ly.kpad * Ly.cout)});
            segs.push_back({Ly.gb, (unsigned)Ly.cout});
        }
        segs.push_back({u->gwh, 32});
        segs.push_back({u->gbh, 1});
        u->nsegs = (int)segs.size();
        u->hsegs = segs;
        if (ualloc(u, (void**)&u->segs, segs.size() * sizeof(GradSeg), st)) return bail(RN_ERR_NO_MEMORY);
        if (cudaMemcpy(u->segs, segs.data(), segs.size() * sizeof(GradSeg), cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(fail(st, RN_ERR_CUDA, "gradient table upload"));
    }
    refresh_weights(u, nullptr, ctx().stream);
    if (cudaStreamSynchronize(ctx().stream) != cudaSuccess) return bail(cuda_fail(st, cudaGetLastError(), "unet init"));
    *out = u;
    return ok(st);
}

void rn_unet_free(rn_unet* u) {
    if (!u) return;
    cudaDeviceSynchronize();
    for (void* p : u->allocs) cudaFree(p);
    if (u->host_loss) cudaFreeHost(u->host_loss);
    delete u;
}

int rn_unet_param_count(const rn_unet* u, uint64_t* count, rn_status* st) {
    if (!u || !count) return fail(st, RN_ERR_INVALID, "null argument");
    *count = u->param_count;
    return ok(st);
}

int rn_unet_forward(rn_unet* u, const float* input, int batch, float* output, rn_status* st) {
    if (!u || !input || !output) return fail(st, RN_ERR_INVALID, "null argument");
    RN_TRY(check_shape(u, batch, st));
    cudaStream_t s = ctx().stream;
    const size_t M = pixels(u, 0);
    input_kernel<<<grid_for(M), 256, 0, s>>>(input, M, u->TC[T_IN], u->T[T_IN]);
    if (u->implicit) {
        RN_TRY(forward_all(u, s, st, output));         // the head in the last layer's epilogue
    } else {
        RN_TRY(forward_all(u, s, st));
        head_kernel<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(u->T[14], u->wh, u->bh, M, output, nullptr, 0.0f,
                                                               nullptr, nullptr, nullptr, nullptr);
    }
    RN_CUDA(cudaGetLastError(), st);
    return ok(st);
}

// Forward and backward on one batch: the gradients are left in the network, *loss (if
// given) receives the batch's mean squared error.
int rn_unet_backward(rn_unet* u, const float* input, const float* target, int batch, float* loss, rn_status* st) {
    if (!u || !input || !target) return fail(st, RN_ERR_INVALID, "null argument");
    if (u->inference) return fail(st, RN_ERR_INVALID, "network created for inference only");
    RN_TRY(check_shape(u, batch, st));
    cudaStream_t s = ctx().stream;
    const size_t M = pixels(u, 0);
    input_kernel<<<grid_for(M), 256, 0, s>>>(input, M, u->TC[T_IN], u->T[T_IN]);
    RN_TRY(forward_all(u, s, st));
    // zero the gradient accumulators
    for (int t = 0; t < T_COUNT; ++t) RN_CUDA(cudaMemsetAsync(u->dT[t], 0, u->Tn[t] * 4, s), st);
    for (int l = 0; l < kLayers; ++l) {
        RN_CUDA(cudaMemsetAsync(u->L[l].gw, 0, (size_t)u->L[l].kpad * u->L[l].cout * 4, s), st);
        RN_CUDA(cudaMemsetAsync(u->L[l].gb, 0, (size_t)u->L[l].cout * 4, s), st);
    }
    RN_CUDA(cudaMemsetAsync(u->gwh, 0, 32 * 4, s), st);
    RN_CUDA(cudaMemsetAsync(u->gbh, 0, 4, s), st);
    RN_CUDA(cudaMemsetAsync(u->loss, 0, 4, s), st);
    head_kernel<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(u->T[14], u->wh, u->bh, M, nullptr, target, 1.0f / (float)M,
                                                           u->dT[14], u->gwh, u->gbh, u->loss);
    for (int l = kLayers - 1; l >= 0; --l) {
        RN_TRY(conv_backward(u, l, s, st));
        // pooled tensors feed encoder levels: their gradients flow back through the pool
        if (l == 6) pool_back_kernel<<<grid_for(u->Tn[6]), 256, 0, s>>>(u->dT[T_P2], u->B, u->H >> 2, u->W >> 2, 128, u->dT[6]);
        if (l == 4) pool_back_kernel<<<grid_for(u->Tn[4]), 256, 0, s>>>(u->dT[T_P1], u->B, u->H >> 1, u->W >> 1, 64, u->dT[4]);
        if (l == 2) pool_back_kernel<<<grid_for(u->Tn[2]), 256, 0, s>>>(u->dT[T_P0], u->B, u->H, u->W, 32, u->dT[2]);
    }
    RN_CUDA(cudaMemcpyAsync(u->host_loss, u->loss, 4, cudaMemcpyDeviceToHost, s), st);
    RN_CUDA(cudaStreamSynchronize(s), st);
    RN_TRY(check_device_error(st, "rn_unet_backward"));
    if (loss) *loss = *u->host_loss / (float)M;
    return ok(st);
}

// The update from the gradients the network holds: their global norm, the adaptive clip
// factor, and (lr > 0) one Adam step with the BF16 copies refreshed.
int rn_unet_apply(rn_unet* u, float lr, rn_status* st) {
    if (!u) return fail(st, RN_ERR_INVALID, "null argument");
    if (u->inference) return fail(st, RN_ERR_INVALID, "network created for inference only");
    cudaStream_t s = ctx().stream;
    RN_CUDA(cudaMemsetAsync(u->gstats, 0, 4, s), st);
    grad_sumsq_kernel<<<dim3(64, u->nsegs), 256, 0, s>>>(u->segs, u->gstats);
    clip_kernel<<<1, 1, 0, s>>>(u->gstats, u->clip_ratio);
    if (lr > 0.0f) {
        ++u->step;
        const AdamArgs a{lr, 0.9f, 0.999f, 1e-8f, 1.0f / (1.0f - std::pow(0.9f, (float)u->step)),
                         1.0f / (1.0f - std::pow(0.999f, (float)u->step)), u->gstats + 2};
        refresh_weights(u, &a, s);
    }
    RN_CUDA(cudaMemcpyAsync(u->host_loss + 1, u->gstats + 1, 8, cudaMemcpyDeviceToHost, s), st);
    RN_CUDA(cudaStreamSynchronize(s), st);
    RN_TRY(check_device_error(st, "rn_unet_apply"));
    return ok(st);
}

int rn_unet_train_step(rn_unet* u, const float* input, const float* target, int batch, float lr, float* loss,
                       rn_status* st) {
    RN_TRY(rn_unet_backward(u, input, target, batch, loss, st));
    return rn_unet_apply(u, lr, st);
}

// The gradients as one flat FP32 array (the gradient table's order: per layer the weight
// gradient [kpad][cout] then the bias, then the head's 32 + 1), for an exchange between
// data-parallel ranks: copied to (to_flat != 0) or from a DEVICE array of
// rn_unet_grad_count values on the library's stream (asynchronous).
int rn_unet_grad_count(const rn_unet* u, uint64_t* count, rn_status* st) {
    if (!u || !count) return fail(st, RN_ERR_INVALID, "null argument");
    uint64_t n = 0;
    for (const GradSeg& g : u->hsegs) n += g.n;
    *count = n;
    return ok(st);
}
int rn_unet_grads_flat(rn_unet* u, float* dev, int to_flat, rn_status* st) {
    if (!u || !dev) return fail(st, RN_ERR_INVALID, "null argument");
    if (u->inference) return fail(st, RN_ERR_INVALID, "network created for inference only");
    cudaStream_t s = ctx().stream;
    size_t o = 0;
    for (const GradSeg& g : u->hsegs) {
        float* seg = const_cast<float*>(g.p);
        if (to_flat) RN_CUDA(cudaMemcpyAsync(dev + o, seg, (size_t)g.n * 4, cudaMemcpyDeviceToDevice, s), st);
        else RN_CUDA(cudaMemcpyAsync(seg, dev + o, (size_t)g.n * 4, cudaMemcpyDeviceToDevice, s), st);
        o += g.n;
    }
    return ok(st);
}

// Parameters (host, FP32, rn_unet_param_count of them, in layer order: w[cout][9 cin], b).
int rn_unet_get_params(rn_unet* u, float* host, rn_status* st) {
    if (!u || !host) return fail(st, RN_ERR_INVALID, "null argument");
    RN_CUDA(cudaDeviceSynchronize(), st);
    size_t o = 0;
    for_params(u, [&](float* d, size_t n) { cudaMemcpy(host + o, d, n * 4, cudaMemcpyDeviceToHost); o += n; });
    return ok(st);
}
int rn_unet_set_params(rn_unet* u, const float* host, rn_status* st) {
    if (!u || !host) return fail(st, RN_ERR_INVALID, "null argument");
    RN_CUDA(cudaDeviceSynchronize(), st);
    size_t o = 0;
    for_params(u, [&](float* d, size_t n) { cudaMemcpy(d, host + o, n * 4, cudaMemcpyHostToDevice); o += n; });
    refresh_weights(u, nullptr, ctx().stream);
    RN_CUDA(cudaStreamSynchronize(ctx().stream), st);
    return ok(st);
}
// Adaptive gradient clipping for the following train steps: the global gradient norm is
// limited to `ratio` x a running mean of past (clipped) norms; 0 turns clipping off.
int rn_unet_set_clip(rn_unet* u, float ratio, rn_status* st) {
    if (!u || !(ratio >= 0.0f)) return fail(st, RN_ERR_INVALID, "clip ratio must be >= 0");
    u->clip_ratio = ratio;
    return ok(st);
}
// The last train step's global gradient norm (before clipping) and the factor applied.
int rn_unet_last_grad_norm(const rn_unet* u, float* norm, float* scale, rn_status* st) {
    if (!u) return fail(st, RN_ERR_INVALID, "null argument");
    if (norm) *norm = u->host_loss[1];
    if (scale) *scale = u->host_loss[2];
    return ok(st);
}


// One AO frame by the surrogate: the 4-spp trace, the network, the confidence-band test per
// 16 x 16 tile and the fallback tiles traced at spp_full. Device pointers; batch-1 network
// whose shape covers the frame.
int rn_surrogate_ao(rn_unet* u, const rn_gbuf* g, const float* depth, const rn_accel* accel, int spp_full, float radius,
                    float k, float* ao, float* ao4_out, float* pred_out, uint8_t* tile_flags,
                    rn_surrogate_stats* stats, rn_status* st) {
    if (!u || !g || !depth || !accel || !ao) return fail(st, RN_ERR_INVALID, "null argument");
    if (!g->position || !g->normal || !g->mask) return fail(st, RN_ERR_INVALID, "null G-buffer plane");
    if (u->B != 1) return fail(st, RN_ERR_INVALID, "the surrogate frame needs a batch-1 network (batch %d)", u->B);
    const int w = g->w, h = g->h;
    if (w <= 0 || h <= 0 || w > u->W || h > u->H)
        return fail(st, RN_ERR_INVALID, "frame %dx%d does not fit the network's %dx%d", w, h, u->W, u->H);
    if (spp_full <= 0 || !(radius > 0.0f) || !(k >= 0.0f)) return fail(st, RN_ERR_INVALID, "spp %d radius %g k %g", spp_full, radius, k);
    if (accel->device != ctx().device) return fail(st, RN_ERR_STATE, "accelerator built on another device");
    cudaStream_t s = ctx().stream;
    const size_t np = (size_t)w * h, npad = (size_t)u->W * u->H;
    const int tx = (w + kTile - 1) / kTile, ty = (h + kTile - 1) / kTile;
    void *p_ao4, *p_pred, *p_fb, *p_aofb, *p_st;
    RN_TRY(ws_get(WS_SUR_AO4, np * 4, &p_ao4, st));
    RN_TRY(ws_get(WS_SUR_PRED, npad * 4, &p_pred, st));
    RN_TRY(ws_get(WS_SUR_FB, np + (size_t)tx * ty, &p_fb, st));
    RN_TRY(ws_get(WS_SUR_AOFB, np * 8, &p_aofb, st));          // open-ray counts, then the pixel list
    RN_TRY(ws_get(WS_SUR_STATS, 16 + kDepthBlocks * 12, &p_st, st));
    float* a4 = ao4_out ? ao4_out : (float*)p_ao4;
    float* pr = (float*)p_pred;
    uint8_t* fbm = (uint8_t*)p_fb;
    uint8_t* tf = tile_flags ? tile_flags : fbm + np;
    unsigned* counts = (unsigned*)p_st;          // covered tiles, fallback tiles, fallback pixels
    float* mean = (float*)p_st + 3;
    double* psum = (double*)((char*)p_st + 16);
    uint32_t* open = (uint32_t*)p_aofb;
    uint32_t* fb_list = open + np;
    unsigned* pcnt = (unsigned*)(psum + kDepthBlocks);
    RN_CUDA(cudaMemsetAsync(counts, 0, 12, s), st);
    RN_CUDA(cudaMemsetAsync(open, 0, np * 4, s), st);
    // 1. the 4-spp trace
    RN_TRY(trace_ao_device(g->position, g->normal, g->mask, w, h, accel, kSppIn, radius, a4, st));
    // 2. features straight into the network's input, 3. the network
    depth_partial_kernel<<<kDepthBlocks, 256, 0, s>>>(depth, g->mask, np, psum, pcnt);
    depth_mean_kernel<<<1, 32, 0, s>>>(psum, pcnt, kDepthBlocks, mean);
    features_kernel<<<grid_for(npad), 256, 0, s>>>(depth, g->normal, g->mask, a4, w, h, u->W, u->H, mean, radius,
                                                    u->TC[T_IN], u->T[T_IN]);
    if (u->implicit) {
        RN_TRY(forward_all(u, s, st, pr));             // the head in the last layer's epilogue
    } else {
        RN_TRY(forward_all(u, s, st));
        head_kernel<<<(unsigned)((npad + 255) / 256), 256, 0, s>>>(u->T[14], u->wh, u->bh, npad, pr, nullptr, 0.0f,
                                                                  nullptr, nullptr, nullptr, nullptr);
    }
    // 4. the band test, 5. the fallback trace, 6. the composite
    band_kernel<<<dim3(tx, ty), kTile * kTile, 0, s>>>(pr, u->W, a4, g->mask, w, h, k, tf, fbm, counts, fb_list);
    // the fallback pixels' rays, one thread per (pixel, sample): a few tiles' worth of work
    // spreads over the whole GPU instead of a few warps
    const TraceParams tp = ao_trace_params(g->position, g->normal, fbm, w, h, accel, spp_full, radius);
    if (launch_ao_samples(tp, fb_list, counts + 2, open, ctx().sm_count, s) != RN_OK)
        return cuda_fail(st, cudaGetLastError(), "ao_samples_kernel");
    composite_kernel<<<grid_for(np), 256, 0, s>>>(pr, u->W, open, spp_full, g->mask, fbm, w, h, ao);
    if (pred_out) RN_CUDA(cudaMemcpy2DAsync(pred_out, (size_t)w * 4, pr, (size_t)u->W * 4, (size_t)w * 4, h,
                                            cudaMemcpyDeviceToDevice, s), st);
    RN_CUDA(cudaGetLastError(), st);
    unsigned hc[3] = {0, 0, 0};
    float hm = 0.0f;
    RN_CUDA(cudaMemcpyAsync(hc, counts, 12, cudaMemcpyDeviceToHost, s), st);
    RN_CUDA(cudaMemcpyAsync(&hm, mean, 4, cudaMemcpyDeviceToHost, s), st);
    RN_TRY(check_device_error(st, "rn_surrogate_ao"));
    if (stats) {
        stats->tiles_covered = hc[0];
        stats->tiles_fallback = hc[1];
        stats->mean_depth = hm;
        stats->reserved = 0.0f;
    }
    return ok(st);
}

// Training state: master weights, then Adam's first and second moments (each in the params'
// order and layout), and the step count.
int rn_unet_get_state(rn_unet* u, float* host, uint64_t* step, rn_status* st) {
    if (!u || !host || !step) return fail(st, RN_ERR_INVALID, "null argument");
    RN_CUDA(cudaDeviceSynchronize(), st);
    size_t o = 0;
    auto get = [&](float* d, size_t n) { cudaMemcpy(host + o, d, n * 4, cudaMemcpyDeviceToHost); o += n; };
    for_params(u, get);
    for_moments(u, 0, get);
    for_moments(u, 1, get);
    *step = (uint64_t)u->step;
    RN_CUDA(cudaGetLastError(), st);
    return ok(st);
}
int rn_unet_set_state(rn_unet* u, const float* host, uint64_t step, rn_status* st) {
    if (!u || !host) return fail(st, RN_ERR_INVALID, "null argument");
    RN_CUDA(cudaDeviceSynchronize(), st);
    size_t o = 0;
    auto put = [&](float* d, size_t n) { cudaMemcpy(d, host + o, n * 4, cudaMemcpyHostToDevice); o += n; };
    for_params(u, put);
    for_moments(u, 0, put);
    for_moments(u, 1, put);
    u->step = (int)step;
    refresh_weights(u, nullptr, ctx().stream);
    RN_CUDA(cudaStreamSynchronize(ctx().stream), st);
    return ok(st);
}

// Gradients of the last train step (lr 0 keeps them), same order and layout as the params.
int rn_unet_get_grads(rn_unet* u, float* host, rn_status* st) {
    if (!u || !host) return fail(st, RN_ERR_INVALID, "null argument");
    RN_CUDA(cudaDeviceSynchronize(), st);
    size_t o = 0;
    std::vector<float> gt;
    for (int l = 0; l < kLayers; ++l) {
        auto& Ly = u->L[l];
        gt.resize((size_t)Ly.kpad * Ly.cout);
        RN_CUDA(cudaMemcpy(gt.data(), Ly.gw, gt.size() * 4, cudaMemcpyDeviceToHost), st);
        for (int co = 0; co < Ly.cout; ++co)
            for (int k = 0; k < 9 * Ly.cin; ++k) host[o++] = gt[(size_t)k * Ly.cout + co];
        RN_CUDA(cudaMemcpy(host + o, Ly.gb, (size_t)Ly.cout * 4, cudaMemcpyDeviceToHost), st);
        o += Ly.cout;
    }
    RN_CUDA(cudaMemcpy(host + o, u->gwh, 32 * 4, cudaMemcpyDeviceToHost), st);
    o += 32;
    RN_CUDA(cudaMemcpy(host + o, u->gbh, 4, cudaMemcpyDeviceToHost), st);
    return ok(st);
}

}  // extern "C"
