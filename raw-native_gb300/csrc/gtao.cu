// gtao.cu -- ground-truth-based ambient occlusion (Jimenez, Wu, Pesce, Jarabo 2016) on the
// GPU: raw::post's GTAO pass (src/renderer/post_gtao.cpp:64-135) over the view-space
// G-buffer (:36-53), the screen-space approximation that the ray-traced oracle judges
// with the same reconcile.
//
// The view-space G-buffer is computed as the reference computes it, in float with one
// rounding per operation (bit-identical). GTAO itself runs in FP32 where the reference
// uses FP64; each slice's screen direction is formed in FP64, because it is the difference
// of two projections 1e-3 of the depth apart, and the march positions are kept relative to
// the pixel, so their floor (which pixel a sample falls in) is exact. The parity contract is
// the reference's own for its GPU pass: |gpu - cpu| <= 1e-3 on all but 0.1 % of pixels
// (raw/renderer/post_parity.hpp:15-19).
#include "rn_internal.h"
#include "rn_device.cuh"
#include <algorithm>
#include <cmath>

namespace rn {
namespace {

struct View16 { float m[16]; };

__device__ __forceinline__ float row4(const float* r, float x, float y, float z, float w) {
    return fadd(fadd(fadd(fmul(r[0], x), fmul(r[1], y)), fmul(r[2], z)), fmul(r[3], w));
}

__global__ void view_gbuffer_kernel(int w, int h, const float* __restrict__ pos, const float* __restrict__ nrm,
                                    const uint8_t* __restrict__ mask, const View16 V, float* __restrict__ vpos,
                                    float* __restrict__ vnrm, float* __restrict__ vdepth) {
    const size_t n = (size_t)w * h;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float px = 0.0f, py = 0.0f, pz = 0.0f, nx = 0.0f, ny = 0.0f, nz = 0.0f, d = -1.0f;
        if (mask[i]) {
            const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
            const float a = nrm[3 * i], b = nrm[3 * i + 1], c = nrm[3 * i + 2];
            px = row4(V.m + 0, x, y, z, 1.0f);
            py = row4(V.m + 4, x, y, z, 1.0f);
            pz = row4(V.m + 8, x, y, z, 1.0f);
            const v3 nv = normalize(mk(row4(V.m + 0, a, b, c, 0.0f), row4(V.m + 4, a, b, c, 0.0f), row4(V.m + 8, a, b, c, 0.0f)));
            nx = nv.x; ny = nv.y; nz = nv.z;
            d = -pz;
        }
        vpos[3 * i] = px; vpos[3 * i + 1] = py; vpos[3 * i + 2] = pz;
        vnrm[3 * i] = nx; vnrm[3 * i + 1] = ny; vnrm[3 * i + 2] = nz;
        vdepth[i] = d;
    }
}

struct GtaoArgs {
    int w, h;
    const float* pos;
    const float* nrm;
    const float* depth;
    double tan_half, aspect;
    float radius;
    int slices, steps;
    float* out;
};

__device__ __forceinline__ bool valid_px(const GtaoArgs& a, int x, int y) {
    return x >= 0 && y >= 0 && x < a.w && y < a.h && a.depth[(size_t)y * a.w + x] >= 0.0f;
}

// 1 / depth interpolated bilinearly between the four nearest pixel centres, or the nearest
// pixel's depth when one of them is empty or they differ by more than 10 % (post_gtao.cpp:14-33).
// (fx, fy) = (x0 + rx, y0 + ry): the pixel (x0, y0) of the march and the offset from its corner.
__device__ float sample_depth(const GtaoArgs& a, int px, int py, float rx, float ry, int sx, int sy) {
    const float nearest = a.depth[(size_t)sy * a.w + sx];
    const float gx = rx - 0.5f, gy = ry - 0.5f;
    const float flx = floorf(gx), fly = floorf(gy);
    const int x0 = px + (int)flx, y0 = py + (int)fly;
    const float ax = gx - flx, ay = gy - fly;
    float k[4], lo = 1e30f, hi = 0.0f;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int qx = x0 + (q & 1), qy = y0 + (q >> 1);
        if (!valid_px(a, qx, qy)) return nearest;
        const float d = a.depth[(size_t)qy * a.w + qx];
        lo = fminf(lo, d);
        hi = fmaxf(hi, d);
        k[q] = 1.0f / d;
    }
    if (hi > 1.1f * lo) return nearest;
    const float inv = (k[0] * (1.0f - ax) + k[1] * ax) * (1.0f - ay) + (k[2] * (1.0f - ax) + k[3] * ax) * ay;
    return 1.0f / inv;
}

__device__ __forceinline__ void project_d(const GtaoArgs& a, double px, double py, double pz, double& sx, double& sy) {
    const double w = -pz;
    sx = (px / (w * a.tan_half * a.aspect) * 0.5 + 0.5) * a.w;
    sy = (1.0 - (py / (w * a.tan_half) * 0.5 + 0.5)) * a.h;
}

__global__ void __launch_bounds__(256) gtao_kernel(const GtaoArgs a) {
    const float kPi = 3.14159265358979f;
    const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (x >= a.w || y >= a.h) return;
    const size_t i = (size_t)y * a.w + x;
    const float depth = a.depth[i];
    if (depth < 0.0f) { a.out[i] = 1.0f; return; }
    const float P[3] = {a.pos[3 * i], a.pos[3 * i + 1], a.pos[3 * i + 2]};
    const float N[3] = {a.nrm[3 * i], a.nrm[3 * i + 1], a.nrm[3 * i + 2]};
    const float pl = sqrtf(P[0] * P[0] + P[1] * P[1] + P[2] * P[2]);
    const float V[3] = {-P[0] / pl, -P[1] / pl, -P[2] / pl};
    const float tan_half = (float)a.tan_half, aspect = (float)a.aspect;
    const float rpx = a.radius * a.h / (2.0f * tan_half * depth);
    float T[3] = {1.0f - V[0] * V[0], -V[0] * V[1], -V[0] * V[2]};
    const float tl = sqrtf(T[0] * T[0] + T[1] * T[1] + T[2] * T[2]);
    T[0] /= tl; T[1] /= tl; T[2] /= tl;
    const float B[3] = {V[1] * T[2] - V[2] * T[1], V[2] * T[0] - V[0] * T[2], V[0] * T[1] - V[1] * T[0]};
    double sx0, sy0;
    project_d(a, P[0], P[1], P[2], sx0, sy0);
    // the pixel's view-space position recomputed from its centre is what the samples are
    // compared against: S (below) minus P
    float sum = 0.0f;
    for (int s = 0; s < a.slices; ++s) {
        float sp, cp;
        sincospif((s + 0.5f) / a.slices, &sp, &cp);
        const float dir[3] = {cp * T[0] + sp * B[0], cp * T[1] + sp * B[1], cp * T[2] + sp * B[2]};
        const double e = 1e-3 * (double)depth;
        double sx1, sy1;
        project_d(a, P[0] + dir[0] * e, P[1] + dir[1] * e, P[2] + dir[2] * e, sx1, sy1);
        const double ddl = hypot(sx1 - sx0, sy1 - sy0);
        if (ddl < 1e-12) continue;
        const float c = (float)((sx1 - sx0) / ddl), sn = (float)((sy1 - sy0) / ddl);
        const float dv = dir[0] * V[0] + dir[1] * V[1] + dir[2] * V[2];
        const float od[3] = {dir[0] - dv * V[0], dir[1] - dv * V[1], dir[2] - dv * V[2]};
        float ax[3] = {od[1] * V[2] - od[2] * V[1], od[2] * V[0] - od[0] * V[2], od[0] * V[1] - od[1] * V[0]};
        const float al = sqrtf(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
        ax[0] /= al; ax[1] /= al; ax[2] /= al;
        const float na = N[0] * ax[0] + N[1] * ax[1] + N[2] * ax[2];
        const float pn[3] = {N[0] - ax[0] * na, N[1] - ax[1] * na, N[2] - ax[2] * na};
        const float pnl = sqrtf(pn[0] * pn[0] + pn[1] * pn[1] + pn[2] * pn[2]);
        if (pnl < 1e-9f) continue;
        const float sgn = (od[0] * pn[0] + od[1] * pn[1] + od[2] * pn[2]) >= 0.0f ? 1.0f : -1.0f;
        const float cn = fminf(fmaxf((pn[0] * V[0] + pn[1] * V[1] + pn[2] * V[2]) / pnl, 0.0f), 1.0f);
        const float nang = sgn * acosf(cn);
        float hc[2] = {cosf(nang + kPi / 2), cosf(nang - kPi / 2)};
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const float sd = side == 0 ? 1.0f : -1.0f;
            for (int k = 1; k <= a.steps; ++k) {
                const float off = sd * rpx * k / a.steps;
                // the sample relative to the pixel's corner: fx = x + rx
                const float rx = 0.5f + off * c, ry = 0.5f + off * sn;
                const float frx = floorf(rx), fry = floorf(ry);
                const int sx = x + (int)frx, sy = y + (int)fry;
                if (!valid_px(a, sx, sy) || (sx == x && sy == y)) continue;
                const float D = sample_depth(a, x, y, rx, ry, sx, sy);
                const float fx = (float)x + rx, fy = (float)y + ry;
                const float S[3] = {(fx / a.w * 2.0f - 1.0f) * D * tan_half * aspect, (1.0f - fy / a.h * 2.0f) * D * tan_half, -D};
                const float d[3] = {S[0] - P[0], S[1] - P[1], S[2] - P[2]};
                const float dl = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                if (dl < 1e-9f || dl > a.radius) continue;
                hc[side] = fmaxf(hc[side], (d[0] * V[0] + d[1] * V[1] + d[2] * V[2]) / dl);
            }
        }
        const float h1 = nang + fminf(acosf(fminf(fmaxf(hc[0], -1.0f), 1.0f)) - nang, kPi / 2);
        const float h0 = nang + fmaxf(-acosf(fminf(fmaxf(hc[1], -1.0f), 1.0f)) - nang, -kPi / 2);
        const float sn2 = sinf(nang);
        const float a0 = (cn + 2.0f * h0 * sn2 - cosf(2.0f * h0 - nang)) * 0.25f;
        const float a1 = (cn + 2.0f * h1 * sn2 - cosf(2.0f * h1 - nang)) * 0.25f;
        sum += pnl * (a0 + a1);
    }
    a.out[i] = sum / a.slices;
}

}  // namespace

int launch_gtao(int w, int h, const float* pos, const float* nrm, const uint8_t* mask, const float* view16,
                float fovy, float radius, int slices, int steps, float* vpos, float* vnrm, float* vdepth, float* out,
                cudaStream_t s) {
    View16 V;
    for (int k = 0; k < 16; ++k) V.m[k] = view16[k];
    const size_t n = (size_t)w * h;
    const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 65535u * 8);
    view_gbuffer_kernel<<<blocks, 256, 0, s>>>(w, h, pos, nrm, mask, V, vpos, vnrm, vdepth);
    GtaoArgs a{w, h, vpos, vnrm, vdepth, std::tan(0.5 * (double)fovy), (double)((float)w / (float)h), radius, slices,
               steps, out};
    gtao_kernel<<<dim3((w + 15) / 16, (h + 15) / 16), 256, 0, s>>>(a);
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}

}  // namespace rn
