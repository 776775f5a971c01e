// raster.cu -- the G-buffer the AO passes read, on the GPU: raw-native's CPU rasterizer
// (src/renderer/raster.cpp:9-126, default RasterOptions) restated per pixel.
//
// The reference walks triangles in scene order and, inside each triangle's pixel box,
// keeps a fragment when its screen-linear depth is below the pixel's current one. A pixel's
// final state depends only on that order and those comparisons, so here one thread per
// pixel walks the same triangle list in the same order: the winner, its depth, and the
// position and normal interpolated for it are the reference's, bit for bit (every
// operation is one IEEE rounding in the reference's order).
//
// Triangle set-up (clip-space transform, near-plane clip into at most two triangles,
// perspective divide, screen mapping, area, pixel box) runs once per triangle into two
// fixed record slots, so record order is scene order.
#include "rn_internal.h"
#include "rn_device.cuh"

namespace rn {
namespace {

struct ClipV { float cs[4]; v3 wp, wn; };

struct RasterTri {
    float sx[3], sy[3], sz[3];
    float invw[3];
    float wp[9], wn[9];
    float area;
    int minx, maxx, miny, maxy;    // minx > maxx: no pixels
};

__device__ __forceinline__ ClipV lerp_v(const ClipV& a, const ClipV& b, float t) {
    ClipV r;
    for (int k = 0; k < 4; ++k) r.cs[k] = fadd(a.cs[k], fmul(fsub(b.cs[k], a.cs[k]), t));
    r.wp = mk(fadd(a.wp.x, fmul(fsub(b.wp.x, a.wp.x), t)), fadd(a.wp.y, fmul(fsub(b.wp.y, a.wp.y), t)),
              fadd(a.wp.z, fmul(fsub(b.wp.z, a.wp.z), t)));
    r.wn = mk(fadd(a.wn.x, fmul(fsub(b.wn.x, a.wn.x), t)), fadd(a.wn.y, fmul(fsub(b.wn.y, a.wn.y), t)),
              fadd(a.wn.z, fmul(fsub(b.wn.z, a.wn.z), t)));
    return r;
}

// raster.cpp:30-57: drawTri's set-up.
__device__ void setup_tri(const ClipV v[3], int w, int h, RasterTri& T) {
    T.minx = 1; T.maxx = 0; T.miny = 1; T.maxy = 0;
    for (int k = 0; k < 3; ++k) {
        T.invw[k] = fdiv(1.0f, v[k].cs[3]);
        const float nx = fmul(v[k].cs[0], T.invw[k]), ny = fmul(v[k].cs[1], T.invw[k]);
        T.sx[k] = fadd(fmul(fadd(fmul(nx, 0.5f), 0.5f), (float)w), 0.0f);
        T.sy[k] = fadd(fmul(fsub(1.0f, fadd(fmul(ny, 0.5f), 0.5f)), (float)h), 0.0f);
        T.sz[k] = v[k].cs[3];
        T.wp[3 * k] = v[k].wp.x; T.wp[3 * k + 1] = v[k].wp.y; T.wp[3 * k + 2] = v[k].wp.z;
        T.wn[3 * k] = v[k].wn.x; T.wn[3 * k + 1] = v[k].wn.y; T.wn[3 * k + 2] = v[k].wn.z;
    }
    const float mnx = smin(smin(T.sx[0], T.sx[1]), T.sx[2]), mxx = smax(smax(T.sx[0], T.sx[1]), T.sx[2]);
    const float mny = smin(smin(T.sy[0], T.sy[1]), T.sy[2]), mxy = smax(smax(T.sy[0], T.sy[1]), T.sy[2]);
    T.area = fsub(fmul(fsub(T.sx[1], T.sx[0]), fsub(T.sy[2], T.sy[0])), fmul(fsub(T.sy[1], T.sy[0]), fsub(T.sx[2], T.sx[0])));
    if (fabsf(T.area) < 1e-9f) return;
    // (int)floor / (int)ceil of values far outside the frame saturate; clamp before converting
    const float fx0 = fmaxf(floorf(mnx), -1.0f), fx1 = fminf(ceilf(mxx), (float)w);
    const float fy0 = fmaxf(floorf(mny), -1.0f), fy1 = fminf(ceilf(mxy), (float)h);
    T.minx = max(0, (int)fx0);
    T.maxx = min(w - 1, (int)fx1);
    T.miny = max(0, (int)fy0);
    T.maxy = min(h - 1, (int)fy1);
}

// raster.cpp:103-123: clip-space vertices, near clip, up to two records per triangle.
__global__ void raster_setup(const float* __restrict__ tris, const float* __restrict__ nrm, uint32_t n,
                             const float* __restrict__ vp, float nearZ, int w, int h, RasterTri* __restrict__ out) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    ClipV v[3];
    bool behind = false;
    for (int k = 0; k < 3; ++k) {
        const float* p = tris + (size_t)t * 9 + 3 * k;
        const float* q = nrm + (size_t)t * 9 + 3 * k;
        for (int r = 0; r < 4; ++r) {
            const float* m = vp + 4 * r;
            v[k].cs[r] = fadd(fadd(fadd(fmul(m[0], p[0]), fmul(m[1], p[1])), fmul(m[2], p[2])), fmul(m[3], 1.0f));
        }
        v[k].wp = mk(p[0], p[1], p[2]);
        v[k].wn = mk(q[0], q[1], q[2]);
        behind = behind || v[k].cs[3] <= 1e-6f;
    }
    RasterTri& A = out[2 * (size_t)t];
    RasterTri& B = out[2 * (size_t)t + 1];
    A.minx = B.minx = 1;
    A.maxx = B.maxx = 0;
    if (!behind) { setup_tri(v, w, h, A); return; }
    ClipV c[4];
    int m = 0;
    for (int k = 0; k < 3; ++k) {
        const ClipV& a = v[k];
        const ClipV& b = v[(k + 1) % 3];
        const bool ain = a.cs[3] >= nearZ, bin = b.cs[3] >= nearZ;
        if (ain) c[m++] = a;
        if (ain != bin) c[m++] = lerp_v(a, b, fdiv(fsub(nearZ, a.cs[3]), fsub(b.cs[3], a.cs[3])));
    }
    for (int k = 1; k + 1 < m; ++k) {
        const ClipV tv[3] = {c[0], c[k], c[k + 1]};
        setup_tri(tv, w, h, k == 1 ? A : B);
    }
}

// raster.cpp:58-81 per pixel, triangles in scene order.
__global__ void raster_pixels(const RasterTri* __restrict__ recs, uint32_t nrec, int w, int h, float* __restrict__ depth,
                              float* __restrict__ pos, float* __restrict__ nrm, uint8_t* __restrict__ mask) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const float px = fadd((float)x, 0.5f), py = fadd((float)y, 0.5f);
    float best = __int_as_float(0x7f800000);
    int win = -1;
    float bw0 = 0.0f, bw1 = 0.0f, bw2 = 0.0f;
    for (uint32_t r = 0; r < nrec; ++r) {
        const RasterTri& T = recs[r];
        if (x < T.minx || x > T.maxx || y < T.miny || y > T.maxy) continue;
        const float w0 = fdiv(fsub(fmul(fsub(T.sx[1], px), fsub(T.sy[2], py)), fmul(fsub(T.sy[1], py), fsub(T.sx[2], px))), T.area);
        const float w1 = fdiv(fsub(fmul(fsub(T.sx[2], px), fsub(T.sy[0], py)), fmul(fsub(T.sy[2], py), fsub(T.sx[0], px))), T.area);
        const float w2 = fsub(fsub(1.0f, w0), w1);
        if (w0 < 0.0f || w1 < 0.0f || w2 < 0.0f) continue;
        const float d = fadd(fadd(fmul(w0, T.sz[0]), fmul(w1, T.sz[1])), fmul(w2, T.sz[2]));
        if (d >= best) continue;
        best = d; win = (int)r; bw0 = w0; bw1 = w1; bw2 = w2;
    }
    const size_t i = (size_t)y * w + x;
    depth[i] = best;
    if (win < 0) {
        pos[3 * i] = pos[3 * i + 1] = pos[3 * i + 2] = 0.0f;
        nrm[3 * i] = nrm[3 * i + 1] = nrm[3 * i + 2] = 0.0f;
        mask[i] = 0;
        return;
    }
    const RasterTri& T = recs[win];
    const float iw = fadd(fadd(fmul(bw0, T.invw[0]), fmul(bw1, T.invw[1])), fmul(bw2, T.invw[2]));
    float P[3], N[3];
    for (int a = 0; a < 3; ++a) {
        P[a] = fdiv(fadd(fadd(fmul(fmul(bw0, T.wp[a]), T.invw[0]), fmul(fmul(bw1, T.wp[3 + a]), T.invw[1])),
                         fmul(fmul(bw2, T.wp[6 + a]), T.invw[2])), iw);
        N[a] = fdiv(fadd(fadd(fmul(fmul(bw0, T.wn[a]), T.invw[0]), fmul(fmul(bw1, T.wn[3 + a]), T.invw[1])),
                         fmul(fmul(bw2, T.wn[6 + a]), T.invw[2])), iw);
    }
    const v3 nn = normalize(mk(N[0], N[1], N[2]));
    pos[3 * i] = P[0]; pos[3 * i + 1] = P[1]; pos[3 * i + 2] = P[2];
    nrm[3 * i] = nn.x; nrm[3 * i + 1] = nn.y; nrm[3 * i + 2] = nn.z;
    mask[i] = 1;
}

}  // namespace

size_t raster_records_bytes(uint32_t ntri) { return (size_t)2 * ntri * sizeof(RasterTri); }

int launch_raster(const float* tris, const float* nrm, uint32_t ntri, const float* d_vp, float nearZ, int w, int h,
                  void* records, float* depth, float* pos, float* nrmo, uint8_t* mask, cudaStream_t s) {
    RasterTri* recs = (RasterTri*)records;
    if (ntri) raster_setup<<<(ntri + 127) / 128, 128, 0, s>>>(tris, nrm, ntri, d_vp, nearZ, w, h, recs);
    const dim3 blk(32, 8), grid((w + 31) / 32, (h + 7) / 8);
    raster_pixels<<<grid, blk, 0, s>>>(recs, 2 * ntri, w, h, depth, pos, nrmo, mask);
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}

}  // namespace rn
