// raster.cu -- the G-buffer the AO passes read, on the GPU: raw-native's CPU rasterizer
// (src/renderer/raster.cpp:9-126, default RasterOptions), bit for bit, for any triangle count.
//
// The reference walks triangles in scene order and, inside each triangle's pixel box, keeps
// a fragment when its screen-linear depth is below the pixel's current one. The surviving
// fragment of a pixel is therefore the first triangle, in scene order, among those with the
// smallest depth there: the minimum of the key (depth bits, record index), since positive
// floats order like their bit patterns. That minimum does not depend on the order fragments
// arrive in, so the GPU rasterizes in bins and keeps it with a 64-bit atomicMin:
//
//   1. set-up, one thread per triangle: clip-space transform, near-plane clip into at most
//      two triangles, perspective divide, screen mapping, area, pixel box -> two record
//      slots per triangle (slot order = scene order);
//   2. count each record's 8 x 8 pixel tiles, prefix sum, emit (record, tile) pairs;
//   3. one thread per pixel of each pair: edge weights, depth, atomicMin(key);
//   4. resolve, one thread per pixel: the winning record's weights again, then position and
//      normal interpolated exactly as the reference does.
// Every float operation of steps 1, 3 and 4 is one IEEE rounding in the reference's order.
#include "rn_internal.h"
#include "rn_device.cuh"

namespace rn {

int scan_exclusive_u32(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* bsum, uint32_t* total, cudaStream_t s);

namespace {

constexpr int kBin = 8;     // bin edge in pixels

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
        T.invw[k] = frcp(v[k].cs[3]);
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

__device__ __forceinline__ uint32_t tiles_of(const RasterTri& T) {
    if (T.minx > T.maxx || T.miny > T.maxy) return 0;
    return (uint32_t)((T.maxx / kBin - T.minx / kBin + 1) * (T.maxy / kBin - T.miny / kBin + 1));
}

__global__ void count_tiles(const RasterTri* __restrict__ recs, uint32_t nrec, uint32_t* __restrict__ cnt) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nrec) cnt[r] = tiles_of(recs[r]);
}

// One (record, bin) pair per entry: bin index in the low 32 bits of the pair's tile word.
__global__ void emit_pairs(const RasterTri* __restrict__ recs, uint32_t nrec, const uint32_t* __restrict__ off,
                           uint2* __restrict__ pairs, uint32_t cap) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    const RasterTri& T = recs[r];
    const uint32_t n = tiles_of(T);
    if (!n) return;
    const int bx0 = T.minx / kBin, bx1 = T.maxx / kBin, by0 = T.miny / kBin, by1 = T.maxy / kBin;
    uint32_t o = off[r];
    for (int by = by0; by <= by1; ++by)
        for (int bx = bx0; bx <= bx1; ++bx) {
            if (o < cap) pairs[o] = make_uint2(r, ((uint32_t)by << 16) | (uint32_t)bx);
            ++o;
        }
}

// raster.cpp:58-63: the edge weights of pixel (x, y) in record T; false when outside.
__device__ __forceinline__ bool weights(const RasterTri& T, int x, int y, float& w0, float& w1, float& w2) {
    const float px = fadd((float)x, 0.5f), py = fadd((float)y, 0.5f);
    w0 = fdiv(fsub(fmul(fsub(T.sx[1], px), fsub(T.sy[2], py)), fmul(fsub(T.sy[1], py), fsub(T.sx[2], px))), T.area);
    w1 = fdiv(fsub(fmul(fsub(T.sx[2], px), fsub(T.sy[0], py)), fmul(fsub(T.sy[2], py), fsub(T.sx[0], px))), T.area);
    w2 = fsub(fsub(1.0f, w0), w1);
    return !(w0 < 0.0f || w1 < 0.0f || w2 < 0.0f);
}
__device__ __forceinline__ float frag_depth(const RasterTri& T, float w0, float w1, float w2) {
    return fadd(fadd(fmul(w0, T.sz[0]), fmul(w1, T.sz[1])), fmul(w2, T.sz[2]));
}

// 64 threads per pair (one per pixel of the 8 x 8 bin), four pairs per block.
__global__ void raster_pairs(const RasterTri* __restrict__ recs, const uint2* __restrict__ pairs, uint32_t npairs,
                             int w, unsigned long long* __restrict__ keys) {
    const uint32_t pi = blockIdx.x * 4 + threadIdx.x / 64;
    if (pi >= npairs) return;
    const uint2 pr = pairs[pi];
    const RasterTri& T = recs[pr.x];
    const int x = (int)(pr.y & 0xFFFFu) * kBin + (int)(threadIdx.x & 7u);
    const int y = (int)(pr.y >> 16) * kBin + (int)((threadIdx.x >> 3) & 7u);
    if (x < T.minx || x > T.maxx || y < T.miny || y > T.maxy) return;
    float w0, w1, w2;
    if (!weights(T, x, y, w0, w1, w2)) return;
    const float d = frag_depth(T, w0, w1, w2);
    const unsigned long long key = ((unsigned long long)__float_as_uint(d) << 32) | pr.x;
    atomicMin(keys + (size_t)y * w + x, key);
}

// raster.cpp:64-80 for the surviving fragment of each pixel.
__global__ void raster_resolve(const RasterTri* __restrict__ recs, const unsigned long long* __restrict__ keys, int w,
                               int h, float* __restrict__ depth, float* __restrict__ pos, float* __restrict__ nrm,
                               uint8_t* __restrict__ mask, const float* __restrict__ albedo_tri,
                               float* __restrict__ albedo) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const size_t i = (size_t)y * w + x;
    const unsigned long long key = keys[i];
    if (key == ~0ull) {
        if (depth) depth[i] = __int_as_float(0x7f800000);
        pos[3 * i] = pos[3 * i + 1] = pos[3 * i + 2] = 0.0f;
        nrm[3 * i] = nrm[3 * i + 1] = nrm[3 * i + 2] = 0.0f;
        if (albedo) albedo[3 * i] = albedo[3 * i + 1] = albedo[3 * i + 2] = 0.0f;
        mask[i] = 0;
        return;
    }
    const uint32_t rec = (uint32_t)(key & 0xFFFFFFFFull);
    const RasterTri& T = recs[rec];
    if (albedo) {                   // a record's triangle is rec / 2 (two record slots per triangle)
        const float* a = albedo_tri + 3 * (size_t)(rec >> 1);
        albedo[3 * i] = a[0]; albedo[3 * i + 1] = a[1]; albedo[3 * i + 2] = a[2];
    }
    float w0, w1, w2;
    weights(T, x, y, w0, w1, w2);
    if (depth) depth[i] = frag_depth(T, w0, w1, w2);
    const float iw = fadd(fadd(fmul(w0, T.invw[0]), fmul(w1, T.invw[1])), fmul(w2, T.invw[2]));
    float P[3], N[3];
    for (int a = 0; a < 3; ++a) {
        P[a] = fdiv(fadd(fadd(fmul(fmul(w0, T.wp[a]), T.invw[0]), fmul(fmul(w1, T.wp[3 + a]), T.invw[1])),
                         fmul(fmul(w2, T.wp[6 + a]), T.invw[2])), iw);
        N[a] = fdiv(fadd(fadd(fmul(fmul(w0, T.wn[a]), T.invw[0]), fmul(fmul(w1, T.wn[3 + a]), T.invw[1])),
                         fmul(fmul(w2, T.wn[6 + a]), T.invw[2])), iw);
    }
    const v3 nn = normalize(mk(N[0], N[1], N[2]));
    pos[3 * i] = P[0]; pos[3 * i + 1] = P[1]; pos[3 * i + 2] = P[2];
    nrm[3 * i] = nn.x; nrm[3 * i + 1] = nn.y; nrm[3 * i + 2] = nn.z;
    mask[i] = 1;
}

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

// Scratch layout: records (2 per triangle), tile counts and offsets, scan block sums, the
// pair total, the per-pixel keys, then the pairs.
size_t raster_scratch_bytes(uint32_t ntri, size_t npx, size_t npairs) {
    const size_t nrec = 2 * (size_t)ntri;
    return align256(nrec * sizeof(RasterTri)) + 2 * align256(nrec * 4 + 4) + align256(((nrec + 2047) / 2048 + 1) * 8) +
           256 + align256(npx * 8) + align256(npairs * sizeof(uint2));
}

int launch_raster(const float* tris, const float* nrm, uint32_t ntri, const float* d_vp, float nearZ, int w, int h,
                  char* scratch, size_t scratch_bytes, float* depth, float* pos, float* nrmo, uint8_t* mask,
                  cudaStream_t s, size_t* pairs_needed, const float* albedo_tri, float* albedo) {
    const uint32_t nrec = 2 * ntri;
    const size_t npx = (size_t)w * h;
    size_t off = 0;
    auto take = [&](size_t b) { char* p = scratch + off; off += align256(b); return p; };
    RasterTri* recs = (RasterTri*)take((size_t)nrec * sizeof(RasterTri));
    uint32_t* cnt = (uint32_t*)take((size_t)nrec * 4 + 4);
    uint32_t* ofs = (uint32_t*)take((size_t)nrec * 4 + 4);
    uint32_t* bsum = (uint32_t*)take(((size_t)(nrec + 2047) / 2048 + 1) * 8);
    uint32_t* total = (uint32_t*)take(256);
    unsigned long long* keys = (unsigned long long*)take(npx * 8);
    uint2* pairs = (uint2*)(scratch + off);
    const size_t cap = off < scratch_bytes ? (scratch_bytes - off) / sizeof(uint2) : 0;
    uint32_t npairs = 0;
    if (cudaMemsetAsync(keys, 0xFF, npx * 8, s) != cudaSuccess) return RN_ERR_CUDA;
    if (ntri) {
        raster_setup<<<(ntri + 127) / 128, 128, 0, s>>>(tris, nrm, ntri, d_vp, nearZ, w, h, recs);
        count_tiles<<<(nrec + 255) / 256, 256, 0, s>>>(recs, nrec, cnt);
        scan_exclusive_u32(cnt, ofs, nrec, bsum, total, s);
        if (cudaMemcpyAsync(&npairs, total, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return RN_ERR_CUDA;
        if (npairs > cap) { *pairs_needed = npairs; return RN_ERR_NO_MEMORY; }
        emit_pairs<<<(nrec + 255) / 256, 256, 0, s>>>(recs, nrec, ofs, pairs, (uint32_t)cap);
        if (npairs) raster_pairs<<<(npairs + 3) / 4, 256, 0, s>>>(recs, pairs, npairs, w, keys);
    }
    const dim3 blk(32, 8), grid((w + 31) / 32, (h + 7) / 8);
    raster_resolve<<<grid, blk, 0, s>>>(recs, keys, w, h, depth, pos, nrmo, mask, albedo_tri, albedo);
    *pairs_needed = npairs;
    return cudaGetLastError() == cudaSuccess ? RN_OK : RN_ERR_CUDA;
}

}  // namespace rn
