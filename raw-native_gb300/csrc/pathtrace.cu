// pathtrace.cu -- raw-native's path tracer (interface v4, v2 scenes) on the GPU, bit for bit.
//
// The reference: raw::rt::pathTraceCpu (src/renderer/rt_pt_cpu.cpp) over the scene queries
// and next-event estimation of src/renderer/rt_pt_ctx.hpp and the random numbers and lobe of
// src/renderer/rt_pt_math.hpp; its GPU counterpart is raw::gpu_check::pathTraceGpu
// (raw/renderer/rt_pt_gpu.hpp, a WGSL pass), judged there only statistically. Here every
// AOV equals the CPU's bytes:
//   - every float32 operation is the CPU's, in its order, one rounding each (the explicit
//     round-to-nearest intrinsics of rn_device.cuh; no contraction);
//   - the sampler angles 2 pi u (u = k / 2^24 from PCG2D) take their cos and sin from the
//     device function plus the host libm's correction table (the AO sampler's: the same
//     2^24 angles);
//   - the closest hit is rt::closest's (nearest t, ties to the lowest triangle index; the
//     4-wide walk of trace_device.cuh) and visibility its any-hit answer;
//   - the lobe's energy table is built on the host in float64 exactly as
//     src/renderer/rt_pt_energy.cpp builds it, then read on the device;
//   - per pixel the samples are summed in sample order and the moments kept in float64.
//
// Code size: the walks, the surface query, the lobe's evaluation and its energy terms are
// called from several places of a path's bounce; they are kept out of line (one copy each)
// so that the kernel fits the instruction cache (inlined, fetch stalls dominated).
//
// Work: samples of a slice are traced in parallel, one thread per (pixel, sample), a warp
// on an 8 x 4 pixel tile for one sample index (coherent primary rays); each sample's eight
// colour terms go to a slice buffer, and a second kernel adds them per pixel in sample
// order into running sums that persist across slices (the CPU's loop order, so any slice
// size gives the same bits). The last slice's pass also scales the sums, forms the
// variances and traces the pixel-centre ray (depth, triangle, motion).
#include "rn_internal.h"
#include "rn_device.cuh"
#include "trace_device.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

struct rn_ptscene {
    int device = -1;
    uint32_t nvert = 0, ntri = 0, ntex = 0, ntexels = 0, nemit = 0;
    float area = 0.0f;
    float sun_dir[3] = {0, 0, 0}, sun_irr[3] = {0, 0, 0}, sky[3] = {0, 0, 0};
    void* block = nullptr;     // one device allocation holding every array below
    float* nrm = nullptr;      // 3 a vertex
    float* uv = nullptr;       // 2 a vertex
    uint32_t* idx = nullptr;   // 3 a triangle
    uint32_t* tritex = nullptr;
    uint32_t* texent = nullptr;
    uint32_t* texels = nullptr;
    float* mat = nullptr;      // 7 a texture
    float* tris = nullptr;     // 9 a triangle, input order (trianglesOf)
    uint32_t* emit = nullptr;
    float* cdf = nullptr;
    rn_accel* accel = nullptr;
};

namespace rn {
namespace {

using namespace trace_dev;

constexpr int kMu = 64, kRough = 128;
constexpr int kNodes = kMu * kRough * 2, kTableFloats = kNodes + kRough * 2;
constexpr float kPiF = 3.14159265f;

// ================================================================ the energy table (host, float64)
// src/renderer/rt_pt_energy.cpp:11-40 with the split albedo of src/renderer/pbr_tables.cpp:23-50
// and the Gauss-Legendre nodes of src/renderer/brdf.cpp:95-109. Host code is built without
// contraction (-ffp-contract=off), as the reference's is.
constexpr double kPiD = 3.14159265358979323846;

double radical_inverse(uint32_t b) {
    b = (b << 16) | (b >> 16);
    b = ((b & 0x55555555u) << 1) | ((b & 0xAAAAAAAAu) >> 1);
    b = ((b & 0x33333333u) << 2) | ((b & 0xCCCCCCCCu) >> 2);
    b = ((b & 0x0F0F0F0Fu) << 4) | ((b & 0xF0F0F0F0u) >> 4);
    b = ((b & 0x00FF00FFu) << 8) | ((b & 0xFF00FF00u) >> 8);
    return b * 2.3283064365386963e-10;
}
double lambda_d(double mu, double a) {
    const double m2 = mu * mu;
    return 0.5 * (-1.0 + std::sqrt(1.0 + a * a * (1.0 - m2) / m2));
}
void albedo_split(double mu, double a, int n, double& outA, double& outB) {
    const double vx = std::sqrt(std::max(0.0, 1.0 - mu * mu)), vy = 0.0, vz = mu;
    const double hx = a * vx, hz = vz;
    const double lv = std::sqrt(hx * hx + hz * hz);
    const double nx = hx / lv, ny = 0.0, nz = hz / lv;
    const double t1x = 0.0, t1y = 1.0, t1z = 0.0;
    const double t2x = ny * t1z - nz * t1y, t2y = nz * t1x - nx * t1z, t2z = nx * t1y - ny * t1x;
    const double g1 = 1.0 / (1.0 + lambda_d(mu, a));
    double sa = 0.0, sb = 0.0;
    for (int k = 0; k < n; ++k) {
        const double u1 = (k + 0.5) / n, u2 = radical_inverse((uint32_t)k);
        const double r = std::sqrt(u1), phi = 2.0 * kPiD * u2, s = 0.5 * (1.0 + nz);
        const double p1 = r * std::cos(phi), p2 = (1.0 - s) * std::sqrt(1.0 - p1 * p1) + s * r * std::sin(phi);
        const double p3 = std::sqrt(std::max(0.0, 1.0 - p1 * p1 - p2 * p2));
        double mx = t1x * p1 + t2x * p2 + nx * p3, my = t1y * p1 + t2y * p2 + ny * p3, mz = t1z * p1 + t2z * p2 + nz * p3;
        mx = a * mx; my = a * my; mz = std::max(1e-12, mz);
        const double lm = std::sqrt(mx * mx + my * my + mz * mz);
        mx = mx / lm; my = my / lm; mz = mz / lm;
        const double vom = vx * mx + vy * my + vz * mz, li = 2.0 * vom * mz - vz;
        if (li <= 0.0) continue;
        const double w = (1.0 / (1.0 + lambda_d(mu, a) + lambda_d(li, a))) / g1;
        const double c = 1.0 - vom, c5 = c * c * c * c * c;
        sa += w * (1.0 - c5); sb += w * c5;
    }
    outA = sa / n; outB = sb / n;
}
void gauss_legendre01(int n, std::vector<double>& x, std::vector<double>& w) {
    x.assign(n, 0.0); w.assign(n, 0.0);
    for (int i = 0; i < n; ++i) {
        double z = std::cos(kPiD * (i + 0.75) / (n + 0.5)), pp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p1 = 1.0, p2 = 0.0;
            for (int j = 1; j <= n; ++j) { const double p3 = p2; p2 = p1; p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j; }
            pp = n * (z * p1 - p2) / (z * z - 1.0);
            const double z1 = z;
            z = z1 - p1 / pp;
            if (std::fabs(z - z1) < 1e-15) break;
        }
        x[i] = 0.5 * (1.0 - z); w[i] = 1.0 / ((1.0 - z * z) * pp * pp);
    }
}
// rt_pt_math.hpp:93-107 on the host (the means are formed from the float table as read).
void table_ab_host(const float* t, float mu, float rough, float& A, float& B) {
    const float x = std::sqrt(std::clamp(mu, 0.0f, 1.0f)) * float(kMu - 1), y = std::clamp(rough, 0.0f, 1.0f) * float(kRough - 1);
    const int x0 = std::min(int(x), kMu - 2), y0 = std::min(int(y), kRough - 2);
    const float fx = x - float(x0), fy = y - float(y0);
    const float* p = t + (std::size_t(y0) * kMu + std::size_t(x0)) * 2;
    const float* q = p + std::size_t(kMu) * 2;
    const float a0 = p[0] * (1.0f - fx) + p[2] * fx, b0 = p[1] * (1.0f - fx) + p[3] * fx;
    const float a1 = q[0] * (1.0f - fx) + q[2] * fx, b1 = q[1] * (1.0f - fx) + q[3] * fx;
    A = a0 * (1.0f - fy) + a1 * fy; B = b0 * (1.0f - fy) + b1 * fy;
}
const std::vector<float>& energy_table_host() {
    static std::vector<float> t;
    static std::once_flag once;
    std::call_once(once, [] {
        t.assign(kTableFloats, 0.0f);
        // rows are independent and each is written by one thread: identical for any count
        const int threads = (int)std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        for (int th = 0; th < threads; ++th)
            pool.emplace_back([th, threads] {
                for (int i = th; i < kRough; i += threads) {
                    const double r = double(i) / (kRough - 1), a = std::max(1e-4, r * r);
                    for (int j = 0; j < kMu; ++j) {
                        const double u = double(j) / (kMu - 1), mu = std::max(u * u, 1e-4);
                        double A = 0.0, B = 0.0;
                        albedo_split(mu, a, 1 << 12, A, B);
                        t[(std::size_t(i) * kMu + std::size_t(j)) * 2] = float(A);
                        t[(std::size_t(i) * kMu + std::size_t(j)) * 2 + 1] = float(B);
                    }
                }
            });
        for (auto& p : pool) p.join();
        std::vector<double> x, w;
        gauss_legendre01(64, x, w);
        for (int i = 0; i < kRough; ++i) {
            const float r = float(i) / float(kRough - 1);
            double sa = 0.0, sb = 0.0;
            for (std::size_t k = 0; k < x.size(); ++k) {
                float A, B;
                table_ab_host(t.data(), float(x[k]), r, A, B);
                sa += w[k] * double(A) * x[k]; sb += w[k] * double(B) * x[k];
            }
            t[kNodes + std::size_t(i) * 2] = float(2.0 * sa);
            t[kNodes + std::size_t(i) * 2 + 1] = float(2.0 * sb);
        }
    });
    return t;
}
// The table on each device, uploaded once (held until the process exits).
std::mutex g_table_mutex;
float* g_table_dev[64] = {};
int device_table(int dev, const float** out, rn_status* st) {
    if (dev < 0 || dev >= 64) return fail(st, RN_ERR_STATE, "device ordinal %d", dev);
    const std::vector<float>& t = energy_table_host();
    std::lock_guard<std::mutex> lock(g_table_mutex);
    if (!g_table_dev[dev]) {
        void* p = nullptr;
        RN_CUDA(cudaMalloc(&p, t.size() * sizeof(float)), st);
        const cudaError_t e = cudaMemcpy(p, t.data(), t.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { cudaFree(p); return cuda_fail(st, e, "energy table upload"); }
        g_table_dev[dev] = (float*)p;
    }
    *out = g_table_dev[dev];
    return RN_OK;
}

// ================================================================ host vector math (camera)
struct hv3 { float x, y, z; };
hv3 hsub(hv3 a, hv3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
float hdot(hv3 a, hv3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
hv3 hcross(hv3 a, hv3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
hv3 hnorm(hv3 v) {
    const float l = std::sqrt(hdot(v, v));
    if (!(l > 0.0f)) return v;
    const float s = 1.0f / l;
    return {v.x * s, v.y * s, v.z * s};
}

// ================================================================ device
struct PtCam { v3 eye, f, s, u; float th, aspect; };

// rt_pt_cpu.cpp:14-20 on the host (std::tan of a float: the host libm's tanf).
PtCam cam_of(const float* c, int w, int h) {
    PtCam k;
    const hv3 eye{c[0], c[1], c[2]}, tgt{c[3], c[4], c[5]}, up{c[6], c[7], c[8]};
    const hv3 f = hnorm(hsub(tgt, eye)), s = hnorm(hcross(f, up)), u = hcross(s, f);
    k.eye = v3{eye.x, eye.y, eye.z};
    k.f = v3{f.x, f.y, f.z}; k.s = v3{s.x, s.y, s.z}; k.u = v3{u.x, u.y, u.z};
    k.th = std::tan(c[9] * 0.5f);
    k.aspect = float(w) / float(h);
    return k;
}

struct PtParams {
    const Node4* nodes;
    const LeafTri* ltris;
    int has_geometry;
    const float* tris;        // 9 a triangle, input order
    const float* nrm;
    const float* uv;
    const uint32_t* idx;
    const uint32_t* tritex;
    const uint32_t* texent;
    const uint32_t* texels;
    const float* mat;         // 7 a texture
    const uint32_t* emit;
    const float* cdf;
    uint32_t nemit;
    float area;
    const float* table;
    const uint8_t* corr;
    v3 sun_dir, sun_irr, sky;
    uint32_t seed_lo, seed_hi, spp, spp_begin, max_bounces, controls;
    int w, h, jitter, rr;
    PtCam cam, prev;
    uint32_t k0, kn;          // this slice: samples [k0, k0 + kn) of the pixel's spp
    uint32_t npix;
    float* samp;              // kSampleFloats x kn x npix (component-major)
    float* acc;               // kAccFloats x npix running sums (component-major)
    double* mom;              // 6 x npix running moments
    int first, last;          // slice flags
    uint32_t* err;
};
constexpr int kSampleFloats = 24;   // L, D, S, E, alb, nrm, dAlb, sAlb

// ---------------------------------------------------------------- random numbers (rt_pt_math.hpp:18-35)
struct R2 { float a, b; uint32_t ka, kb; };
__device__ __forceinline__ R2 rand2(const PtParams& P, uint32_t pixel, uint32_t sample, uint32_t dim) {
    uint32_t x = pixel ^ (P.seed_lo * 0x9E3779B9u), y = (sample * 64u + dim) ^ P.seed_hi;
    x = x * 1664525u + 1013904223u; y = y * 1664525u + 1013904223u;
    x += y * 1664525u; y += x * 1664525u;
    x ^= x >> 16; y ^= y >> 16;
    x += y * 1664525u; y += x * 1664525u;
    x ^= x >> 16; y ^= y >> 16;
    R2 r;
    r.ka = x >> 8; r.kb = y >> 8;
    r.a = unit24(r.ka); r.b = unit24(r.kb);   // float(k) x 5.96046448e-8f = k / 2^24 exactly
    return r;
}

// ---------------------------------------------------------------- small float helpers
__device__ __forceinline__ v3 mulv(v3 a, v3 b) { return mk(fmul(a.x, b.x), fmul(a.y, b.y), fmul(a.z, b.z)); }
__device__ __forceinline__ float maxc(v3 a) { return smax(a.x, smax(a.y, a.z)); }
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return (v < lo) ? lo : (hi < v) ? hi : v; }
__device__ __forceinline__ float lum(v3 c) { return fadd(fadd(fmul(0.2126f, c.x), fmul(0.7152f, c.y)), fmul(0.0722f, c.z)); }

struct Frame { v3 t, b, n; };
// Duff et al. 2017 (rt_pt_math.hpp:38-42)
__device__ __forceinline__ Frame basis(v3 n) {
    const float s = n.z >= 0.0f ? 1.0f : -1.0f;
    const float a = fdiv(-1.0f, fadd(s, n.z)), c = fmul(fmul(n.x, n.y), a);
    Frame f;
    f.t = mk(fadd(1.0f, fmul(fmul(fmul(s, n.x), n.x), a)), fmul(s, c), -fmul(s, n.x));
    f.b = mk(c, fadd(s, fmul(fmul(n.y, n.y), a)), -n.y);
    f.n = n;
    return f;
}
__device__ __forceinline__ v3 to_local(const Frame& f, v3 v) { return mk(dot(v, f.t), dot(v, f.b), dot(v, f.n)); }
__device__ __forceinline__ v3 to_world(const Frame& f, v3 v) { return add(add(scale(f.t, v.x), scale(f.b, v.y)), scale(f.n, v.z)); }

// ---------------------------------------------------------------- the lobe (rt_pt_math.hpp:45-210)
__device__ __forceinline__ float ggx_d(float a2, float cosH) {
    const float d = fadd(fmul(fmul(cosH, cosH), fsub(a2, 1.0f)), 1.0f);
    return fdiv(a2, fmul(fmul(kPiF, d), d));
}
__device__ __forceinline__ float lambda_f(float a2, float cosT) {
    const float c2 = fmul(cosT, cosT);
    return fmul(fadd(-1.0f, fsqrt(fadd(1.0f, fdiv(fmul(a2, fsub(1.0f, c2)), c2)))), 0.5f);
}
// VNDF sampling (Heitz 2018); u2 = kb / 2^24, so phi is the sampler angle kb.
__device__ __noinline__ v3 sample_vndf(const PtParams& P, v3 wo, float a, float u1, uint32_t kb) {
    const v3 vh = normalize(mk(fmul(a, wo.x), fmul(a, wo.y), wo.z));
    const float lensq = fadd(fmul(vh.x, vh.x), fmul(vh.y, vh.y));
    const v3 t1 = lensq > 0.0f ? scale(mk(-vh.y, vh.x, 0.0f), frcp(fsqrt(lensq))) : mk(1.0f, 0.0f, 0.0f);
    const v3 t2 = cross(vh, t1);
    float cphi, sphi;
    sample_sincos(kb, P.corr, cphi, sphi);
    const float r = fsqrt(u1);
    const float p1 = fmul(r, cphi), s = fmul(0.5f, fadd(1.0f, vh.z));
    const float p2 = fadd(fmul(fsub(1.0f, s), fsqrt(smax(0.0f, fsub(1.0f, fmul(p1, p1))))), fmul(s, fmul(r, sphi)));
    const float q = fsub(fsub(1.0f, fmul(p1, p1)), fmul(p2, p2));
    const v3 nh = add(add(scale(t1, p1), scale(t2, p2)), scale(vh, fsqrt(smax(0.0f, q))));
    return normalize(mk(fmul(a, nh.x), fmul(a, nh.y), smax(0.0f, nh.z)));
}
struct Bsdf { v3 base; float rough, metallic, specular; bool legacy; };
__device__ __forceinline__ float lobe_prob(const Bsdf& m) {
    return fadd(m.metallic, fmul(fmul(fsub(1.0f, m.metallic), 0.5f), m.specular));
}
__device__ __forceinline__ v3 f0_of(const Bsdf& m) {
    const float d = fmul(0.04f, m.specular);
    return mk(fadd(d, fmul(fsub(m.base.x, d), m.metallic)), fadd(d, fmul(fsub(m.base.y, d), m.metallic)),
              fadd(d, fmul(fsub(m.base.z, d), m.metallic)));
}
__device__ __forceinline__ float kms(float favg, float eavg) {
    return fdiv(fmul(fmul(favg, favg), eavg), fsub(1.0f, fmul(favg, fsub(1.0f, eavg))));
}
__device__ __forceinline__ void table_ab(const float* __restrict__ t, float mu, float rough, float& A, float& B) {
    const float x = fmul(fsqrt(clampf(mu, 0.0f, 1.0f)), float(kMu - 1)), y = fmul(clampf(rough, 0.0f, 1.0f), float(kRough - 1));
    const int x0 = min((int)x, kMu - 2), y0 = min((int)y, kRough - 2);
    const float fx = fsub(x, float(x0)), fy = fsub(y, float(y0));
    const float* p = t + ((size_t)y0 * kMu + (size_t)x0) * 2;
    const float* q = p + (size_t)kMu * 2;
    const float gx = fsub(1.0f, fx);
    const float a0 = fadd(fmul(__ldg(p), gx), fmul(__ldg(p + 2), fx)), b0 = fadd(fmul(__ldg(p + 1), gx), fmul(__ldg(p + 3), fx));
    const float a1 = fadd(fmul(__ldg(q), gx), fmul(__ldg(q + 2), fx)), b1 = fadd(fmul(__ldg(q + 1), gx), fmul(__ldg(q + 3), fx));
    const float gy = fsub(1.0f, fy);
    A = fadd(fmul(a0, gy), fmul(a1, fy)); B = fadd(fmul(b0, gy), fmul(b1, fy));
}
__device__ __forceinline__ void table_avg(const float* __restrict__ t, float rough, float& A, float& B) {
    const float y = fmul(clampf(rough, 0.0f, 1.0f), float(kRough - 1));
    const int y0 = min((int)y, kRough - 2);
    const float fy = fsub(y, float(y0)), gy = fsub(1.0f, fy);
    const float* p = t + kNodes + (size_t)y0 * 2;
    A = fadd(fmul(__ldg(p), gy), fmul(__ldg(p + 2), fy)); B = fadd(fmul(__ldg(p + 1), gy), fmul(__ldg(p + 3), fy));
}
// The lobe at one surface point for one outgoing direction: every term of energyOf,
// evalLegacy and evalBsdf (rt_pt_math.hpp:113-183) that does not depend on the incoming
// direction, formed once per bounce instead of once per evaluation (the operations and
// their order are the reference's; only their repetition is gone). The bounce evaluates the
// lobe for three incoming directions (the sun, the sampled emitter point, the sampled
// direction), each also giving its Lambert part (lambertCos, rt_pt_math.hpp:184-190, of the
// same pair).
struct Lobe {
    Bsdf m;
    float ps;                       // lobe_prob
    v3 fd;                          // base x (1 - metallic) / pi
    // specular (ps > 0): F0, f90, a^2, Lambda(wo), G1 = 1 / (1 + Lambda(wo)), 4 wo.z
    v3 F0;
    float f90, a2, lo, G1, four_wo;
    // energy compensation (ps > 0, v4 lobe): the table's terms at mu_o and its average
    float on, d, kd, omeo, den_ms, omeso, omesa;
    bool ms_on;                     // E_avg < 1
    v3 km;
};
__device__ __forceinline__ float km_of(const Bsdf& m, float b, float eavg, float kd) {
    return fadd(fmul(m.metallic, kms(fadd(b, fdiv(fsub(1.0f, b), 21.0f)), eavg)), fmul(fsub(1.0f, m.metallic), kd));
}
__device__ __noinline__ void lobe_setup(const PtParams& P, const Bsdf& m, float woz, Lobe& L) {
    L.m = m;
    L.ps = lobe_prob(m);
    const float kd = fdiv(fsub(1.0f, m.metallic), kPiF);
    L.fd = mk(fmul(m.base.x, kd), fmul(m.base.y, kd), fmul(m.base.z, kd));
    if (!(L.ps > 0.0f)) return;
    L.F0 = f0_of(m);
    L.f90 = fadd(m.metallic, fmul(fsub(1.0f, m.metallic), m.specular > 0.0f ? 1.0f : 0.0f));
    const float a = smax(1e-4f, fmul(m.rough, m.rough));
    L.a2 = fmul(a, a);
    L.lo = lambda_f(L.a2, woz);
    L.G1 = frcp(fadd(1.0f, L.lo));
    L.four_wo = fmul(4.0f, woz);
    if (m.legacy) return;
    float oa, ob, aa, ab;
    table_ab(P.table, woz, m.rough, oa, ob);
    table_avg(P.table, m.rough, aa, ab);
    const float eo = smin(1.0f, fadd(oa, ob)), ea = smin(1.0f, fadd(aa, ab));
    L.ms_on = ea < 1.0f;
    L.omeo = fsub(1.0f, eo);
    L.den_ms = fmul(kPiF, fsub(1.0f, ea));
    L.on = m.specular > 0.0f ? 1.0f : 0.0f;
    L.d = fmul(0.04f, m.specular);
    L.kd = kms(fmul(L.on, fadd(L.d, fdiv(fsub(1.0f, L.d), 21.0f))), ea);
    const float eso = fadd(fmul(L.on, fadd(fmul(L.d, oa), ob)), fmul(L.kd, fsub(1.0f, eo)));
    const float esa = fadd(fmul(L.on, fadd(fmul(L.d, aa), ab)), fmul(L.kd, fsub(1.0f, ea)));
    L.omeso = fsub(1.0f, eso);
    L.omesa = fsub(1.0f, esa);
    L.km = mk(km_of(m, m.base.x, ea, L.kd), km_of(m, m.base.y, ea, L.kd), km_of(m, m.base.z, ea, L.kd));
}
// evalBsdf / evalLegacy (f cos and pdf) and lambertCos of one (wo, wi) pair.
struct Eval { v3 fcos; float pdf; v3 lam; };
__device__ __noinline__ Eval eval_lobe(const PtParams& P, const Lobe& L, v3 wo, v3 wi, bool dropCosine) {
    const v3 z = mk(0.0f, 0.0f, 0.0f);
    Eval r{z, 0.0f, z};
    if (wo.z <= 0.0f || wi.z <= 0.0f) return r;
    const Bsdf& m = L.m;
    const float ps = L.ps, cosI = dropCosine ? 1.0f : wi.z;
    v3 f = L.fd;
    float pdf = fdiv(fmul(fsub(1.0f, ps), wi.z), kPiF);
    v3 lam = f;
    if (ps > 0.0f) {
        // the specular terms with the per-bounce parts
        const v3 h = normalize(add(wo, wi));
        const float oh = dot(wo, h);
        const float D = ggx_d(L.a2, h.z);
        const float G2 = frcp(fadd(fadd(1.0f, L.lo), lambda_f(L.a2, wi.z)));
        const float x1 = clampf(fsub(1.0f, oh), 0.0f, 1.0f);
        const float fw = fmul(fmul(fmul(fmul(x1, x1), x1), x1), x1);
        const float spec = fdiv(fmul(D, G2), fmul(L.four_wo, wi.z));
        const v3 F0 = L.F0;
        if (m.legacy) {
            const v3 F = mk(fadd(F0.x, fmul(fsub(1.0f, F0.x), fw)), fadd(F0.y, fmul(fsub(1.0f, F0.y), fw)),
                            fadd(F0.z, fmul(fsub(1.0f, F0.z), fw)));
            f = add(f, scale(F, spec));
        } else {
            // energyOf's terms at mu_i
            float ia, ib;
            table_ab(P.table, wi.z, m.rough, ia, ib);
            const float ei = smin(1.0f, fadd(ia, ib));
            const float ms = L.ms_on ? fdiv(fmul(L.omeo, fsub(1.0f, ei)), L.den_ms) : 0.0f;
            const float esi = fadd(fmul(L.on, fadd(fmul(L.d, ia), ib)), fmul(L.kd, fsub(1.0f, ei)));
            const float wd = fdiv(fmul(L.omeso, fsub(1.0f, esi)), L.omesa);
            f = scale(f, wd);
            lam = f;
            const float f90 = L.f90;
            const v3 F = mk(fadd(F0.x, fmul(fsub(f90, F0.x), fw)), fadd(F0.y, fmul(fsub(f90, F0.y), fw)),
                            fadd(F0.z, fmul(fsub(f90, F0.z), fw)));
            f = add(add(f, scale(F, spec)), scale(L.km, ms));
        }
        pdf = fadd(pdf, fmul(ps, fdiv(fmul(L.G1, D), L.four_wo)));
    }
    r.fcos = scale(f, cosI);
    r.pdf = pdf;
    r.lam = scale(lam, cosI);
    return r;
}
__device__ __forceinline__ v3 spec_albedo(const Bsdf& m, float cosO) {
    if (lobe_prob(m) <= 0.0f) return mk(0.0f, 0.0f, 0.0f);
    const float x1 = clampf(fsub(1.0f, cosO), 0.0f, 1.0f), fw = fmul(fmul(fmul(fmul(x1, x1), x1), x1), x1);
    const v3 F0 = f0_of(m);
    return mk(fadd(F0.x, fmul(fsub(1.0f, F0.x), fw)), fadd(F0.y, fmul(fsub(1.0f, F0.y), fw)),
              fadd(F0.z, fmul(fsub(1.0f, F0.z), fw)));
}
// one-sample mixture; u = (u1, kb / 2^24)
__device__ bool sample_bsdf(const PtParams& P, const Bsdf& m, v3 wo, float pick, float u1, uint32_t kb, v3& wi) {
    if (pick < lobe_prob(m)) {
        const float a = smax(1e-4f, fmul(m.rough, m.rough));
        const v3 h = sample_vndf(P, wo, a, u1, kb);
        wi = sub(scale(h, fmul(2.0f, dot(wo, h))), wo);
    } else {
        float c, s;
        sample_sincos(kb, P.corr, c, s);
        const float r = fsqrt(u1);
        wi = mk(fmul(r, c), fmul(r, s), fsqrt(smax(0.0f, fsub(1.0f, u1))));
    }
    return wi.z > 0.0f;
}

// ---------------------------------------------------------------- scene queries (rt_pt_ctx.hpp:18-79)
struct Surf { v3 p, n, ng, base; const float* m; float t; int tri; };
__device__ __forceinline__ v3 tri_corner(const PtParams& P, int t, int k) { return load3(P.tris + (size_t)t * 9 + 3 * k); }

// The surface at the closest hit (triangle tri at t along o + t d): the hit's barycentrics,
// position, normals, texture coordinates, texel and material (rt_pt_ctx.hpp:18-60).
__device__ __noinline__ void surface_of(const PtParams& P, v3 o, v3 d, int tri, float t, Surf& x) {
    const v3 a = tri_corner(P, tri, 0), b = tri_corner(P, tri, 1), c = tri_corner(P, tri, 2);
    float tt, u, v;
    hit_tri_uv(make_wray(o, d), a, b, c, tt, u, v);      // the winner's u, v (its t is the walk's)
    const uint32_t i0 = __ldg(P.idx + (size_t)tri * 3), i1 = __ldg(P.idx + (size_t)tri * 3 + 1),
                   i2 = __ldg(P.idx + (size_t)tri * 3 + 2);
    const float b0 = fsub(fsub(1.0f, u), v);
    x.t = t; x.tri = tri;
    x.p = add(o, scale(d, t));
    x.ng = normalize(cross(sub(b, a), sub(c, a)));
    const v3 n0 = load3(P.nrm + 3 * (size_t)i0), n1 = load3(P.nrm + 3 * (size_t)i1), n2 = load3(P.nrm + 3 * (size_t)i2);
    x.n = normalize(add(add(scale(n0, b0), scale(n1, u)), scale(n2, v)));
    const float tu = fadd(fadd(fmul(__ldg(P.uv + 2 * (size_t)i0), b0), fmul(__ldg(P.uv + 2 * (size_t)i1), u)),
                          fmul(__ldg(P.uv + 2 * (size_t)i2), v));
    const float tv = fadd(fadd(fmul(__ldg(P.uv + 2 * (size_t)i0 + 1), b0), fmul(__ldg(P.uv + 2 * (size_t)i1 + 1), u)),
                          fmul(__ldg(P.uv + 2 * (size_t)i2 + 1), v));
    const uint32_t tex = __ldg(P.tritex + tri);
    const uint32_t off = __ldg(P.texent + 3 * tex), tw = __ldg(P.texent + 3 * tex + 1), th = __ldg(P.texent + 3 * tex + 2);
    const uint32_t tx = (uint32_t)(int32_t)floorf(fmul(tu, (float)tw)) & (tw - 1);
    const uint32_t ty = (uint32_t)(int32_t)floorf(fmul(tv, (float)th)) & (th - 1);
    const uint32_t col = __ldg(P.texels + off + ty * tw + tx);
    x.m = P.mat + 7 * (size_t)tex;
    const float k = fdiv(__ldg(x.m), 255.0f);
    x.base = mk(fmul((float)(col & 255u), k), fmul((float)((col >> 8) & 255u), k), fmul((float)((col >> 16) & 255u), k));
    if (dot(x.ng, d) > 0.0f) x.ng = scale(x.ng, -1.0f);
    if (dot(x.n, x.ng) < 0.0f) x.n = scale(x.n, -1.0f);
    (void)tt;
}
__device__ __noinline__ bool hit(const PtParams& P, v3 o, v3 d, float tmax, Surf& x) {
    if (!P.has_geometry) return false;
    float t;
    const int tri = walk_closest(P.nodes, P.ltris, o, d, tmax, t, P.err);
    if (tri < 0) return false;
    surface_of(P, o, d, tri, t, x);
    return true;
}
__device__ __noinline__ bool visible(const PtParams& P, v3 p, v3 dir, float tmax) {
    if (!P.has_geometry) return true;
    Counts cn;
    return walk<false>(P.nodes, P.ltris, p, dir, tmax, tmax, P.err, cn) == 0;
}
__device__ __forceinline__ v3 offset_of(const Surf& x, v3 dir) {
    const float e = fmul(2e-4f, fadd(1.0f, smax(fabsf(x.p.x), smax(fabsf(x.p.y), fabsf(x.p.z)))));
    return add(x.p, scale(x.ng, dot(x.ng, dir) > 0.0f ? e : -e));
}
__device__ v3 nee(const PtParams& P, const Surf& x, const Frame& fr, const Lobe& lb, v3 woL, uint32_t px, uint32_t smp,
                  uint32_t base, v3& diff) {
    v3 L = mk(0.0f, 0.0f, 0.0f);
    diff = L;
    const bool dc = (P.controls & RN_PT_DROP_LAMBERT_COSINE) != 0;
    if (maxc(P.sun_irr) > 0.0f) {
        const v3 l = P.sun_dir, lL = to_local(fr, l);
        const Eval e = eval_lobe(P, lb, woL, lL, dc);
        if (maxc(e.fcos) > 0.0f && visible(P, offset_of(x, l), l, 1e30f)) {
            L = add(L, mulv(e.fcos, P.sun_irr));
            diff = add(diff, mulv(e.lam, P.sun_irr));
        }
    }
    if (P.nemit == 0) return L;
    const R2 a = rand2(P, px, smp, base + 2), b = rand2(P, px, smp, base + 3);
    const float target = fmul(a.a, P.area);
    uint32_t lo = 0, hi = P.nemit;              // std::upper_bound: the first cdf > target
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (target < __ldg(P.cdf + mid)) hi = mid; else lo = mid + 1;
    }
    const uint32_t k = lo < P.nemit - 1 ? lo : P.nemit - 1;
    const int et = (int)__ldg(P.emit + k);
    const v3 ta = tri_corner(P, et, 0), tb = tri_corner(P, et, 1), tc = tri_corner(P, et, 2);
    const float su = fsqrt(a.b);
    const v3 q = add(add(scale(ta, fsub(1.0f, su)), scale(tb, fmul(su, fsub(1.0f, b.a)))), scale(tc, fmul(su, b.a)));
    const v3 to = sub(q, x.p);
    const float dist = length(to);
    const v3 l = scale(to, frcp(dist)), lL = to_local(fr, l);
    const float cosL = fabsf(dot(normalize(cross(sub(tb, ta), sub(tc, ta))), l));
    if (cosL <= 0.0f) return L;
    const float pl = fdiv(fmul(dist, dist), fmul(cosL, P.area));
    const Eval e = eval_lobe(P, lb, woL, lL, dc);
    if (maxc(e.fcos) <= 0.0f || !visible(P, offset_of(x, l), l, fmul(dist, fsub(1.0f, 1e-3f)))) return L;
    const float w = (P.controls & RN_PT_MIS_WEIGHT_ONE) ? 1.0f
                                                      : fdiv(fmul(pl, pl), fadd(fmul(pl, pl), fmul(e.pdf, e.pdf)));
    const float* em = P.mat + 7 * (size_t)__ldg(P.tritex + et) + 4;
    const v3 Le = mk(__ldg(em), __ldg(em + 1), __ldg(em + 2));
    const float wp = fdiv(w, pl);
    diff = add(diff, scale(mulv(e.lam, Le), wp));
    return add(L, scale(mulv(e.fcos, Le), wp));
}

struct Sample { v3 L, D, S, E, alb, nrm, dAlb, sAlb; };
// One path's state between bounces (the locals of rt_pt_cpu.cpp:31-97's loop).
struct Path {
    Sample o;
    v3 ro, rd, T, tw, R, wd, ws;
    float prevPdf;
    uint32_t b, px, smp;
};
__device__ __forceinline__ void path_start(Path& s, v3 ro, v3 rd, uint32_t px, uint32_t smp) {
    const v3 z = mk(0.0f, 0.0f, 0.0f);
    s.o = Sample{z, z, z, z, z, z, z, z};
    s.ro = ro; s.rd = rd;
    s.T = mk(1.0f, 1.0f, 1.0f); s.tw = s.T; s.R = z; s.wd = z; s.ws = z;
    s.prevPdf = 0.0f;
    s.b = 0; s.px = px; s.smp = smp;
}
// One bounce (one iteration of rt_pt_cpu.cpp:37-91's loop); false when the path ends.
__device__ __noinline__ bool path_bounce(const PtParams& P, Path& s) {
    const uint32_t b = s.b;
    if (b > P.max_bounces) return false;
    const bool dc = (P.controls & RN_PT_DROP_LAMBERT_COSINE) != 0;
    Surf x0;
    if (!hit(P, s.ro, s.rd, 1e30f, x0)) {
        s.o.L = add(s.o.L, mulv(s.T, P.sky));
        if (b == 0) s.o.E = P.sky; else s.R = add(s.R, mulv(s.tw, P.sky));
        return false;
    }
    const Bsdf bs{x0.base, __ldg(x0.m + 1), __ldg(x0.m + 2), __ldg(x0.m + 3), (P.controls & RN_PT_LEGACY_LOBE_V2) != 0};
    if (b == 0) {
        s.o.alb = x0.base; s.o.nrm = x0.n;
        s.o.dAlb = scale(x0.base, fsub(1.0f, bs.metallic));
        s.o.sAlb = spec_albedo(bs, clampf(-dot(x0.n, s.rd), 0.0f, 1.0f));
    }
    const v3 Le = mk(__ldg(x0.m + 4), __ldg(x0.m + 5), __ldg(x0.m + 6));
    if (maxc(Le) > 0.0f) {
        float w = 1.0f;
        if (b > 0 && !(P.controls & RN_PT_MIS_WEIGHT_ONE)) {
            const float cosL = fabsf(dot(x0.ng, s.rd)), pl = fdiv(fmul(x0.t, x0.t), fmul(cosL, P.area));
            w = fdiv(fmul(s.prevPdf, s.prevPdf), fadd(fmul(s.prevPdf, s.prevPdf), fmul(pl, pl)));
        }
        s.o.L = add(s.o.L, scale(mulv(s.T, Le), w));
        if (b == 0) s.o.E = Le; else s.R = add(s.R, scale(mulv(s.tw, Le), w));
    }
    if (b == P.max_bounces) return false;
    const Frame fr = basis(x0.n);
    const v3 woL = to_local(fr, scale(s.rd, -1.0f));
    if (woL.z <= 0.0f) return false;
    const uint32_t base = 2 + b * 4;
    Lobe lb;
    lobe_setup(P, bs, woL.z, lb);
    v3 nd;
    const v3 Ln = nee(P, x0, fr, lb, woL, s.px, s.smp, base, nd);
    s.o.L = add(s.o.L, mulv(s.T, Ln));
    if (b == 0) { s.o.D = nd; s.o.S = sub(Ln, nd); } else s.R = add(s.R, mulv(s.tw, Ln));
    const R2 u = rand2(P, s.px, s.smp, base), r = rand2(P, s.px, s.smp, base + 1);
    v3 wiL;
    if (!sample_bsdf(P, bs, woL, r.a, u.a, u.kb, wiL)) return false;
    const Eval e = eval_lobe(P, lb, woL, wiL, dc);
    if (e.pdf <= 0.0f) return false;
    const float ip = frcp(e.pdf);
    const v3 step = scale(e.fcos, ip);
    s.T = mulv(s.T, step);
    if (b == 0) { s.wd = scale(e.lam, ip); s.ws = sub(step, s.wd); }
    else s.tw = mulv(s.tw, step);
    s.prevPdf = e.pdf;
    if (P.rr && b >= 3) {
        const float q = smin(0.95f, maxc(s.T));
        if (r.b >= q) return false;
        const float iq = frcp(q);
        s.T = scale(s.T, iq);
        s.tw = scale(s.tw, iq);
    }
    const v3 wi = to_world(fr, wiL);
    s.ro = offset_of(x0, wi);
    s.rd = wi;
    s.b = b + 1;
    return true;
}
// rt_pt_cpu.cpp:92-96: the split's last terms.
__device__ __forceinline__ void path_finish(const PtParams& P, Path& s) {
    s.o.D = add(s.o.D, mulv(s.wd, s.R));
    if (!(P.controls & RN_PT_AOV_DROP_SPECULAR_INDIRECT)) s.o.S = add(s.o.S, mulv(s.ws, s.R));
    if (P.controls & RN_PT_AOV_EMISSION_TO_DIFFUSE) { s.o.D = add(s.o.D, s.o.E); s.o.E = mk(0.0f, 0.0f, 0.0f); }
}
__device__ __forceinline__ void store_sample(const PtParams& P, uint32_t j, uint32_t px, const Sample& o) {
    const size_t stride = (size_t)P.kn * P.npix;
    float* s = P.samp + (size_t)j * P.npix + px;
    const v3* f = &o.L;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        s[(3 * c) * stride] = f[c].x;
        s[(3 * c + 1) * stride] = f[c].y;
        s[(3 * c + 2) * stride] = f[c].z;
    }
}

// rt_pt_cpu.cpp:21-24
__device__ __forceinline__ v3 dir_of(const PtCam& c, float px, float py, int w, int h) {
    const float nx = fsub(fmul(fdiv(px, (float)w), 2.0f), 1.0f), ny = fsub(1.0f, fmul(fdiv(py, (float)h), 2.0f));
    return normalize(add(add(c.f, scale(c.s, fmul(fmul(nx, c.th), c.aspect))), scale(c.u, fmul(ny, c.th))));
}

__device__ __forceinline__ v3 camera_ray(const PtParams& P, int x, int y, uint32_t px, uint32_t smp) {
    float ja = 0.5f, jb = 0.5f;
    if (P.jitter) { const R2 r = rand2(P, px, smp, 0); ja = r.a; jb = r.b; }
    return dir_of(P.cam, fadd((float)x, ja), fadd((float)y, jb), P.w, P.h);
}

// One thread per (pixel, sample of the slice): a warp takes an 8 x 4 pixel tile for one sample.
__global__ void __launch_bounds__(128) pt_paths_kernel(const PtParams P) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    const uint32_t tiles_x = (P.w + kTileW - 1) / kTileW, tiles_y = (P.h + kTileH - 1) / kTileH;
    const uint32_t ntiles = tiles_x * tiles_y;
    if (warp >= ntiles * P.kn) return;
    const uint32_t j = warp / ntiles, tile = warp % ntiles;
    const int x = (int)((tile % tiles_x) * kTileW + (lane % kTileW)), y = (int)((tile / tiles_x) * kTileH + (lane / kTileW));
    if (x >= P.w || y >= P.h) return;
    const uint32_t px = (uint32_t)(y * P.w + x);
    const uint32_t smp = P.spp_begin + P.k0 + j;
    Path s;
    path_start(s, P.cam.eye, camera_ray(P, x, y, px, smp), px, smp);
    while (path_bounce(P, s)) {}
    path_finish(P, s);
    store_sample(P, j, px, s.o);
}

// Path regeneration: persistent threads, each taking the next (pixel, sample) of the slice
// from a counter whenever its path ends, so a warp's lanes are not held by its longest path
// (Russian roulette gives paths of very different lengths). Items run tile-major (a warp's
// first items are one 8 x 4 tile for one sample index); the per-sample terms and their sum
// in sample order are the per-sample kernel's, so the bits are the same.
__global__ void __launch_bounds__(128) pt_regen_kernel(const PtParams P, uint32_t* ctr) {
    const uint32_t tiles_x = (P.w + kTileW - 1) / kTileW, tiles_y = (P.h + kTileH - 1) / kTileH;
    const uint32_t ntiles = tiles_x * tiles_y;
    const unsigned long long total = (unsigned long long)ntiles * 32ull * P.kn;
    Path s;
    uint32_t j = 0;
    bool live = false;
    for (;;) {
        if (!live) {
            const unsigned long long item = atomicAdd(reinterpret_cast<unsigned long long*>(ctr), 1ull);
            if (item >= total) break;
            const uint32_t lane = (uint32_t)(item & 31u);
            const unsigned long long w = item >> 5;
            j = (uint32_t)(w / ntiles);
            const uint32_t tile = (uint32_t)(w % ntiles);
            const int x = (int)((tile % tiles_x) * kTileW + (lane % kTileW)),
                      y = (int)((tile / tiles_x) * kTileH + (lane / kTileW));
            if (x >= P.w || y >= P.h) continue;
            const uint32_t px = (uint32_t)(y * P.w + x);
            const uint32_t smp = P.spp_begin + P.k0 + j;
            path_start(s, P.cam.eye, camera_ray(P, x, y, px, smp), px, smp);
            live = true;
        }
        if (!path_bounce(P, s)) {
            path_finish(P, s);
            store_sample(P, j, s.px, s.o);
            live = false;
        }
    }
}

// ================================================================ the wavefront form
// The same paths with each bounce split over three kernels that run over a pool of path
// slots in HBM: pt_wave_shade (the rest of a bounce after its closest hit: emission, the
// lobe, next-event estimation up to its shadow rays, the sampled direction, Russian
// roulette; a slot whose path ended takes the next (pixel, sample) item), pt_wave_shadow
// (the queued shadow rays' any-hit walks) and pt_wave_extend (the closest-hit walks). A warp
// then runs one kind of code at a time: the bounce as one kernel left warps at different
// points of a large body (instruction-fetch stalls dominated) and its walks diverging
// beside shading.
//
// Order of every float operation is path_bounce's: a bounce's estimate (the sun's and the
// emitter's terms, kept with the throughput it is weighted by) is added once its shadow
// rays are traced, at the start of the slot's next shade pass, before anything else touches
// the path's sums (the next bounce's emission, or the path's end).
namespace wave {
// float components (each an array of Q floats)
enum : int {
    RO = 0, RD = 3, T = 6, TW = 9, R = 12, WD = 15, WS = 18, PREV = 21,
    OL = 22, OD = 25, OS = 28, OE = 31, OALB = 34, ONRM = 37, ODALB = 40, OSALB = 43,   // Sample, in store_sample order
    TP = 46, TWP = 49, LSUN = 52, DSUN = 55, LEM = 58, DEM = 61, HT = 64, NF = 65
};
// u32 components
enum : int { UB = 0, UPX = 1, USMP = 2, UJ = 3, UTRI = 4, UFL = 5, NU = 6 };
// a slot's mode (bits 0-1) and its pending estimate
enum : uint32_t {
    M_FRESH = 0,      // takes the next item
    M_TRACE = 1,      // its ray was traced (or is about to be): the next shade pass continues the bounce
    M_END = 2,        // its path ended after an estimate: finish once the estimate is added
    M_IDLE = 3,       // no items left
    F_NEE = 4,        // the last bounce ran next-event estimation (add it before anything else)
    F_SUN = 8,        // ... with a sun shadow ray
    F_EM = 16,        // ... with an emitter shadow ray
    F_B0 = 32         // ... at bounce 0 (the estimate sets D and S instead of adding to R)
};
}  // namespace wave

struct WaveBufs {
    float* f;             // NF x Q
    uint32_t* u;          // NU x Q
    uint8_t* vis;         // 2 x Q: the sun ray and the emitter ray reached their light
    float* qf;            // 7 x 2Q: the shadow rays' origin, direction, limit
    uint32_t* qu;         // 2Q: slot << 1 | (emitter ray)
    uint32_t* ctr;        // [0] shadow rays queued [1] live slots [2..3] the 64-bit item counter
    uint32_t Q;
};
__device__ __forceinline__ v3 wld3(const WaveBufs& W, int c, uint32_t i) {
    const size_t q = W.Q;
    return mk(W.f[c * q + i], W.f[(c + 1) * q + i], W.f[(c + 2) * q + i]);
}
__device__ __forceinline__ void wst3(const WaveBufs& W, int c, uint32_t i, v3 v) {
    const size_t q = W.Q;
    W.f[c * q + i] = v.x; W.f[(c + 1) * q + i] = v.y; W.f[(c + 2) * q + i] = v.z;
}
__device__ __forceinline__ uint32_t& wu(const WaveBufs& W, int c, uint32_t i) { return W.u[(size_t)c * W.Q + i]; }
__device__ __forceinline__ float& wf(const WaveBufs& W, int c, uint32_t i) { return W.f[(size_t)c * W.Q + i]; }

// `n` consecutive slots of a counter for each lane of a full warp, one atomic a warp.
__device__ __forceinline__ uint32_t wave_reserve(uint32_t* ctr, uint32_t n) {
    const int lane = threadIdx.x & 31;
    uint32_t incl = n;
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    uint32_t base = 0;
    if (lane == 31 && total) base = atomicAdd(ctr, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    return base + incl - n;
}

// path_finish and store_sample from the slot's arrays.
__device__ void wave_finish(const PtParams& P, const WaveBufs& W, uint32_t i) {
    using namespace wave;
    Sample o;
    o.L = wld3(W, OL, i); o.D = wld3(W, OD, i); o.S = wld3(W, OS, i); o.E = wld3(W, OE, i);
    o.alb = wld3(W, OALB, i); o.nrm = wld3(W, ONRM, i); o.dAlb = wld3(W, ODALB, i); o.sAlb = wld3(W, OSALB, i);
    const v3 R = wld3(W, wave::R, i);
    o.D = add(o.D, mulv(wld3(W, WD, i), R));
    if (!(P.controls & RN_PT_AOV_DROP_SPECULAR_INDIRECT)) o.S = add(o.S, mulv(wld3(W, WS, i), R));
    if (P.controls & RN_PT_AOV_EMISSION_TO_DIFFUSE) { o.D = add(o.D, o.E); o.E = mk(0.0f, 0.0f, 0.0f); }
    store_sample(P, wu(W, UJ, i), wu(W, UPX, i), o);
}

// path_start into the slot's arrays.
__device__ void wave_start(const PtParams& P, const WaveBufs& W, uint32_t i, uint32_t j, uint32_t px, uint32_t smp,
                           v3 rd) {
    using namespace wave;
    const v3 z = mk(0.0f, 0.0f, 0.0f), one = mk(1.0f, 1.0f, 1.0f);
    wst3(W, RO, i, P.cam.eye); wst3(W, RD, i, rd);
    wst3(W, T, i, one); wst3(W, TW, i, one);
    wst3(W, wave::R, i, z); wst3(W, WD, i, z); wst3(W, WS, i, z);
    wf(W, PREV, i) = 0.0f;
    for (int c = OL; c < OL + 24; c += 3) wst3(W, c, i, z);
    wu(W, UB, i) = 0; wu(W, UPX, i) = px; wu(W, USMP, i) = smp; wu(W, UJ, i) = j;
}

// One bounce after its closest hit, for a slot in M_TRACE (path_bounce from the hit on):
// returns the slot's next mode; next-event estimation leaves its flags in *fl and its
// shadow rays in the ray arguments.
__device__ __noinline__ uint32_t wave_bounce(const PtParams& P, const WaveBufs& W, uint32_t i, uint32_t& fl,
                                             v3& sun_o, v3& em_o, v3& em_d, float& em_t) {
    using namespace wave;
    const uint32_t b = wu(W, UB, i);
    if (b > P.max_bounces) return M_FRESH;
    const bool dc = (P.controls & RN_PT_DROP_LAMBERT_COSINE) != 0;
    const int tri = (int)wu(W, UTRI, i);
    const v3 ro = wld3(W, RO, i), rd = wld3(W, RD, i);
    v3 T = wld3(W, wave::T, i), tw = wld3(W, TW, i);
    if (tri < 0) {
        wst3(W, OL, i, add(wld3(W, OL, i), mulv(T, P.sky)));
        if (b == 0) wst3(W, OE, i, P.sky); else wst3(W, wave::R, i, add(wld3(W, wave::R, i), mulv(tw, P.sky)));
        return M_FRESH;
    }
    Surf x0;
    surface_of(P, ro, rd, tri, wf(W, HT, i), x0);
    const Bsdf bs{x0.base, __ldg(x0.m + 1), __ldg(x0.m + 2), __ldg(x0.m + 3), (P.controls & RN_PT_LEGACY_LOBE_V2) != 0};
    if (b == 0) {
        wst3(W, OALB, i, x0.base); wst3(W, ONRM, i, x0.n);
        wst3(W, ODALB, i, scale(x0.base, fsub(1.0f, bs.metallic)));
        wst3(W, OSALB, i, spec_albedo(bs, clampf(-dot(x0.n, rd), 0.0f, 1.0f)));
    }
    const v3 Le = mk(__ldg(x0.m + 4), __ldg(x0.m + 5), __ldg(x0.m + 6));
    if (maxc(Le) > 0.0f) {
        float w = 1.0f;
        if (b > 0 && !(P.controls & RN_PT_MIS_WEIGHT_ONE)) {
            const float pp = wf(W, PREV, i);
            const float cosL = fabsf(dot(x0.ng, rd)), pl = fdiv(fmul(x0.t, x0.t), fmul(cosL, P.area));
            w = fdiv(fmul(pp, pp), fadd(fmul(pp, pp), fmul(pl, pl)));
        }
        wst3(W, OL, i, add(wld3(W, OL, i), scale(mulv(T, Le), w)));
        if (b == 0) wst3(W, OE, i, Le); else wst3(W, wave::R, i, add(wld3(W, wave::R, i), scale(mulv(tw, Le), w)));
    }
    if (b == P.max_bounces) return M_FRESH;
    const Frame fr = basis(x0.n);
    const v3 woL = to_local(fr, scale(rd, -1.0f));
    if (woL.z <= 0.0f) return M_FRESH;
    const uint32_t base = 2 + b * 4;
    Lobe lb;
    lobe_setup(P, bs, woL.z, lb);
    // next-event estimation (nee) up to its shadow rays: the terms each adds when its ray
    // reaches the light
    fl = F_NEE | (b == 0 ? F_B0 : 0u);
    if (maxc(P.sun_irr) > 0.0f) {
        const v3 l = P.sun_dir, lL = to_local(fr, l);
        const Eval e = eval_lobe(P, lb, woL, lL, dc);
        if (maxc(e.fcos) > 0.0f) {
            wst3(W, LSUN, i, mulv(e.fcos, P.sun_irr));
            wst3(W, DSUN, i, mulv(e.lam, P.sun_irr));
            sun_o = offset_of(x0, l);
            fl |= F_SUN;
        }
    }
    if (P.nemit != 0) {
        const R2 a = rand2(P, wu(W, UPX, i), wu(W, USMP, i), base + 2), bb = rand2(P, wu(W, UPX, i), wu(W, USMP, i), base + 3);
        const float target = fmul(a.a, P.area);
        uint32_t lo = 0, hi = P.nemit;              // std::upper_bound: the first cdf > target
        while (lo < hi) {
            const uint32_t mid = lo + (hi - lo) / 2;
            if (target < __ldg(P.cdf + mid)) hi = mid; else lo = mid + 1;
        }
        const uint32_t k = lo < P.nemit - 1 ? lo : P.nemit - 1;
        const int et = (int)__ldg(P.emit + k);
        const v3 ta = tri_corner(P, et, 0), tb = tri_corner(P, et, 1), tc = tri_corner(P, et, 2);
        const float su = fsqrt(a.b);
        const v3 q = add(add(scale(ta, fsub(1.0f, su)), scale(tb, fmul(su, fsub(1.0f, bb.a)))), scale(tc, fmul(su, bb.a)));
        const v3 to = sub(q, x0.p);
        const float dist = length(to);
        const v3 l = scale(to, frcp(dist)), lL = to_local(fr, l);
        const float cosL = fabsf(dot(normalize(cross(sub(tb, ta), sub(tc, ta))), l));
        if (cosL > 0.0f) {
            const float pl = fdiv(fmul(dist, dist), fmul(cosL, P.area));
            const Eval e = eval_lobe(P, lb, woL, lL, dc);
            if (maxc(e.fcos) > 0.0f) {
                const float w = (P.controls & RN_PT_MIS_WEIGHT_ONE)
                                    ? 1.0f
                                    : fdiv(fmul(pl, pl), fadd(fmul(pl, pl), fmul(e.pdf, e.pdf)));
                const float* em = P.mat + 7 * (size_t)__ldg(P.tritex + et) + 4;
                const v3 Lem = mk(__ldg(em), __ldg(em + 1), __ldg(em + 2));
                const float wp = fdiv(w, pl);
                wst3(W, DEM, i, scale(mulv(e.lam, Lem), wp));
                wst3(W, LEM, i, scale(mulv(e.fcos, Lem), wp));
                em_o = offset_of(x0, l);
                em_d = l;
                em_t = fmul(dist, fsub(1.0f, 1e-3f));
                fl |= F_EM;
            }
        }
    }
    wst3(W, TP, i, T);
    wst3(W, TWP, i, tw);
    // the sampled direction
    const R2 u = rand2(P, wu(W, UPX, i), wu(W, USMP, i), base), r = rand2(P, wu(W, UPX, i), wu(W, USMP, i), base + 1);
    v3 wiL;
    if (!sample_bsdf(P, bs, woL, r.a, u.a, u.kb, wiL)) return M_END;
    const Eval e = eval_lobe(P, lb, woL, wiL, dc);
    if (e.pdf <= 0.0f) return M_END;
    const float ip = frcp(e.pdf);
    const v3 step = scale(e.fcos, ip);
    T = mulv(T, step);
    if (b == 0) {
        const v3 wd = scale(e.lam, ip);
        wst3(W, WD, i, wd);
        wst3(W, WS, i, sub(step, wd));
    } else {
        tw = mulv(tw, step);
    }
    if (P.rr && b >= 3) {
        const float q = smin(0.95f, maxc(T));
        if (r.b >= q) return M_END;
        const float iq = frcp(q);
        T = scale(T, iq);
        tw = scale(tw, iq);
    }
    const v3 wi = to_world(fr, wiL);
    wst3(W, wave::T, i, T);
    wst3(W, TW, i, tw);
    wf(W, PREV, i) = e.pdf;
    wst3(W, RO, i, offset_of(x0, wi));
    wst3(W, RD, i, wi);
    wu(W, UB, i) = b + 1;
    return M_TRACE;
}

template <int kMinBlocks>
__global__ void __launch_bounds__(128, kMinBlocks) pt_wave_shade(const PtParams P, const WaveBufs W,
                                                                 unsigned long long total) {
    using namespace wave;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31u;
    const bool in = i < W.Q;
    uint32_t fl = in ? wu(W, UFL, i) : (uint32_t)M_IDLE;
    uint32_t mode = fl & 3u;
    // 1. the last bounce's estimate, its shadow rays now traced (nee's sums, then the
    //    bounce's use of them: L += T Ln, then D and S at bounce 0 or R += tw Ln)
    if (fl & F_NEE) {
        v3 L = mk(0.0f, 0.0f, 0.0f), diff = L;
        if ((fl & F_SUN) && W.vis[i]) { L = add(L, wld3(W, LSUN, i)); diff = add(diff, wld3(W, DSUN, i)); }
        if ((fl & F_EM) && W.vis[W.Q + i]) { diff = add(diff, wld3(W, DEM, i)); L = add(L, wld3(W, LEM, i)); }
        wst3(W, OL, i, add(wld3(W, OL, i), mulv(wld3(W, TP, i), L)));
        if (fl & F_B0) { wst3(W, OD, i, diff); wst3(W, OS, i, sub(L, diff)); }
        else wst3(W, wave::R, i, add(wld3(W, wave::R, i), mulv(wld3(W, TWP, i), L)));
    }
    // 2. the bounce after the closest hit, or the end of a path that ended after its estimate
    uint32_t nfl = 0;
    v3 sun_o = mk(0.0f, 0.0f, 0.0f), em_o = sun_o, em_d = sun_o;
    float em_t = 0.0f;
    if (mode == M_TRACE) {
        mode = wave_bounce(P, W, i, nfl, sun_o, em_o, em_d, em_t);
        // a path that ended before any estimate (a miss, the bounce limit, a surface seen
        // from behind) is finished now; one that ended after it (M_END) in the next pass
        if (mode == M_FRESH) wave_finish(P, W, i);
    } else if (mode == M_END) {
        wave_finish(P, W, i);
        mode = M_FRESH;
    }
    // 3. free slots take the next items (one atomic a warp per round)
    const uint32_t tiles_x = (P.w + kTileW - 1) / kTileW, tiles_y = (P.h + kTileH - 1) / kTileH;
    const uint32_t ntiles = tiles_x * tiles_y;
    for (int round = 0; round < 64; ++round) {
        const unsigned need = __ballot_sync(0xffffffffu, in && mode == M_FRESH);
        if (!need) break;
        const int leader = __ffs(need) - 1;
        unsigned long long first = 0;
        if ((int)lane == leader)
            first = atomicAdd(reinterpret_cast<unsigned long long*>(W.ctr + 2), (unsigned long long)__popc(need));
        first = __shfl_sync(0xffffffffu, first, leader);
        if (in && mode == M_FRESH) {
            const unsigned long long item = first + __popc(need & ((1u << lane) - 1u));
            if (item >= total) {
                mode = M_IDLE;
            } else {
                const uint32_t l = (uint32_t)(item & 31u);
                const unsigned long long w = item >> 5;
                const uint32_t j = (uint32_t)(w / ntiles), tile = (uint32_t)(w % ntiles);
                const int x = (int)((tile % tiles_x) * kTileW + (l % kTileW)), y = (int)((tile / tiles_x) * kTileH + (l / kTileW));
                if (x < P.w && y < P.h) {
                    const uint32_t px = (uint32_t)(y * P.w + x), smp = P.spp_begin + P.k0 + j;
                    wave_start(P, W, i, j, px, smp, camera_ray(P, x, y, px, smp));
                    mode = M_TRACE;
                }
            }
        }
    }
    // 4. the estimate's shadow rays into the queue; the slot's state; the live count
    const uint32_t nr = ((nfl & F_SUN) ? 1u : 0u) + ((nfl & F_EM) ? 1u : 0u);
    uint32_t pos = wave_reserve(W.ctr, nr);
    const size_t q2 = 2 * (size_t)W.Q;
    if (nfl & F_SUN) {
        W.qf[pos] = sun_o.x; W.qf[q2 + pos] = sun_o.y; W.qf[2 * q2 + pos] = sun_o.z;
        W.qf[3 * q2 + pos] = P.sun_dir.x; W.qf[4 * q2 + pos] = P.sun_dir.y; W.qf[5 * q2 + pos] = P.sun_dir.z;
        W.qf[6 * q2 + pos] = 1e30f;
        W.qu[pos] = i << 1;
        ++pos;
    }
    if (nfl & F_EM) {
        W.qf[pos] = em_o.x; W.qf[q2 + pos] = em_o.y; W.qf[2 * q2 + pos] = em_o.z;
        W.qf[3 * q2 + pos] = em_d.x; W.qf[4 * q2 + pos] = em_d.y; W.qf[5 * q2 + pos] = em_d.z;
        W.qf[6 * q2 + pos] = em_t;
        W.qu[pos] = (i << 1) | 1u;
    }
    if (in) wu(W, UFL, i) = mode | nfl;
    const unsigned live = __ballot_sync(0xffffffffu, in && mode != M_IDLE);
    if (lane == 0 && live) atomicAdd(W.ctr + 1, (uint32_t)__popc(live));
}

// The queued shadow rays (visible(): the any-hit walk of the AO kernel).
__global__ void __launch_bounds__(128) pt_wave_shadow(const PtParams P, const WaveBufs W) {
    const uint32_t n = W.ctr[0];
    const size_t q2 = 2 * (size_t)W.Q;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n && k < q2; k += gridDim.x * blockDim.x) {
        const v3 o = mk(W.qf[k], W.qf[q2 + k], W.qf[2 * q2 + k]);
        const v3 d = mk(W.qf[3 * q2 + k], W.qf[4 * q2 + k], W.qf[5 * q2 + k]);
        const float tmax = W.qf[6 * q2 + k];
        const uint32_t s = W.qu[k];
        bool vis = true;
        if (P.has_geometry) {
            Counts cn;
            vis = walk<false>(P.nodes, P.ltris, o, d, tmax, tmax, P.err, cn) == 0;
        }
        W.vis[(size_t)(s & 1u) * W.Q + (s >> 1)] = vis ? 1 : 0;
    }
}

// The closest hits of the slots' rays (rt::closest); also restarts the queue and live counts
// for the next shade pass.
__global__ void __launch_bounds__(128) pt_wave_extend(const PtParams P, const WaveBufs W) {
    using namespace wave;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) { W.ctr[0] = 0; W.ctr[1] = 0; }
    if (i >= W.Q || (wu(W, UFL, i) & 3u) != M_TRACE) return;
    float t = 0.0f;
    int tri = -1;
    if (P.has_geometry) tri = walk_closest(P.nodes, P.ltris, wld3(W, RO, i), wld3(W, RD, i), 1e30f, t, P.err);
    wu(W, UTRI, i) = (uint32_t)tri;
    wf(W, HT, i) = t;
}

// Per pixel: the slice's samples added in sample order to the running sums (rt_pt_cpu.cpp:
// 132-141); after the last slice the means, the variances and the pixel-centre ray.
struct PtOutDev {
    float *radiance, *albedo, *normal, *depth, *variance;
    int32_t* triangle;
    float* motion;
    float *diffuse, *specular, *emission, *diffuse_albedo, *specular_albedo, *diffuse_variance, *specular_variance;
};
__device__ __forceinline__ void put3(float* v, size_t p, v3 a) {
    if (v) { v[p * 3] = a.x; v[p * 3 + 1] = a.y; v[p * 3 + 2] = a.z; }
}
__device__ __forceinline__ float var_of(double s1, double s2, uint32_t n) {
    return n > 1 ? (float)(__ddiv_rn(__ddiv_rn(__dsub_rn(s2, __ddiv_rn(__dmul_rn(s1, s1), (double)n)), (double)(n - 1)),
                                     (double)n))
                 : 0.0f;
}
__global__ void __launch_bounds__(128) pt_accum_kernel(const PtParams P, const PtOutDev O) {
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x;
    if (px >= P.npix) return;
    float a[kSampleFloats];
    double m[6];
    if (P.first) {
#pragma unroll
        for (int c = 0; c < kSampleFloats; ++c) a[c] = 0.0f;
#pragma unroll
        for (int c = 0; c < 6; ++c) m[c] = 0.0;
    } else {
#pragma unroll
        for (int c = 0; c < kSampleFloats; ++c) a[c] = P.acc[(size_t)c * P.npix + px];
#pragma unroll
        for (int c = 0; c < 6; ++c) m[c] = P.mom[(size_t)c * P.npix + px];
    }
    const size_t stride = (size_t)P.kn * P.npix;
    for (uint32_t j = 0; j < P.kn; ++j) {
        const float* s = P.samp + (size_t)j * P.npix + px;
        float v[kSampleFloats];
#pragma unroll
        for (int c = 0; c < kSampleFloats; ++c) { v[c] = s[c * stride]; a[c] = fadd(a[c], v[c]); }
        // luminance of L, D and S, their moments in float64
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const double l = (double)lum(mk(v[3 * q], v[3 * q + 1], v[3 * q + 2]));
            m[2 * q] = __dadd_rn(m[2 * q], l);
            m[2 * q + 1] = __dadd_rn(m[2 * q + 1], __dmul_rn(l, l));
        }
    }
    if (!P.last) {
#pragma unroll
        for (int c = 0; c < kSampleFloats; ++c) P.acc[(size_t)c * P.npix + px] = a[c];
#pragma unroll
        for (int c = 0; c < 6; ++c) P.mom[(size_t)c * P.npix + px] = m[c];
        return;
    }
    const float inv = P.spp ? frcp((float)P.spp) : 0.0f;
    const size_t p = px;
    const v3 L = mk(a[0], a[1], a[2]), D = mk(a[3], a[4], a[5]), S = mk(a[6], a[7], a[8]), E = mk(a[9], a[10], a[11]);
    const v3 alb = mk(a[12], a[13], a[14]), nrm = mk(a[15], a[16], a[17]), da = mk(a[18], a[19], a[20]),
             sa = mk(a[21], a[22], a[23]);
    put3(O.radiance, p, scale(L, inv)); put3(O.albedo, p, scale(alb, inv)); put3(O.normal, p, scale(nrm, inv));
    put3(O.diffuse, p, scale(D, inv)); put3(O.specular, p, scale(S, inv)); put3(O.emission, p, scale(E, inv));
    put3(O.diffuse_albedo, p, scale(da, inv)); put3(O.specular_albedo, p, scale(sa, inv));
    if (O.variance) O.variance[p] = var_of(m[0], m[1], P.spp);
    if (O.diffuse_variance) O.diffuse_variance[p] = var_of(m[2], m[3], P.spp);
    if (O.specular_variance) O.specular_variance[p] = var_of(m[4], m[5], P.spp);
    // the pixel-centre ray (rt_pt_cpu.cpp:111-122)
    const int x = (int)(px % (uint32_t)P.w), y = (int)(px / (uint32_t)P.w);
    float depth = 0.0f, mx = 0.0f, my = 0.0f;
    int32_t tri = -1;
    if (O.depth || O.triangle || O.motion) {
        Surf c;
        if (hit(P, P.cam.eye, dir_of(P.cam, fadd((float)x, 0.5f), fadd((float)y, 0.5f), P.w, P.h), 1e30f, c)) {
            depth = dot(sub(c.p, P.cam.eye), P.cam.f);
            tri = c.tri;
            const v3 v = sub(c.p, P.prev.eye);
            const float zz = dot(v, P.prev.f);
            const float nx = fdiv(dot(v, P.prev.s), fmul(fmul(zz, P.prev.th), P.prev.aspect));
            const float ny = fdiv(dot(v, P.prev.u), fmul(zz, P.prev.th));
            mx = fsub(fmul(fadd(fmul(nx, 0.5f), 0.5f), (float)P.w), fadd((float)x, 0.5f));
            my = fsub(fmul(fsub(1.0f, fadd(fmul(ny, 0.5f), 0.5f)), (float)P.h), fadd((float)y, 0.5f));
        }
    }
    if (O.depth) O.depth[p] = depth;
    if (O.triangle) O.triangle[p] = tri;
    if (O.motion) { O.motion[p * 2] = mx; O.motion[p * 2 + 1] = my; }
}

// trianglesOf(geo) on the device: 9 floats a triangle from the indexed vertices.
__global__ void gather_tris_kernel(const float* __restrict__ pos, const uint32_t* __restrict__ idx, uint32_t ntri,
                                   float* __restrict__ tris) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    for (int k = 0; k < 3; ++k) {
        const uint32_t v = idx[3 * (size_t)t + k];
        tris[9 * (size_t)t + 3 * k] = pos[3 * (size_t)v];
        tris[9 * (size_t)t + 3 * k + 1] = pos[3 * (size_t)v + 1];
        tris[9 * (size_t)t + 3 * k + 2] = pos[3 * (size_t)v + 2];
    }
}

}  // namespace
}  // namespace rn

using namespace rn;

extern "C" {

int rn_pt_scene_create(const rn_pt_scene_desc* sd, rn_ptscene** out, rn_status* st) {
    if (!out) return fail(st, RN_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (!sd) return fail(st, RN_ERR_INVALID, "null scene");
    if (sd->ntri > 0 && (!sd->pos || !sd->nrm || !sd->uv || !sd->idx || !sd->tri_texture))
        return fail(st, RN_ERR_INVALID, "null geometry arrays");
    if (sd->ntri >= (1u << 28)) return fail(st, RN_ERR_INVALID, "%u triangles: at most 2^28 - 1", sd->ntri);
    if (sd->ntex == 0 || !sd->tex_entries || !sd->texels || !sd->materials)
        return fail(st, RN_ERR_INVALID, "a scene needs at least one texture and its material");
    // every index in range, every texture a power of two inside the texel array
    for (uint32_t i = 0; i < 3 * sd->ntri; ++i)
        if (sd->idx[i] >= sd->nvert) return fail(st, RN_ERR_INVALID, "index %u of triangle %u out of range", sd->idx[i], i / 3);
    for (uint32_t t = 0; t < sd->ntri; ++t)
        if (sd->tri_texture[t] >= sd->ntex) return fail(st, RN_ERR_INVALID, "triangle %u: texture %u", t, sd->tri_texture[t]);
    for (uint32_t k = 0; k < sd->ntex; ++k) {
        const uint64_t off = sd->tex_entries[3 * k], w = sd->tex_entries[3 * k + 1], h = sd->tex_entries[3 * k + 2];
        if (w == 0 || h == 0 || (w & (w - 1)) || (h & (h - 1)) || off + w * h > sd->ntexels)
            return fail(st, RN_ERR_INVALID, "texture %u: %llux%llu at %llu (sizes must be powers of two inside the texels)",
                        k, (unsigned long long)w, (unsigned long long)h, (unsigned long long)off);
    }
    RN_TRY(ensure_ctx(st));
    Context& c = ctx();
    const float* table = nullptr;
    RN_TRY(device_table(c.device, &table, st));
    rn_ptscene* s = new rn_ptscene();
    s->device = c.device;
    s->nvert = sd->nvert; s->ntri = sd->ntri; s->ntex = sd->ntex; s->ntexels = sd->ntexels;
    std::memcpy(s->sun_dir, sd->sun_dir, sizeof s->sun_dir);
    std::memcpy(s->sun_irr, sd->sun_irradiance, sizeof s->sun_irr);
    std::memcpy(s->sky, sd->sky, sizeof s->sky);
    // trianglesOf and finishPtScene's emitter list and inclusive area CDF, on the host in
    // triangle order (a float running sum: its rounding is the reference's)
    std::vector<float> tris((size_t)sd->ntri * 9);
    for (uint32_t t = 0; t < sd->ntri; ++t)
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) tris[9 * (size_t)t + 3 * k + a] = sd->pos[3 * (size_t)sd->idx[3 * (size_t)t + k] + a];
    std::vector<uint32_t> emit;
    std::vector<float> cdf;
    float area = 0.0f;
    for (uint32_t t = 0; t < sd->ntri; ++t) {
        const float* e = sd->materials[sd->tri_texture[t]].emission;
        if (e[0] <= 0.0f && e[1] <= 0.0f && e[2] <= 0.0f) continue;
        const float* q = &tris[9 * (size_t)t];
        const hv3 a{q[0], q[1], q[2]}, b{q[3], q[4], q[5]}, cc{q[6], q[7], q[8]};
        const hv3 cr = hcross(hsub(b, a), hsub(cc, a));
        area += 0.5f * std::sqrt(hdot(cr, cr));
        emit.push_back(t);
        cdf.push_back(area);
    }
    s->nemit = (uint32_t)emit.size();
    s->area = area;
    // one device block for every array
    const size_t nv = sd->nvert, nt = sd->ntri;
    const size_t sizes[] = {nv * 12, nv * 8, nt * 12, nt * 4, (size_t)sd->ntex * 12, (size_t)sd->ntexels * 4,
                            (size_t)sd->ntex * 28, nt * 36, emit.size() * 4, cdf.size() * 4, nv * 12};
    size_t offs[11], total = 0;
    for (int i = 0; i < 11; ++i) { offs[i] = total; total += (sizes[i] + 255) & ~(size_t)255; }
    if (cudaMalloc(&s->block, total ? total : 256) != cudaSuccess) {
        delete s;
        return cuda_fail(st, cudaGetLastError(), "path tracer scene allocation");
    }
    char* base = (char*)s->block;
    s->nrm = (float*)(base + offs[0]); s->uv = (float*)(base + offs[1]); s->idx = (uint32_t*)(base + offs[2]);
    s->tritex = (uint32_t*)(base + offs[3]); s->texent = (uint32_t*)(base + offs[4]);
    s->texels = (uint32_t*)(base + offs[5]); s->mat = (float*)(base + offs[6]); s->tris = (float*)(base + offs[7]);
    s->emit = (uint32_t*)(base + offs[8]); s->cdf = (float*)(base + offs[9]);
    float* d_pos = (float*)(base + offs[10]);
    std::vector<float> mats((size_t)sd->ntex * 7);
    for (uint32_t k = 0; k < sd->ntex; ++k) {
        const rn_pt_material& m = sd->materials[k];
        const float v[7] = {m.base_factor, m.roughness, m.metallic, m.specular, m.emission[0], m.emission[1], m.emission[2]};
        std::memcpy(&mats[7 * (size_t)k], v, sizeof v);
    }
    const struct { void* d; const void* h; size_t n; } up[] = {
        {s->nrm, sd->nrm, sizes[0]}, {s->uv, sd->uv, sizes[1]}, {s->idx, sd->idx, sizes[2]},
        {s->tritex, sd->tri_texture, sizes[3]}, {s->texent, sd->tex_entries, sizes[4]}, {s->texels, sd->texels, sizes[5]},
        {s->mat, mats.data(), sizes[6]}, {s->emit, emit.data(), sizes[8]}, {s->cdf, cdf.data(), sizes[9]},
        {d_pos, sd->pos, sizes[10]}};
    int rc = RN_OK;
    for (const auto& u : up)
        if (rc == RN_OK && u.n && cudaMemcpyAsync(u.d, u.h, u.n, cudaMemcpyHostToDevice, c.stream) != cudaSuccess)
            rc = cuda_fail(st, cudaGetLastError(), "path tracer scene upload");
    if (rc == RN_OK && nt) {
        gather_tris_kernel<<<(unsigned)((nt + 255) / 256), 256, 0, c.stream>>>(d_pos, s->idx, (uint32_t)nt, s->tris);
        if (cudaGetLastError() != cudaSuccess) rc = cuda_fail(st, cudaGetLastError(), "gather_tris_kernel");
    }
    if (rc == RN_OK) rc = rn_accel_build(s->tris, (uint32_t)nt, RN_DEVICE_PTRS, &s->accel, st);
    // the uploads read the host vectors above: finish them before they go out of scope
    const cudaError_t e = cudaStreamSynchronize(c.stream);
    if (rc == RN_OK && e != cudaSuccess) rc = cuda_fail(st, e, "rn_pt_scene_create");
    if (rc != RN_OK) { rn_pt_scene_free(s); return rc; }
    *out = s;
    return ok(st);
}

void rn_pt_scene_free(rn_ptscene* s) {
    if (!s) return;
    if (s->accel) rn_accel_free(s->accel);
    if (s->block) cudaFree(s->block);
    delete s;
}

int rn_pt_scene_info(const rn_ptscene* s, uint32_t* emitters, float* emitter_area, rn_status* st) {
    if (!s) return fail(st, RN_ERR_INVALID, "null scene");
    if (emitters) *emitters = s->nemit;
    if (emitter_area) *emitter_area = s->area;
    return ok(st);
}

int rn_pathtrace(const rn_ptscene* s, const rn_pt_desc* d, int flags, rn_pt_out* out, rn_status* st) {
    if (!s || !d || !out) return fail(st, RN_ERR_INVALID, "null argument");
    if (d->width <= 0 || d->height <= 0 || (size_t)d->width * (size_t)d->height > ((size_t)1 << 30))
        return fail(st, RN_ERR_INVALID, "frame size %dx%d", d->width, d->height);
    if (d->max_bounces > 1024) return fail(st, RN_ERR_INVALID, "max_bounces %u", d->max_bounces);
    RN_TRY(ensure_ctx(st));
    Context& c = ctx();
    if (s->device != c.device) return fail(st, RN_ERR_STATE, "scene belongs to device %d", s->device);
    const float* table = nullptr;
    RN_TRY(device_table(c.device, &table, st));
    const bool dev = (flags & RN_DEVICE_PTRS) != 0;
    const uint32_t npix = (uint32_t)d->width * (uint32_t)d->height;
    PtParams P{};
    P.nodes = s->accel->d_nodes; P.ltris = s->accel->d_tris; P.has_geometry = s->ntri > 0;
    P.tris = s->tris; P.nrm = s->nrm; P.uv = s->uv; P.idx = s->idx; P.tritex = s->tritex; P.texent = s->texent;
    P.texels = s->texels; P.mat = s->mat; P.emit = s->emit; P.cdf = s->cdf; P.nemit = s->nemit; P.area = s->area;
    P.table = table; P.corr = c.trig_corr;
    const hv3 sd = hnorm(hv3{s->sun_dir[0], s->sun_dir[1], s->sun_dir[2]});
    P.sun_dir = v3{sd.x, sd.y, sd.z};
    P.sun_irr = v3{s->sun_irr[0], s->sun_irr[1], s->sun_irr[2]};
    P.sky = v3{s->sky[0], s->sky[1], s->sky[2]};
    P.seed_lo = (uint32_t)d->seed; P.seed_hi = (uint32_t)(d->seed >> 32);
    P.spp = d->spp; P.spp_begin = d->spp_begin; P.max_bounces = d->max_bounces; P.controls = d->controls;
    P.w = d->width; P.h = d->height; P.jitter = d->jitter != 0; P.rr = d->russian_roulette != 0;
    P.cam = cam_of(d->camera, d->width, d->height);
    P.prev = cam_of(d->previous, d->width, d->height);
    P.npix = npix;
    P.err = c.dev_error;
    // output planes: the caller's device arrays, or one staging block
    const int comps[14] = {3, 3, 3, 1, 1, 1, 2, 3, 3, 3, 3, 3, 1, 1};
    void* user[14] = {out->radiance, out->albedo, out->normal, out->depth, out->variance, out->triangle, out->motion,
                      out->diffuse, out->specular, out->emission, out->diffuse_albedo, out->specular_albedo,
                      out->diffuse_variance, out->specular_variance};
    void* dplane[14] = {};
    if (dev) {
        for (int i = 0; i < 14; ++i) dplane[i] = user[i];
    } else {
        size_t total = 0, offs[14];
        for (int i = 0; i < 14; ++i) { offs[i] = total; if (user[i]) total += ((size_t)npix * comps[i] * 4 + 255) & ~(size_t)255; }
        void* blk = nullptr;
        RN_TRY(ws_get(WS_PT_OUT, total ? total : 256, &blk, st));
        for (int i = 0; i < 14; ++i) dplane[i] = user[i] ? (char*)blk + offs[i] : nullptr;
    }
    PtOutDev O{(float*)dplane[0], (float*)dplane[1], (float*)dplane[2], (float*)dplane[3], (float*)dplane[4],
               (int32_t*)dplane[5], (float*)dplane[6], (float*)dplane[7], (float*)dplane[8], (float*)dplane[9],
               (float*)dplane[10], (float*)dplane[11], (float*)dplane[12], (float*)dplane[13]};
    // slices: at most kSliceBytes of per-sample terms at a time
    const size_t per_sample = (size_t)npix * kSampleFloats * sizeof(float);
    const size_t kSliceBytes = (size_t)1 << 31;
    uint32_t kn_max = (uint32_t)std::max<size_t>(1, std::min<size_t>(d->spp ? d->spp : 1, kSliceBytes / per_sample));
    if (c.tune.pt_slice > 0) kn_max = std::min(kn_max, (uint32_t)c.tune.pt_slice);
    void* samp = nullptr;
    RN_TRY(ws_get(WS_PT_SAMPLES, per_sample * kn_max, &samp, st));
    P.samp = (float*)samp;
    if (d->spp > kn_max) {
        void* acc = nullptr;
        RN_TRY(ws_get(WS_PT_ACC, (size_t)npix * (kSampleFloats * sizeof(float) + 6 * sizeof(double)), &acc, st));
        P.mom = (double*)acc;
        P.acc = (float*)((char*)acc + (size_t)npix * 6 * sizeof(double));
    }
    const uint32_t tiles = ((uint32_t)(d->width + 7) / 8) * ((uint32_t)(d->height + 3) / 4);
    uint32_t* ctr = nullptr;                       // the regeneration kernel's item counter (8 bytes)
    if (c.tune.pt_regen) {
        void* cp = nullptr;
        RN_TRY(ws_get(WS_PT_CTR, 8, &cp, st));
        ctr = (uint32_t*)cp;
    }
    // the wavefront form's slots (pt_wave x 1024 at most)
    WaveBufs W{};
    if (c.tune.pt_wave) {
        const unsigned long long most = (unsigned long long)tiles * 32ull * kn_max;
        W.Q = (uint32_t)std::min<unsigned long long>(most, (unsigned long long)c.tune.pt_wave * 1024ull);
        const size_t Q = W.Q;
        size_t off = 0;
        auto take = [&](size_t bytes) { const size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
        const size_t o_f = take(wave::NF * Q * 4), o_u = take(wave::NU * Q * 4), o_vis = take(2 * Q);
        const size_t o_qf = take(7 * 2 * Q * 4), o_qu = take(2 * Q * 4), o_ctr = take(16);
        void* blk = nullptr;
        RN_TRY(ws_get(WS_PT_WAVE, off, &blk, st));
        char* b8 = (char*)blk;
        W.f = (float*)(b8 + o_f); W.u = (uint32_t*)(b8 + o_u); W.vis = (uint8_t*)(b8 + o_vis);
        W.qf = (float*)(b8 + o_qf); W.qu = (uint32_t*)(b8 + o_qu); W.ctr = (uint32_t*)(b8 + o_ctr);
    }
    uint32_t k0 = 0;
    do {
        P.k0 = k0;
        P.kn = std::min(kn_max, d->spp - k0);
        P.first = k0 == 0;
        P.last = k0 + P.kn >= d->spp;
        if (P.kn > 0 && c.tune.pt_wave) {
            // every slot free, the counts at zero; then shade -> shadow rays -> closest hits
            // until a shade pass leaves no live slot (read every 8 passes)
            const unsigned long long total = (unsigned long long)tiles * 32ull * P.kn;
            RN_CUDA(cudaMemsetAsync(W.u + (size_t)wave::UFL * W.Q, 0, (size_t)W.Q * 4, c.stream), st);
            RN_CUDA(cudaMemsetAsync(W.ctr, 0, 16, c.stream), st);
            const unsigned grid = (W.Q + 127) / 128, sgrid = (unsigned)c.sm_count * 8u;
            const unsigned long long max_passes = (total / W.Q + 2) * ((unsigned long long)d->max_bounces + 3) + 64;
            bool done = false;
            for (unsigned long long pass = 0; !done; ++pass) {
                if (pass > max_passes) return fail(st, RN_ERR_BUDGET, "path tracer: more than %llu passes", max_passes);
                switch (c.tune.pt_shade_blocks) {   // resident blocks per SM: a register budget
                    case 6: pt_wave_shade<6><<<grid, 128, 0, c.stream>>>(P, W, total); break;
                    case 8: pt_wave_shade<8><<<grid, 128, 0, c.stream>>>(P, W, total); break;
                    default: pt_wave_shade<4><<<grid, 128, 0, c.stream>>>(P, W, total); break;
                }
                if ((pass & 7) == 7) {
                    uint32_t live = 0;
                    RN_CUDA(cudaMemcpyAsync(&live, W.ctr + 1, 4, cudaMemcpyDeviceToHost, c.stream), st);
                    RN_CUDA(cudaStreamSynchronize(c.stream), st);
                    done = live == 0;
                }
                if (!done) {
                    pt_wave_shadow<<<sgrid, 128, 0, c.stream>>>(P, W);
                    pt_wave_extend<<<grid, 128, 0, c.stream>>>(P, W);
                }
                const cudaError_t le = cudaGetLastError();
                if (le != cudaSuccess) return cuda_fail(st, le, "pt_wave kernels");
            }
        } else if (P.kn > 0 && c.tune.pt_regen) {
            RN_CUDA(cudaMemsetAsync(ctr, 0, 8, c.stream), st);
            pt_regen_kernel<<<c.sm_count * c.tune.pt_regen, 128, 0, c.stream>>>(P, ctr);
            const cudaError_t le = cudaGetLastError();
            if (le != cudaSuccess) return cuda_fail(st, le, "pt_regen_kernel");
        } else if (P.kn > 0) {
            const uint64_t warps = (uint64_t)tiles * P.kn;
            pt_paths_kernel<<<(unsigned)((warps + 3) / 4), 128, 0, c.stream>>>(P);
            const cudaError_t le = cudaGetLastError();
            if (le != cudaSuccess) return cuda_fail(st, le, "pt_paths_kernel");
        }
        pt_accum_kernel<<<(npix + 127) / 128, 128, 0, c.stream>>>(P, O);
        const cudaError_t le = cudaGetLastError();
        if (le != cudaSuccess) return cuda_fail(st, le, "pt_accum_kernel");
        k0 += P.kn;
    } while (k0 < d->spp);
    if (!dev)
        for (int i = 0; i < 14; ++i)
            if (user[i]) RN_CUDA(cudaMemcpyAsync(user[i], dplane[i], (size_t)npix * comps[i] * 4, cudaMemcpyDeviceToHost,
                                                 c.stream), st);
    RN_CUDA(cudaStreamSynchronize(c.stream), st);
    RN_TRY(check_device_error(st, "rn_pathtrace"));
    return ok(st);
}

}  // extern "C"
