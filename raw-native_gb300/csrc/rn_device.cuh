// rn_device.cuh -- device-side building blocks of the AO path, shared by every kernel.
//
// Exactness contract. The reference defines its answers with float32 operations in a fixed
// order on a host without fused multiply-add. Every helper here that feeds a parity-checked
// value uses the explicitly rounded intrinsics (__fadd_rn, __fmul_rn, __fdiv_rn, __fsqrt_rn):
// one IEEE round-to-nearest per operation, never contracted, whatever -fmad says. Code that
// only needs to be conservative (box tests) may use anything faster.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace rn {

// ------------------------------------------------------------------ exact float32 ops
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }
// 1 / a rounded once to nearest: the same value as fdiv(1.0f, a) (both are the correctly
// rounded quotient), from the cheaper reciprocal intrinsic.
__device__ __forceinline__ float frcp(float a) { return __frcp_rn(a); }
// std::min / std::max on floats: (b < a) ? b : a and (a < b) ? b : a.
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }

struct v3 { float x, y, z; };
__device__ __forceinline__ v3 mk(float x, float y, float z) { return v3{x, y, z}; }
__device__ __forceinline__ v3 add(v3 a, v3 b) { return mk(fadd(a.x, b.x), fadd(a.y, b.y), fadd(a.z, b.z)); }
__device__ __forceinline__ v3 sub(v3 a, v3 b) { return mk(fsub(a.x, b.x), fsub(a.y, b.y), fsub(a.z, b.z)); }
__device__ __forceinline__ v3 scale(v3 a, float s) { return mk(fmul(a.x, s), fmul(a.y, s), fmul(a.z, s)); }
// raw/math/vec.hpp:11-16: dot sums left to right; cross as written there.
__device__ __forceinline__ float dot(v3 a, v3 b) { return fadd(fadd(fmul(a.x, b.x), fmul(a.y, b.y)), fmul(a.z, b.z)); }
__device__ __forceinline__ v3 cross(v3 a, v3 b) {
    return mk(fsub(fmul(a.y, b.z), fmul(a.z, b.y)), fsub(fmul(a.z, b.x), fmul(a.x, b.z)),
              fsub(fmul(a.x, b.y), fmul(a.y, b.x)));
}
__device__ __forceinline__ float length(v3 v) { return fsqrt(dot(v, v)); }
__device__ __forceinline__ v3 normalize(v3 v) {
    const float l = length(v);
    return l > 0.0f ? scale(v, frcp(l)) : v;
}
__device__ __forceinline__ v3 load3(const float* p) { return mk(p[0], p[1], p[2]); }
__device__ __forceinline__ void store3(float* p, const v3& v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }

// ------------------------------------------------------------------ sampler
// src/renderer/ray_ao.cpp:8-12 (and ssao.cpp:6-10): integer hash, exact float in [0,1).
__device__ __forceinline__ uint32_t hash24(uint32_t x, uint32_t y, uint32_t s) {
    uint32_t h = x * 374761393u + y * 668265263u + s * 2246822519u;
    h = (h ^ (h >> 13)) * 1274126177u;
    h ^= h >> 16;
    return h & 0xFFFFFFu;
}
// (h & 0xFFFFFF) / 2^24: the division by a power of two is exact, so a multiply by 2^-24 is
// the same value.
__device__ __forceinline__ float unit24(uint32_t k) { return fmul((float)k, 5.9604644775390625e-8f); }

// The sample angle of 24-bit index k: phi = 6.2831853f * (k / 2^24), as both passes form it.
__device__ __forceinline__ float sample_angle(uint32_t k) { return fmul(6.2831853f, unit24(k)); }

// sin and cos of an angle in [0, 2 pi) on the device: a three-constant Cody-Waite reduction
// by pi/2 (1.5703125 + 4.838267923e-4 + 2.563344068e-12; the first product is exact) to
// |r| <= pi/4, then the Taylor series of sin to r^11 and of cos to r^12 in Horner form
// (truncation below 2e-10). About one unit in the last place; the correction table below
// supplies the host's last bits. No slow path: the argument range is fixed.
__device__ __forceinline__ void angle_sincos(float phi, float& s, float& c) {
    const float j = rintf(phi * 0.636619772f);
    float r = __fmaf_rn(-j, 1.5703125f, phi);
    r = __fmaf_rn(-j, 4.838267923e-4f, r);
    r = __fmaf_rn(-j, 2.563344068e-12f, r);
    const float r2 = r * r;
    float ps = __fmaf_rn(r2, -2.50521084e-8f, 2.75573192e-6f);
    ps = __fmaf_rn(r2, ps, -1.98412698e-4f);
    ps = __fmaf_rn(r2, ps, 8.33333333e-3f);
    ps = __fmaf_rn(r2, ps, -1.66666667e-1f);
    const float sr = __fmaf_rn(r * r2, ps, r);
    float pc = __fmaf_rn(r2, 2.08767570e-9f, -2.75573192e-7f);
    pc = __fmaf_rn(r2, pc, 2.48015873e-5f);
    pc = __fmaf_rn(r2, pc, -1.38888889e-3f);
    pc = __fmaf_rn(r2, pc, 4.16666667e-2f);
    pc = __fmaf_rn(r2, pc, -0.5f);
    const float cr = __fmaf_rn(r2, pc, 1.0f);
    const int q = (int)j & 3;
    s = q == 0 ? sr : q == 1 ? cr : q == 2 ? -sr : -cr;
    c = q == 0 ? cr : q == 1 ? -sr : q == 2 ? -cr : sr;
}

// cos and sin of the sample angle with the host C library's bits. The reference takes
// std::cos/std::sin of a float (the host libm's cosf/sinf), which differ from the correctly
// rounded value on about 1.3% of these 2^24 angles. `corr` holds one byte per angle, the
// cos difference in the low nibble and the sin difference in the high nibble (two's
// complement, in units in the last place) between the host's value and angle_sincos's,
// built once per process over every angle; adding it to the bit pattern gives the host's
// value exactly (a caller may fetch the byte ahead and use apply_corr). corr == nullptr
// selects the device function alone.
__device__ __forceinline__ float bump_ulps(float v, int d) { return __int_as_float(__float_as_int(v) + d); }
__device__ __forceinline__ void apply_corr(int d, float& c, float& s) {
    c = bump_ulps(c, ((d & 15) ^ 8) - 8);
    s = bump_ulps(s, ((d >> 4) ^ 8) - 8);
}
__device__ __forceinline__ void sample_sincos(uint32_t k, const uint8_t* __restrict__ corr, float& c, float& s) {
    angle_sincos(sample_angle(k), s, c);
    if (corr) apply_corr(__ldg(corr + k), c, s);
}

// ------------------------------------------------------------------ rays
// Per-ray constants of the watertight test (raw/math/primitives.hpp:17-20, :32-37): the
// axis permutation kz, the x/y swap, and the shear sx, sy, sz.
struct WRay {
    v3 o, d;
    int kz;
    bool sw;
    float sx, sy, sz;
};
__device__ __forceinline__ v3 wframe(v3 v, int kz, bool sw) {
    const v3 p = kz == 0 ? mk(v.y, v.z, v.x) : kz == 1 ? mk(v.z, v.x, v.y) : v;
    return sw ? mk(p.y, p.x, p.z) : p;
}
__device__ __forceinline__ WRay make_wray(v3 o, v3 d) {
    WRay r;
    r.o = o; r.d = d;
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    r.kz = ax > ay ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    v3 q = wframe(d, r.kz, false);
    r.sw = q.z < 0.0f;
    if (r.sw) q = mk(q.y, q.x, q.z);
    r.sx = fdiv(q.x, q.z); r.sy = fdiv(q.y, q.z); r.sz = frcp(q.z);
    return r;
}

// The reference's hit rule (raw/math/primitives.hpp:31-64): the watertight sign test
// decides; t comes from Moeller-Trumbore unless its determinant is within 1e-7 of zero,
// then from the sheared sums. Returns true with t when the test accepts and t > 1e-4.
// u and v are not formed: no caller of the AO path reads them.
__device__ __forceinline__ bool hit_tri(const WRay& r, v3 a, v3 b, v3 c, float& t) {
    const v3 A = wframe(sub(a, r.o), r.kz, r.sw), B = wframe(sub(b, r.o), r.kz, r.sw),
             C = wframe(sub(c, r.o), r.kz, r.sw);
    const float Ax = fsub(A.x, fmul(r.sx, A.z)), Ay = fsub(A.y, fmul(r.sy, A.z));
    const float Bx = fsub(B.x, fmul(r.sx, B.z)), By = fsub(B.y, fmul(r.sy, B.z));
    const float Cx = fsub(C.x, fmul(r.sx, C.z)), Cy = fsub(C.y, fmul(r.sy, C.z));
    const float U = fsub(fmul(Cx, By), fmul(Cy, Bx));
    const float V = fsub(fmul(Ax, Cy), fmul(Ay, Cx));
    const float W = fsub(fmul(Bx, Ay), fmul(By, Ax));
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = fadd(fadd(U, V), W);
    if (det == 0.0f) return false;
    const v3 e1 = sub(b, a), e2 = sub(c, a), p = cross(r.d, e2);
    const float dm = dot(e1, p);
    if (dm > -1e-7f && dm < 1e-7f) {
        const float T = fadd(fadd(fmul(U, fmul(r.sz, A.z)), fmul(V, fmul(r.sz, B.z))), fmul(W, fmul(r.sz, C.z)));
        t = fmul(T, frcp(det));
    } else {
        const float inv = frcp(dm);
        const v3 q = cross(sub(r.o, a), e1);
        t = fmul(dot(e2, q), inv);
    }
    return t > 1e-4f;
}

// The same test with the barycentrics the closest-hit consumers read (primitives.hpp:52-63):
// u and v from the sheared sums where Moeller-Trumbore's determinant is unusable, else
// Moeller-Trumbore's, clamped at 0 and renormalized when their sum passes 1.
__device__ __forceinline__ bool hit_tri_uv(const WRay& r, v3 a, v3 b, v3 c, float& t, float& u, float& v) {
    const v3 A = wframe(sub(a, r.o), r.kz, r.sw), B = wframe(sub(b, r.o), r.kz, r.sw),
             C = wframe(sub(c, r.o), r.kz, r.sw);
    const float Ax = fsub(A.x, fmul(r.sx, A.z)), Ay = fsub(A.y, fmul(r.sy, A.z));
    const float Bx = fsub(B.x, fmul(r.sx, B.z)), By = fsub(B.y, fmul(r.sy, B.z));
    const float Cx = fsub(C.x, fmul(r.sx, C.z)), Cy = fsub(C.y, fmul(r.sy, C.z));
    const float U = fsub(fmul(Cx, By), fmul(Cy, Bx));
    const float V = fsub(fmul(Ax, Cy), fmul(Ay, Cx));
    const float W = fsub(fmul(Bx, Ay), fmul(By, Ax));
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = fadd(fadd(U, V), W);
    if (det == 0.0f) return false;
    const v3 e1 = sub(b, a), e2 = sub(c, a), p = cross(r.d, e2);
    const float dm = dot(e1, p);
    if (dm > -1e-7f && dm < 1e-7f) {
        const float T = fadd(fadd(fmul(U, fmul(r.sz, A.z)), fmul(V, fmul(r.sz, B.z))), fmul(W, fmul(r.sz, C.z)));
        const float inv = frcp(det);
        t = fmul(T, inv); u = fmul(V, inv); v = fmul(W, inv);
        return t > 1e-4f;
    }
    const float inv = frcp(dm);
    const v3 tv = sub(r.o, a), q = cross(tv, e1);
    u = smax(0.0f, fmul(dot(tv, p), inv));
    v = smax(0.0f, fmul(dot(r.d, q), inv));
    t = fmul(dot(e2, q), inv);
    const float s = fadd(u, v);
    if (s > 1.0f) { u = fdiv(u, s); v = fdiv(v, s); }
    return t > 1e-4f;
}

// ------------------------------------------------------------------ misc
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Order-preserving float <-> uint maps for atomicMin/atomicMax on floats.
__device__ __forceinline__ unsigned f2ord(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

}  // namespace rn
