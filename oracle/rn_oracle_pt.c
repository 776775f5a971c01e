/*
 * rn_oracle_pt.c -- CPU restatement of raw-native's path tracer (interface v4, the v2 scene
 * path: raw::rt::pathTraceCpu for a scene without v3 fields). Included at the end of
 * rn_oracle.c and built into the same librn_oracle.so.
 *
 * TEST INFRASTRUCTURE ONLY, like the rest of the oracle: the GPU path tracer is compared
 * against it; nothing in the product links it.
 *
 * Float32 in the reference's operation order (one rounding per operator, sums left to
 * right, no contraction: build with -ffp-contract=off), the moments in float64 as the
 * reference keeps them, the energy table built in float64 as the reference builds it.
 * Sources followed (paths inside the raw-native tree):
 *   src/renderer/rt_pt_math.hpp      PCG2D, frame, GGX, VNDF sampling, the v4 lobe, energy reads
 *   src/renderer/rt_pt_energy.cpp    the energy table
 *   src/renderer/pbr_tables.cpp:11-58  the split albedo by VNDF sampling (albedoSplit)
 *   src/renderer/brdf.cpp:95-109     Gauss-Legendre nodes on [0, 1]
 *   src/renderer/rt_pt_ctx.hpp       the hit surface, the offset, next-event estimation
 *   src/renderer/rt_pt_cpu.cpp       tracePath, the camera, the per-pixel loop, the moments
 *   src/renderer/rt_pt_scene.cpp:31-45  the emitter list and its area CDF (finishPtScene)
 *   src/renderer/rt_bvh.cpp:125-157  closest hit (ties to the lowest index) and occlusion
 * The closest hit runs over the oracle's own SAH BVH (a conservative box test over the
 * reference's triangle test: the nearest t, ties to the lowest triangle index, which is
 * the answer of the reference's PLOC walk and of a scan of every triangle).
 */

/* ------------------------------------------------------------------ energy table (float64) */
#define PT_MU 64
#define PT_ROUGH 128
#define PT_NODES (PT_MU * PT_ROUGH * 2)
#define PT_FLOATS (PT_NODES + PT_ROUGH * 2)
static const double kPiD = 3.14159265358979323846;
static const float kPiF = 3.14159265f;

static double pt_radical_inverse(uint32_t b) {
    b = (b << 16) | (b >> 16);
    b = ((b & 0x55555555u) << 1) | ((b & 0xAAAAAAAAu) >> 1);
    b = ((b & 0x33333333u) << 2) | ((b & 0xCCCCCCCCu) >> 2);
    b = ((b & 0x0F0F0F0Fu) << 4) | ((b & 0xF0F0F0F0u) >> 4);
    b = ((b & 0x00FF00FFu) << 8) | ((b & 0xFF00FF00u) >> 8);
    return b * 2.3283064365386963e-10;
}
static double pt_lambda_d(double mu, double a) {
    const double m2 = mu * mu;
    return 0.5 * (-1.0 + sqrt(1.0 + a * a * (1.0 - m2) / m2));
}
/* src/renderer/pbr_tables.cpp:23-50: A and B of the white single-scattering lobe at (mu, alpha). */
static void pt_albedo_split(double mu, double a, int n, double* outA, double* outB) {
    const double vx = sqrt((0.0 < 1.0 - mu * mu) ? 1.0 - mu * mu : 0.0), vy = 0.0, vz = mu;
    const double vhx = a * vx, vhz = vz;
    const double lv = sqrt(vhx * vhx + vhz * vhz);
    const double vnx = vhx / lv, vny = 0.0, vnz = vhz / lv;
    const double t1x = 0.0, t1y = 1.0, t1z = 0.0;
    const double t2x = vny * t1z - vnz * t1y, t2y = vnz * t1x - vnx * t1z, t2z = vnx * t1y - vny * t1x;
    const double g1 = 1.0 / (1.0 + pt_lambda_d(mu, a));
    double sa = 0.0, sb = 0.0;
    for (int k = 0; k < n; ++k) {
        const double u1 = (k + 0.5) / n, u2 = pt_radical_inverse((uint32_t)k);
        const double r = sqrt(u1), phi = 2.0 * kPiD * u2, s = 0.5 * (1.0 + vnz);
        const double p1 = r * cos(phi), p2 = (1.0 - s) * sqrt(1.0 - p1 * p1) + s * r * sin(phi);
        const double q = 1.0 - p1 * p1 - p2 * p2;
        const double p3 = sqrt((0.0 < q) ? q : 0.0);
        double mx = t1x * p1 + t2x * p2 + vnx * p3, my = t1y * p1 + t2y * p2 + vny * p3,
               mz = t1z * p1 + t2z * p2 + vnz * p3;
        mx = a * mx; my = a * my; mz = (1e-12 < mz) ? mz : 1e-12;
        const double lm = sqrt(mx * mx + my * my + mz * mz);
        mx = mx / lm; my = my / lm; mz = mz / lm;
        const double vom = vx * mx + vy * my + vz * mz, li = 2.0 * vom * mz - vz;
        if (li <= 0.0) continue;
        const double w = (1.0 / (1.0 + pt_lambda_d(mu, a) + pt_lambda_d(li, a))) / g1;
        const double c = 1.0 - vom, c5 = c * c * c * c * c;
        sa += w * (1.0 - c5); sb += w * c5;
    }
    *outA = sa / n; *outB = sb / n;
}
/* src/renderer/brdf.cpp:95-109: n Gauss-Legendre nodes and weights on [0, 1]. */
static void pt_gauss_legendre01(int n, double* x, double* w) {
    for (int i = 0; i < n; ++i) {
        double z = cos(kPiD * (i + 0.75) / (n + 0.5)), pp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p1 = 1.0, p2 = 0.0;
            for (int j = 1; j <= n; ++j) { const double p3 = p2; p2 = p1; p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j; }
            pp = n * (z * p1 - p2) / (z * z - 1.0);
            const double z1 = z;
            z = z1 - p1 / pp;
            if (fabs(z - z1) < 1e-15) break;
        }
        x[i] = 0.5 * (1.0 - z); w[i] = 1.0 / ((1.0 - z * z) * pp * pp);
    }
}
static inline float pt_clampf(float v, float lo, float hi) { return (v < lo) ? lo : (hi < v) ? hi : v; }
/* rt_pt_math.hpp:93-107: bilinear (A, B) in (sqrt(mu), roughness), and a row's means. */
static void pt_table_ab(const float* t, float mu, float rough, float* A, float* B) {
    const int N = PT_MU, R = PT_ROUGH;
    const float x = sqrtf(pt_clampf(mu, 0.0f, 1.0f)) * (float)(N - 1), y = pt_clampf(rough, 0.0f, 1.0f) * (float)(R - 1);
    const int x0 = (int)x < N - 2 ? (int)x : N - 2, y0 = (int)y < R - 2 ? (int)y : R - 2;
    const float fx = x - (float)x0, fy = y - (float)y0;
    const float* p = t + ((size_t)y0 * N + (size_t)x0) * 2;
    const float* q = p + (size_t)N * 2;
    const float a0 = p[0] * (1.0f - fx) + p[2] * fx, b0 = p[1] * (1.0f - fx) + p[3] * fx;
    const float a1 = q[0] * (1.0f - fx) + q[2] * fx, b1 = q[1] * (1.0f - fx) + q[3] * fx;
    *A = a0 * (1.0f - fy) + a1 * fy; *B = b0 * (1.0f - fy) + b1 * fy;
}
static void pt_table_avg(const float* t, float rough, float* A, float* B) {
    const int R = PT_ROUGH;
    const float y = pt_clampf(rough, 0.0f, 1.0f) * (float)(R - 1);
    const int y0 = (int)y < R - 2 ? (int)y : R - 2;
    const float fy = y - (float)y0;
    const float* p = t + PT_NODES + (size_t)y0 * 2;
    *A = p[0] * (1.0f - fy) + p[2] * fy; *B = p[1] * (1.0f - fy) + p[3] * fy;
}
typedef struct { float* t; int row0, rows; } pt_table_job;
static void pt_table_row(void* ctx, int i) {
    float* t = (float*)ctx;
    const double r = (double)i / (PT_ROUGH - 1), r2 = r * r, a = (1e-4 < r2) ? r2 : 1e-4;
    for (int j = 0; j < PT_MU; ++j) {
        const double u = (double)j / (PT_MU - 1), u2 = u * u, mu = (u2 < 1e-4) ? 1e-4 : u2;
        double A = 0.0, B = 0.0;
        pt_albedo_split(mu, a, 1 << 12, &A, &B);
        t[((size_t)i * PT_MU + (size_t)j) * 2] = (float)A;
        t[((size_t)i * PT_MU + (size_t)j) * 2 + 1] = (float)B;
    }
}
/* src/renderer/rt_pt_energy.cpp:11-40: the nodes (rows in parallel, one thread a row), then
 * each row's cosine-weighted means of the float table as pt_table_ab reads it. */
RNO_API int rno_pt_energy_table(float* t, int threads) {
    parallel_rows(PT_ROUGH, threads, pt_table_row, t);
    double x[64], w[64];
    pt_gauss_legendre01(64, x, w);
    for (int i = 0; i < PT_ROUGH; ++i) {
        const float r = (float)i / (float)(PT_ROUGH - 1);
        double sa = 0.0, sb = 0.0;
        for (int k = 0; k < 64; ++k) {
            float A, B;
            pt_table_ab(t, (float)x[k], r, &A, &B);
            sa += w[k] * (double)A * x[k]; sb += w[k] * (double)B * x[k];
        }
        t[PT_NODES + (size_t)i * 2] = (float)(2.0 * sa);
        t[PT_NODES + (size_t)i * 2 + 1] = (float)(2.0 * sb);
    }
    return PT_FLOATS;
}

/* ------------------------------------------------------------------ random numbers, frame */
static inline void pt_pcg2d(uint32_t* x, uint32_t* y) {
    *x = *x * 1664525u + 1013904223u; *y = *y * 1664525u + 1013904223u;
    *x += *y * 1664525u; *y += *x * 1664525u;
    *x ^= *x >> 16; *y ^= *y >> 16;
    *x += *y * 1664525u; *y += *x * 1664525u;
    *x ^= *x >> 16; *y ^= *y >> 16;
}
typedef struct { float a, b; } pt_r2;
static inline pt_r2 pt_rand2(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t dim) {
    uint32_t x = pixel ^ ((uint32_t)seed * 0x9E3779B9u), y = (sample * 64u + dim) ^ (uint32_t)(seed >> 32);
    pt_pcg2d(&x, &y);
    pt_r2 r = {(float)(x >> 8) * 5.96046448e-8f, (float)(y >> 8) * 5.96046448e-8f};
    return r;
}
typedef struct { v3 t, b, n; } pt_frame;
static inline pt_frame pt_basis(v3 n) {
    const float s = n.z >= 0.0f ? 1.0f : -1.0f;
    const float a = -1.0f / (s + n.z), c = n.x * n.y * a;
    pt_frame f = {v3m(1.0f + s * n.x * n.x * a, s * c, -s * n.x), v3m(c, s + n.y * n.y * a, -n.y), n};
    return f;
}
static inline v3 pt_to_local(const pt_frame* f, v3 v) { return v3m(dot3(v, f->t), dot3(v, f->b), dot3(v, f->n)); }
static inline v3 pt_to_world(const pt_frame* f, v3 v) { return add3(add3(mul3(f->t, v.x), mul3(f->b, v.y)), mul3(f->n, v.z)); }
static inline v3 pt_mulv(v3 a, v3 b) { return v3m(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline float pt_maxc(v3 a) { return smax(a.x, smax(a.y, a.z)); }
static inline float pt_lum(v3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

/* ------------------------------------------------------------------ the lobe (rt_pt_math.hpp:62-210) */
static inline float pt_ggx_d(float a2, float cosH) {
    const float d = cosH * cosH * (a2 - 1.0f) + 1.0f;
    return a2 / (kPiF * d * d);
}
static inline float pt_lambda(float a2, float cosT) {
    const float c2 = cosT * cosT;
    return (-1.0f + sqrtf(1.0f + a2 * (1.0f - c2) / c2)) * 0.5f;
}
static v3 pt_sample_vndf(v3 wo, float a, float u1, float u2) {
    const v3 vh = norm3(v3m(a * wo.x, a * wo.y, wo.z));
    const float lensq = vh.x * vh.x + vh.y * vh.y;
    const v3 t1 = lensq > 0.0f ? mul3(v3m(-vh.y, vh.x, 0.0f), 1.0f / sqrtf(lensq)) : v3m(1.0f, 0.0f, 0.0f);
    const v3 t2 = cross3(vh, t1);
    const float r = sqrtf(u1), phi = 2.0f * kPiF * u2;
    const float p1 = r * cosf(phi), s = 0.5f * (1.0f + vh.z);
    const float p2 = (1.0f - s) * sqrtf(smax(0.0f, 1.0f - p1 * p1)) + s * (r * sinf(phi));
    const v3 nh = add3(add3(mul3(t1, p1), mul3(t2, p2)), mul3(vh, sqrtf(smax(0.0f, 1.0f - p1 * p1 - p2 * p2))));
    return norm3(v3m(a * nh.x, a * nh.y, smax(0.0f, nh.z)));
}
typedef struct { v3 base; float rough, metallic, specular; int legacy; const float* table; } pt_bsdf;
static inline float pt_lobe_prob(const pt_bsdf* m) { return m->metallic + (1.0f - m->metallic) * 0.5f * m->specular; }
static inline v3 pt_f0(const pt_bsdf* m) {
    const float d = 0.04f * m->specular;
    return v3m(d + (m->base.x - d) * m->metallic, d + (m->base.y - d) * m->metallic, d + (m->base.z - d) * m->metallic);
}
static inline float pt_kms(float favg, float eavg) { return favg * favg * eavg / (1.0f - favg * (1.0f - eavg)); }
typedef struct { float ms, wd, kd, eavg; } pt_energy;
static pt_energy pt_energy_of(const pt_bsdf* m, float muO, float muI) {
    float oa, ob, ia, ib, aa, ab;
    pt_table_ab(m->table, muO, m->rough, &oa, &ob);
    pt_table_ab(m->table, muI, m->rough, &ia, &ib);
    pt_table_avg(m->table, m->rough, &aa, &ab);
    const float eo = smin(1.0f, oa + ob), ei = smin(1.0f, ia + ib), ea = smin(1.0f, aa + ab);
    pt_energy e;
    e.eavg = ea;
    e.ms = ea < 1.0f ? (1.0f - eo) * (1.0f - ei) / (kPiF * (1.0f - ea)) : 0.0f;
    const float on = m->specular > 0.0f ? 1.0f : 0.0f, d = 0.04f * m->specular;
    e.kd = pt_kms(on * (d + (1.0f - d) / 21.0f), ea);
    const float eso = on * (d * oa + ob) + e.kd * (1.0f - eo), esi = on * (d * ia + ib) + e.kd * (1.0f - ei);
    const float esa = on * (d * aa + ab) + e.kd * (1.0f - ea);
    e.wd = (1.0f - eso) * (1.0f - esi) / (1.0f - esa);
    return e;
}
typedef struct { v3 fcos; float pdf; } pt_eval;
static pt_eval pt_eval_legacy(const pt_bsdf* m, v3 wo, v3 wi, int dropCosine) {
    pt_eval r = {{0, 0, 0}, 0.0f};
    if (wo.z <= 0.0f || wi.z <= 0.0f) return r;
    const float ps = pt_lobe_prob(m), cosI = dropCosine ? 1.0f : wi.z;
    const float kd = (1.0f - m->metallic) / kPiF;
    v3 f = v3m(m->base.x * kd, m->base.y * kd, m->base.z * kd);
    float pdf = (1.0f - ps) * wi.z / kPiF;
    if (ps > 0.0f) {
        const float a = smax(1e-4f, m->rough * m->rough), a2 = a * a;
        const v3 h = norm3(add3(wo, wi));
        const float oh = dot3(wo, h), D = pt_ggx_d(a2, h.z);
        const float G2 = 1.0f / (1.0f + pt_lambda(a2, wo.z) + pt_lambda(a2, wi.z)), G1 = 1.0f / (1.0f + pt_lambda(a2, wo.z));
        const float x1 = pt_clampf(1.0f - oh, 0.0f, 1.0f);
        const float fw = x1 * x1 * x1 * x1 * x1;
        const v3 F0 = pt_f0(m);
        const v3 F = v3m(F0.x + (1.0f - F0.x) * fw, F0.y + (1.0f - F0.y) * fw, F0.z + (1.0f - F0.z) * fw);
        const float spec = D * G2 / (4.0f * wo.z * wi.z);
        f = add3(f, mul3(F, spec));
        pdf += ps * (G1 * D / (4.0f * wo.z));
    }
    r.fcos = mul3(f, cosI); r.pdf = pdf;
    return r;
}
static inline float pt_km(const pt_bsdf* m, float b, const pt_energy* en) {
    return m->metallic * pt_kms(b + (1.0f - b) / 21.0f, en->eavg) + (1.0f - m->metallic) * en->kd;
}
static pt_eval pt_eval_bsdf(const pt_bsdf* m, v3 wo, v3 wi, int dropCosine) {
    if (m->legacy) return pt_eval_legacy(m, wo, wi, dropCosine);
    pt_eval r = {{0, 0, 0}, 0.0f};
    if (wo.z <= 0.0f || wi.z <= 0.0f) return r;
    const float ps = pt_lobe_prob(m), cosI = dropCosine ? 1.0f : wi.z;
    const float kd = (1.0f - m->metallic) / kPiF;
    v3 f = v3m(m->base.x * kd, m->base.y * kd, m->base.z * kd);
    float pdf = (1.0f - ps) * wi.z / kPiF;
    if (ps > 0.0f) {
        const pt_energy en = pt_energy_of(m, wo.z, wi.z);
        f = mul3(f, en.wd);
        const float a = smax(1e-4f, m->rough * m->rough), a2 = a * a;
        const v3 h = norm3(add3(wo, wi));
        const float oh = dot3(wo, h), D = pt_ggx_d(a2, h.z);
        const float G2 = 1.0f / (1.0f + pt_lambda(a2, wo.z) + pt_lambda(a2, wi.z)), G1 = 1.0f / (1.0f + pt_lambda(a2, wo.z));
        const float x1 = pt_clampf(1.0f - oh, 0.0f, 1.0f);
        const float fw = x1 * x1 * x1 * x1 * x1;
        const v3 F0 = pt_f0(m);
        const float f90 = m->metallic + (1.0f - m->metallic) * (m->specular > 0.0f ? 1.0f : 0.0f);
        const v3 F = v3m(F0.x + (f90 - F0.x) * fw, F0.y + (f90 - F0.y) * fw, F0.z + (f90 - F0.z) * fw);
        const float spec = D * G2 / (4.0f * wo.z * wi.z);
        const v3 kms = v3m(pt_km(m, m->base.x, &en), pt_km(m, m->base.y, &en), pt_km(m, m->base.z, &en));
        f = add3(add3(f, mul3(F, spec)), mul3(kms, en.ms));
        pdf += ps * (G1 * D / (4.0f * wo.z));
    }
    r.fcos = mul3(f, cosI); r.pdf = pdf;
    return r;
}
static v3 pt_lambert_cos(const pt_bsdf* m, v3 wo, v3 wi, int dropCosine) {
    if (wo.z <= 0.0f || wi.z <= 0.0f) return v3m(0, 0, 0);
    const float cosI = dropCosine ? 1.0f : wi.z, kd = (1.0f - m->metallic) / kPiF;
    v3 f = v3m(m->base.x * kd, m->base.y * kd, m->base.z * kd);
    if (!m->legacy && pt_lobe_prob(m) > 0.0f) f = mul3(f, pt_energy_of(m, wo.z, wi.z).wd);
    return mul3(f, cosI);
}
static v3 pt_spec_albedo(const pt_bsdf* m, float cosO) {
    if (pt_lobe_prob(m) <= 0.0f) return v3m(0, 0, 0);
    const float x1 = pt_clampf(1.0f - cosO, 0.0f, 1.0f), fw = x1 * x1 * x1 * x1 * x1;
    const v3 F0 = pt_f0(m);
    return v3m(F0.x + (1.0f - F0.x) * fw, F0.y + (1.0f - F0.y) * fw, F0.z + (1.0f - F0.z) * fw);
}
static int pt_sample_bsdf(const pt_bsdf* m, v3 wo, float pick, float u1, float u2, v3* wi) {
    if (pick < pt_lobe_prob(m)) {
        const float a = smax(1e-4f, m->rough * m->rough);
        const v3 h = pt_sample_vndf(wo, a, u1, u2);
        *wi = sub3(mul3(h, 2.0f * dot3(wo, h)), wo);
    } else {
        const float r = sqrtf(u1), phi = 2.0f * kPiF * u2;
        *wi = v3m(r * cosf(phi), r * sinf(phi), sqrtf(smax(0.0f, 1.0f - u1)));
    }
    return wi->z > 0.0f;
}

/* ------------------------------------------------------------------ scene and queries */
typedef struct {               /* the plain-array scene (ref_harness_pt.cpp's PtSceneIn) */
    const float* pos; const float* nrm; const float* uv; uint32_t nvert;
    const uint32_t* idx; const uint32_t* triTex; uint32_t ntri;
    const uint32_t* texEntries; uint32_t ntex;
    const uint32_t* texels; uint32_t ntexels;
    const float* materials;    /* 7 floats each: baseFactor, roughness, metallic, specular, emission */
    float sunDir[3], sunIrr[3], sky[3];
} rno_pt_scene;
typedef struct {
    uint64_t seed;
    uint32_t spp, sppBegin, maxBounces;
    int32_t width, height;
    float camera[10], previous[10];
    int32_t jitter, rr;
    uint32_t controls;         /* bit 0 dropLambertCosine, 1 misWeightOne, 2 aovDropSpecularIndirect,
                                  3 aovEmissionToDiffuse, 4 legacyLobeV2 */
} rno_pt_desc;
typedef struct {
    float *radiance, *albedo, *normal, *depth, *variance;
    int32_t* triangle;
    float* motion;
    float *diffuse, *specular, *emission, *diffuseAlbedo, *specularAlbedo, *diffuseVariance, *specularVariance;
} rno_pt_out;

typedef struct { v3 eye, f, s, u; float th, aspect; } pt_cam;
typedef struct {
    const rno_pt_scene* s;
    const rno_pt_desc* d;
    tri_t* tris;               /* trianglesOf(geo), input order */
    sah_t bvh;
    uint32_t* emitters; float* cdf; uint32_t nemit; float area;
    const float* table;
    pt_cam cam, prev;
    const rno_pt_out* out;
} pt_ctx;
typedef struct { v3 p, n, ng, base; const float* m; float t; int tri; int back; } pt_surf;

/* raw/math/primitives.hpp:31-64 with u and v. */
static int pt_intersect_uv(v3 ro, v3 rd, const tri_t* tri, float* tout, float* uout, float* vout) {
    const float ax = fabsf(rd.x), ay = fabsf(rd.y), az = fabsf(rd.z);
    const int kz = ax > ay ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    v3 d = wframe(rd, kz, 0);
    const int sw = d.z < 0.0f;
    if (sw) d = v3m(d.y, d.x, d.z);
    const float sx = d.x / d.z, sy = d.y / d.z, sz = 1.0f / d.z;
    const v3 A = wframe(sub3(tri->a, ro), kz, sw), B = wframe(sub3(tri->b, ro), kz, sw), C = wframe(sub3(tri->c, ro), kz, sw);
    const float Ax = A.x - sx * A.z, Ay = A.y - sy * A.z;
    const float Bx = B.x - sx * B.z, By = B.y - sy * B.z;
    const float Cx = C.x - sx * C.z, Cy = C.y - sy * C.z;
    const float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return 0;
    const float det = U + V + W;
    if (det == 0.0f) return 0;
    const v3 e1 = sub3(tri->b, tri->a), e2 = sub3(tri->c, tri->a), p = cross3(rd, e2);
    const float dm = dot3(e1, p);
    if (dm > -1e-7f && dm < 1e-7f) {
        const float T = U * (sz * A.z) + V * (sz * B.z) + W * (sz * C.z), inv = 1.0f / det;
        *tout = T * inv; *uout = V * inv; *vout = W * inv;
        return *tout > 1e-4f;
    }
    const float inv = 1.0f / dm;
    const v3 tv = sub3(ro, tri->a), q = cross3(tv, e1);
    float u = smax(0.0f, dot3(tv, p) * inv), v = smax(0.0f, dot3(rd, q) * inv);
    *tout = dot3(e2, q) * inv;
    const float s = u + v;
    if (s > 1.0f) { u /= s; v /= s; }
    *uout = u; *vout = v;
    return *tout > 1e-4f;
}
/* The nearest hit below tMax, ties to the lowest triangle index (rt_bvh.cpp:125-152). */
static int pt_closest(const pt_ctx* c, v3 o, v3 d, float tMax, float* tb, float* ub, float* vb, int* tri) {
    const sah_t* s = &c->bvh;
    if (!s->nnodes || !s->ntri) return 0;
    const v3 inv = v3m(finv(d.x), finv(d.y), finv(d.z));
    int stack[128], sp = 0, any = 0;
    float best = tMax;
    stack[sp++] = 0;
    while (sp) {
        const bnode_t* n = &s->nodes[stack[--sp]];
        if (!sah_entry(&n->box, o, inv, best)) continue;
        if (n->count) {
            for (int i = n->first; i < n->first + n->count; ++i) {
                float t, u, v;
                const int id = s->order[i];
                if (pt_intersect_uv(o, d, &s->tris[i], &t, &u, &v) && (t < best || (any && t == best && id < *tri))) {
                    best = t; *tb = t; *ub = u; *vb = v; *tri = id; any = 1;
                }
            }
        } else {
            if (sp > 125) abort();
            stack[sp++] = n->right; stack[sp++] = n->first;
        }
    }
    return any;
}
/* rt_pt_ctx.hpp:20-44: the surface at the closest hit. */
static int pt_hit(const pt_ctx* c, v3 o, v3 d, float tMax, pt_surf* x) {
    float t, u, v;
    int tri = -1;
    if (!pt_closest(c, o, d, tMax, &t, &u, &v, &tri)) return 0;
    const rno_pt_scene* s = c->s;
    const uint32_t i0 = s->idx[(size_t)tri * 3], i1 = s->idx[(size_t)tri * 3 + 1], i2 = s->idx[(size_t)tri * 3 + 2];
    const float b0 = 1.0f - u - v;
    x->t = t; x->tri = tri;
    x->p = add3(o, mul3(d, t));
    const tri_t* T = &c->tris[tri];
    x->ng = norm3(cross3(sub3(T->b, T->a), sub3(T->c, T->a)));
    const v3 n0 = v3m(s->nrm[3 * i0], s->nrm[3 * i0 + 1], s->nrm[3 * i0 + 2]);
    const v3 n1 = v3m(s->nrm[3 * i1], s->nrm[3 * i1 + 1], s->nrm[3 * i1 + 2]);
    const v3 n2 = v3m(s->nrm[3 * i2], s->nrm[3 * i2 + 1], s->nrm[3 * i2 + 2]);
    x->n = norm3(add3(add3(mul3(n0, b0), mul3(n1, u)), mul3(n2, v)));
    const float tu = s->uv[2 * i0] * b0 + s->uv[2 * i1] * u + s->uv[2 * i2] * v;
    const float tv = s->uv[2 * i0 + 1] * b0 + s->uv[2 * i1 + 1] * u + s->uv[2 * i2 + 1] * v;
    const uint32_t tex = s->triTex[tri];
    const uint32_t off = s->texEntries[3 * tex], tw = s->texEntries[3 * tex + 1], th = s->texEntries[3 * tex + 2];
    const uint32_t tx = (uint32_t)(int32_t)floorf(tu * (float)tw) & (tw - 1);
    const uint32_t ty = (uint32_t)(int32_t)floorf(tv * (float)th) & (th - 1);
    const uint32_t col = s->texels[off + ty * tw + tx];
    x->m = s->materials + 7 * (size_t)tex;
    const float k = x->m[0] / 255.0f;
    x->base = v3m((float)(col & 255u) * k, (float)((col >> 8) & 255u) * k, (float)((col >> 16) & 255u) * k);
    x->back = dot3(x->ng, d) > 0.0f;
    if (dot3(x->ng, d) > 0.0f) x->ng = mul3(x->ng, -1.0f);
    if (dot3(x->n, x->ng) < 0.0f) x->n = mul3(x->n, -1.0f);
    return 1;
}
static int pt_visible(const pt_ctx* c, v3 p, v3 dir, float tMax) { return !sah_occluded(&c->bvh, p, dir, tMax); }
static v3 pt_offset(const pt_surf* x, v3 dir) {
    const float e = 2e-4f * (1.0f + smax(fabsf(x->p.x), smax(fabsf(x->p.y), fabsf(x->p.z))));
    return add3(x->p, mul3(x->ng, dot3(x->ng, dir) > 0.0f ? e : -e));
}
/* rt_pt_ctx.hpp:48-79: the sun and one emitter sample, MIS-weighted; *diff the Lambert share. */
static v3 pt_nee(const pt_ctx* c, const pt_surf* x, const pt_frame* fr, const pt_bsdf* bs, v3 woL, uint32_t px,
                 uint32_t smp, uint32_t base, v3* diff) {
    const rno_pt_scene* s = c->s;
    const rno_pt_desc* d = c->d;
    v3 L = v3m(0, 0, 0);
    *diff = v3m(0, 0, 0);
    const int dc = (d->controls & 1u) != 0;
    const v3 irr = v3m(s->sunIrr[0], s->sunIrr[1], s->sunIrr[2]);
    if (pt_maxc(irr) > 0.0f) {
        const v3 l = norm3(v3m(s->sunDir[0], s->sunDir[1], s->sunDir[2])), lL = pt_to_local(fr, l);
        const pt_eval e = pt_eval_bsdf(bs, woL, lL, dc);
        if (pt_maxc(e.fcos) > 0.0f && pt_visible(c, pt_offset(x, l), l, 1e30f)) {
            L = add3(L, pt_mulv(e.fcos, irr));
            *diff = add3(*diff, pt_mulv(pt_lambert_cos(bs, woL, lL, dc), irr));
        }
    }
    if (!c->nemit) return L;
    const pt_r2 a = pt_rand2(d->seed, px, smp, base + 2), b = pt_rand2(d->seed, px, smp, base + 3);
    const float target = a.a * c->area;
    uint32_t lo = 0, hi = c->nemit;              /* std::upper_bound: the first cdf > target */
    while (lo < hi) { const uint32_t mid = lo + (hi - lo) / 2; if (target < c->cdf[mid]) hi = mid; else lo = mid + 1; }
    const uint32_t k = lo < c->nemit - 1 ? lo : c->nemit - 1;
    const tri_t* t = &c->tris[c->emitters[k]];
    const float su = sqrtf(a.b);
    const v3 q = add3(add3(mul3(t->a, 1.0f - su), mul3(t->b, su * (1.0f - b.a))), mul3(t->c, su * b.a));
    const v3 to = sub3(q, x->p);
    const float dist = len3(to);
    const v3 l = mul3(to, 1.0f / dist), lL = pt_to_local(fr, l);
    const float cosL = fabsf(dot3(norm3(cross3(sub3(t->b, t->a), sub3(t->c, t->a))), l));
    if (cosL <= 0.0f) return L;
    const float pl = dist * dist / (cosL * c->area);
    const pt_eval e = pt_eval_bsdf(bs, woL, lL, dc);
    if (pt_maxc(e.fcos) <= 0.0f || !pt_visible(c, pt_offset(x, l), l, dist * (1.0f - 1e-3f))) return L;
    const float w = (d->controls & 2u) ? 1.0f : pl * pl / (pl * pl + e.pdf * e.pdf);
    const float* em = s->materials + 7 * (size_t)s->triTex[c->emitters[k]] + 4;
    const v3 Le = v3m(em[0], em[1], em[2]);
    *diff = add3(*diff, mul3(pt_mulv(pt_lambert_cos(bs, woL, lL, dc), Le), w / pl));
    return add3(L, mul3(pt_mulv(e.fcos, Le), w / pl));
}

typedef struct { v3 L, D, S, E, alb, nrm, dAlb, sAlb; } pt_sample;
/* rt_pt_cpu.cpp:31-97: one sample of a camera ray. */
static pt_sample pt_trace_path(const pt_ctx* c, v3 ro, v3 rd, uint32_t px, uint32_t smp) {
    const rno_pt_scene* s = c->s;
    const rno_pt_desc* d = c->d;
    pt_sample o;
    memset(&o, 0, sizeof o);
    v3 T = v3m(1, 1, 1), tw = v3m(1, 1, 1), R = v3m(0, 0, 0), wd = v3m(0, 0, 0), ws = v3m(0, 0, 0);
    const v3 sky = v3m(s->sky[0], s->sky[1], s->sky[2]);
    float prevPdf = 0.0f;
    const int dc = (d->controls & 1u) != 0;
    for (uint32_t b = 0; b <= d->maxBounces; ++b) {
        pt_surf x0;
        if (!pt_hit(c, ro, rd, 1e30f, &x0)) {
            o.L = add3(o.L, pt_mulv(T, sky));
            if (b == 0) o.E = sky; else R = add3(R, pt_mulv(tw, sky));
            break;
        }
        const pt_bsdf bs = {x0.base, x0.m[1], x0.m[2], x0.m[3], (d->controls & 16u) != 0, c->table};
        if (b == 0) {
            o.alb = x0.base; o.nrm = x0.n;
            o.dAlb = mul3(x0.base, 1.0f - x0.m[2]);
            o.sAlb = pt_spec_albedo(&bs, pt_clampf(-dot3(x0.n, rd), 0.0f, 1.0f));
        }
        const v3 Le = v3m(x0.m[4], x0.m[5], x0.m[6]);
        if (pt_maxc(Le) > 0.0f) {
            float w = 1.0f;
            if (b > 0 && !(d->controls & 2u)) {
                const float cosL = fabsf(dot3(x0.ng, rd)), pl = x0.t * x0.t / (cosL * c->area);
                w = prevPdf * prevPdf / (prevPdf * prevPdf + pl * pl);
            }
            o.L = add3(o.L, mul3(pt_mulv(T, Le), w));
            if (b == 0) o.E = Le; else R = add3(R, mul3(pt_mulv(tw, Le), w));
        }
        if (b == d->maxBounces) break;
        const pt_frame fr = pt_basis(x0.n);
        const v3 woL = pt_to_local(&fr, mul3(rd, -1.0f));
        if (woL.z <= 0.0f) break;
        const uint32_t base = 2 + b * 4;
        v3 nd;
        const v3 Ln = pt_nee(c, &x0, &fr, &bs, woL, px, smp, base, &nd);
        o.L = add3(o.L, pt_mulv(T, Ln));
        if (b == 0) { o.D = nd; o.S = sub3(Ln, nd); } else R = add3(R, pt_mulv(tw, Ln));
        const pt_r2 u = pt_rand2(d->seed, px, smp, base), r = pt_rand2(d->seed, px, smp, base + 1);
        v3 wiL;
        if (!pt_sample_bsdf(&bs, woL, r.a, u.a, u.b, &wiL)) break;
        const pt_eval e = pt_eval_bsdf(&bs, woL, wiL, dc);
        if (e.pdf <= 0.0f) break;
        const v3 step = mul3(e.fcos, 1.0f / e.pdf);
        T = pt_mulv(T, step);
        if (b == 0) { wd = mul3(pt_lambert_cos(&bs, woL, wiL, dc), 1.0f / e.pdf); ws = sub3(step, wd); }
        else tw = pt_mulv(tw, step);
        prevPdf = e.pdf;
        if (d->rr && b >= 3) {
            const float q = smin(0.95f, pt_maxc(T));
            if (r.b >= q) break;
            T = mul3(T, 1.0f / q);
            tw = mul3(tw, 1.0f / q);
        }
        const v3 wi = pt_to_world(&fr, wiL);
        ro = pt_offset(&x0, wi);
        rd = wi;
    }
    o.D = add3(o.D, pt_mulv(wd, R));
    if (!(d->controls & 4u)) o.S = add3(o.S, pt_mulv(ws, R));
    if (d->controls & 8u) { o.D = add3(o.D, o.E); o.E = v3m(0, 0, 0); }
    return o;
}

static pt_cam pt_cam_of(const float* c, int w, int h) {
    pt_cam k;
    k.eye = v3m(c[0], c[1], c[2]);
    k.f = norm3(sub3(v3m(c[3], c[4], c[5]), k.eye));
    k.s = norm3(cross3(k.f, v3m(c[6], c[7], c[8])));
    k.u = cross3(k.s, k.f);
    k.th = tanf(c[9] * 0.5f);
    k.aspect = (float)w / (float)h;
    return k;
}
static v3 pt_dir_of(const pt_cam* c, float px, float py, int w, int h) {
    const float nx = px / (float)w * 2.0f - 1.0f, ny = 1.0f - py / (float)h * 2.0f;
    return norm3(add3(add3(c->f, mul3(c->s, nx * c->th * c->aspect)), mul3(c->u, ny * c->th)));
}
static void pt_put3(float* v, size_t p, v3 a) { if (v) { v[p * 3] = a.x; v[p * 3 + 1] = a.y; v[p * 3 + 2] = a.z; } }
static float pt_var(double s1, double s2, uint32_t n) {
    return n > 1 ? (float)((s2 - s1 * s1 / n) / (n - 1) / n) : 0.0f;
}
/* rt_pt_cpu.cpp:99-150: one row of pixels. */
static void pt_row(void* p, int y) {
    const pt_ctx* c = (const pt_ctx*)p;
    const rno_pt_desc* d = c->d;
    const rno_pt_out* O = c->out;
    const int W = d->width, H = d->height;
    for (int x = 0; x < W; ++x) {
        const uint32_t px = (uint32_t)(y * W + x);
        v3 sum = v3m(0, 0, 0), alb = sum, nrm = sum, sd = sum, ss = sum, se = sum, sda = sum, ssa = sum;
        double l1 = 0, l2 = 0, d1 = 0, d2 = 0, q1 = 0, q2 = 0;
        for (uint32_t k = 0; k < d->spp; ++k) {
            const uint32_t smp = d->sppBegin + k;
            pt_r2 j = {0.5f, 0.5f};
            if (d->jitter) j = pt_rand2(d->seed, px, smp, 0);
            const v3 dir = pt_dir_of(&c->cam, (float)x + j.a, (float)y + j.b, W, H);
            const pt_sample o = pt_trace_path(c, c->cam.eye, dir, px, smp);
            sum = add3(sum, o.L); alb = add3(alb, o.alb); nrm = add3(nrm, o.nrm);
            sd = add3(sd, o.D); ss = add3(ss, o.S); se = add3(se, o.E); sda = add3(sda, o.dAlb); ssa = add3(ssa, o.sAlb);
            double l = (double)pt_lum(o.L); l1 += l; l2 += l * l;
            l = (double)pt_lum(o.D); d1 += l; d2 += l * l;
            l = (double)pt_lum(o.S); q1 += l; q2 += l * l;
        }
        const float inv = d->spp ? 1.0f / (float)d->spp : 0.0f;
        const size_t q = (size_t)px;
        pt_put3(O->radiance, q, mul3(sum, inv)); pt_put3(O->albedo, q, mul3(alb, inv)); pt_put3(O->normal, q, mul3(nrm, inv));
        pt_put3(O->diffuse, q, mul3(sd, inv)); pt_put3(O->specular, q, mul3(ss, inv)); pt_put3(O->emission, q, mul3(se, inv));
        pt_put3(O->diffuseAlbedo, q, mul3(sda, inv)); pt_put3(O->specularAlbedo, q, mul3(ssa, inv));
        if (O->variance) O->variance[q] = pt_var(l1, l2, d->spp);
        if (O->diffuseVariance) O->diffuseVariance[q] = pt_var(d1, d2, d->spp);
        if (O->specularVariance) O->specularVariance[q] = pt_var(q1, q2, d->spp);
        /* the pixel-centre ray's depth, triangle and motion (rt_pt_cpu.cpp:111-122) */
        float depth = 0.0f, mx = 0.0f, my = 0.0f;
        int32_t tri = -1;
        pt_surf cs;
        if (pt_hit(c, c->cam.eye, pt_dir_of(&c->cam, (float)x + 0.5f, (float)y + 0.5f, W, H), 1e30f, &cs)) {
            depth = dot3(sub3(cs.p, c->cam.eye), c->cam.f);
            tri = cs.tri;
            const v3 v = sub3(cs.p, c->prev.eye);
            const float z = dot3(v, c->prev.f);
            const float nx = dot3(v, c->prev.s) / (z * c->prev.th * c->prev.aspect), ny = dot3(v, c->prev.u) / (z * c->prev.th);
            mx = (nx * 0.5f + 0.5f) * (float)W - ((float)x + 0.5f);
            my = (1.0f - (ny * 0.5f + 0.5f)) * (float)H - ((float)y + 0.5f);
        }
        if (O->depth) O->depth[q] = depth;
        if (O->triangle) O->triangle[q] = tri;
        if (O->motion) { O->motion[q * 2] = mx; O->motion[q * 2 + 1] = my; }
    }
}

/* finishPtScene's emitter list and CDF (rt_pt_scene.cpp:31-45) for a scene's triangles:
 * returns the count; cdf gets the inclusive running area (float, in index order). */
static uint32_t pt_emitters(const rno_pt_scene* s, const tri_t* tris, uint32_t* list, float* cdf, float* area) {
    uint32_t n = 0;
    *area = 0.0f;
    for (uint32_t t = 0; t < s->ntri; ++t) {
        const float* e = s->materials + 7 * (size_t)s->triTex[t] + 4;
        if (e[0] <= 0.0f && e[1] <= 0.0f && e[2] <= 0.0f) continue;
        *area += 0.5f * len3(cross3(sub3(tris[t].b, tris[t].a), sub3(tris[t].c, tris[t].a)));
        list[n] = t; cdf[n] = *area; ++n;
    }
    return n;
}

/* raw::rt::pathTraceCpu (rt_pt_cpu.cpp:126-150) for a v2 scene, with the energy table `table`
 * (rno_pt_energy_table's floats; NULL builds it). Returns the emitter count. */
RNO_API int rno_pathtrace(const rno_pt_scene* s, const rno_pt_desc* d, const float* table, int threads,
                          const rno_pt_out* out) {
    pt_ctx c;
    memset(&c, 0, sizeof c);
    c.s = s; c.d = d; c.out = out;
    float* own = NULL;
    if (!table) { own = (float*)malloc(PT_FLOATS * sizeof(float)); rno_pt_energy_table(own, threads); table = own; }
    c.table = table;
    c.tris = (tri_t*)malloc((size_t)(s->ntri ? s->ntri : 1) * sizeof(tri_t));
    for (uint32_t t = 0; t < s->ntri; ++t) {
        const uint32_t* i = s->idx + (size_t)t * 3;
        c.tris[t].a = v3m(s->pos[3 * i[0]], s->pos[3 * i[0] + 1], s->pos[3 * i[0] + 2]);
        c.tris[t].b = v3m(s->pos[3 * i[1]], s->pos[3 * i[1] + 1], s->pos[3 * i[1] + 2]);
        c.tris[t].c = v3m(s->pos[3 * i[2]], s->pos[3 * i[2] + 1], s->pos[3 * i[2] + 2]);
    }
    sah_build(&c.bvh, c.tris, (int)s->ntri);
    c.emitters = (uint32_t*)malloc((size_t)(s->ntri ? s->ntri : 1) * sizeof(uint32_t));
    c.cdf = (float*)malloc((size_t)(s->ntri ? s->ntri : 1) * sizeof(float));
    c.nemit = pt_emitters(s, c.tris, c.emitters, c.cdf, &c.area);
    c.cam = pt_cam_of(d->camera, d->width, d->height);
    c.prev = pt_cam_of(d->previous, d->width, d->height);
    parallel_rows(d->height, threads, pt_row, &c);
    const int n = (int)c.nemit;
    sah_free(&c.bvh);
    free(c.tris); free(c.emitters); free(c.cdf); free(own);
    return n;
}
