/*
 * rn_oracle.c -- CPU restatement of raw-native's ambient-occlusion path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle the CUDA path is compared against:
 * only the tests, the smoke check and the CPU-baseline leg of the benchmark load
 * it. No product code links it, calls it or falls back to it.
 *
 * Every function restates the reference's algorithm in plain C, in the same float32
 * operation order, and cites the file:line it follows (paths inside the raw-native tree).
 * Build with -ffp-contract=off: the reference's goldens were made on x86-64 without
 * fused multiply-add, and contraction changes float results.
 *
 * Parity pin: oracle/Makefile compiles the reference's own sources into oracle/_ref and
 * tests/test_oracle_pin.py checks this file against it and against the reference's
 * committed SHA-256 goldens (evidence/identity-golden.json).
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define RNO_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------ vector math
 * raw/math/vec.hpp:9-16. Each operator is one rounding; sums go left to right. */
typedef struct { float x, y, z; } v3;
static inline v3 v3m(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 add3(v3 a, v3 b) { return v3m(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub3(v3 a, v3 b) { return v3m(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul3(v3 a, float s) { return v3m(a.x * s, a.y * s, a.z * s); }
static inline float dot3(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross3(v3 a, v3 b) {
    return v3m(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline float len3(v3 v) { return sqrtf(dot3(v, v)); }
static inline v3 norm3(v3 v) { float l = len3(v); return l > 0 ? mul3(v, 1.0f / l) : v; }
/* std::min / std::max on floats: (b < a) ? b : a and (a < b) ? b : a (NaN keeps a). */
static inline float smin(float a, float b) { return (b < a) ? b : a; }
static inline float smax(float a, float b) { return (a < b) ? b : a; }
static inline float v3k(v3 v, int k) { return k == 0 ? v.x : k == 1 ? v.y : v.z; }

typedef struct { v3 a, b, c; } tri_t;

/* ------------------------------------------------------------------ sampler
 * src/renderer/ray_ao.cpp:8-12 (same function at src/renderer/ssao.cpp:6-10). */
static inline float hash01(uint32_t x, uint32_t y, uint32_t s) {
    uint32_t h = x * 374761393u + y * 668265263u + s * 2246822519u;
    h = (h ^ (h >> 13)) * 1274126177u;
    h ^= h >> 16;
    return (float)(h & 0xFFFFFFu) / 16777216.0f;
}
RNO_API float rno_hash01(uint32_t x, uint32_t y, uint32_t s) { return hash01(x, y, s); }

/* ------------------------------------------------------------------ triangle test
 * raw/math/primitives.hpp:17-20 (frame) and :31-64 (watertight sign test, then
 * Moeller-Trumbore t unless its determinant is within 1e-7 of zero). */
static inline v3 wframe(v3 v, int kz, int sw) {
    v3 p = kz == 0 ? v3m(v.y, v.z, v.x) : kz == 1 ? v3m(v.z, v.x, v.y) : v;
    return sw ? v3m(p.y, p.x, p.z) : p;
}
static int intersect_tri(v3 ro, v3 rd, const tri_t* tri, float* tout) {
    const float ax = fabsf(rd.x), ay = fabsf(rd.y), az = fabsf(rd.z);
    const int kz = ax > ay ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    v3 d = wframe(rd, kz, 0);
    const int sw = d.z < 0.0f;
    if (sw) d = v3m(d.y, d.x, d.z);
    const float sx = d.x / d.z, sy = d.y / d.z, sz = 1.0f / d.z;
    const v3 A = wframe(sub3(tri->a, ro), kz, sw), B = wframe(sub3(tri->b, ro), kz, sw),
             C = wframe(sub3(tri->c, ro), kz, sw);
    const float Ax = A.x - sx * A.z, Ay = A.y - sy * A.z;
    const float Bx = B.x - sx * B.z, By = B.y - sy * B.z;
    const float Cx = C.x - sx * C.z, Cy = C.y - sy * C.z;
    const float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return 0;
    const float det = U + V + W;
    if (det == 0.0f) return 0;
    const v3 e1 = sub3(tri->b, tri->a), e2 = sub3(tri->c, tri->a), p = cross3(rd, e2);
    const float dm = dot3(e1, p);
    float t;
    if (dm > -1e-7f && dm < 1e-7f) {
        const float T = U * (sz * A.z) + V * (sz * B.z) + W * (sz * C.z), inv = 1.0f / det;
        t = T * inv;
    } else {
        const float inv = 1.0f / dm;
        const v3 tv = sub3(ro, tri->a), q = cross3(tv, e1);
        t = dot3(e2, q) * inv;
    }
    *tout = t;
    return t > 1e-4f;
}
RNO_API int rno_intersect(const float* ray6, const float* tri9, float* t) {
    return intersect_tri(v3m(ray6[0], ray6[1], ray6[2]), v3m(ray6[3], ray6[4], ray6[5]),
                         (const tri_t*)tri9, t);
}

/* ------------------------------------------------------------------ binned-SAH BVH
 * src/renderer/bvh.cpp:35-138: 12 bins, leaves of up to 4 triangles, stable partition,
 * iterative any-hit walk whose slab exit is widened by 1.0000008. */
typedef struct { v3 mn, mx; } aabb_t;
typedef struct { aabb_t box; int first, count, right; } bnode_t;
typedef struct {
    tri_t* tris; int ntri;
    bnode_t* nodes; int nnodes, cap;
    int* order;
    v3* centres;
} sah_t;
static inline aabb_t box_empty(void) { aabb_t b = {{1e30f, 1e30f, 1e30f}, {-1e30f, -1e30f, -1e30f}}; return b; }
static inline void box_grow(aabb_t* b, v3 p) {
    b->mn = v3m(smin(b->mn.x, p.x), smin(b->mn.y, p.y), smin(b->mn.z, p.z));
    b->mx = v3m(smax(b->mx.x, p.x), smax(b->mx.y, p.y), smax(b->mx.z, p.z));
}
static inline float sah_area(const aabb_t* b) {
    const v3 d = sub3(b->mx, b->mn);
    return d.x < 0 ? 0.0f : 2.0f * (d.x * d.y + d.y * d.z + d.z * d.x);
}
static inline aabb_t box_unite(aabb_t a, const aabb_t* b) { box_grow(&a, b->mn); box_grow(&a, b->mx); return a; }
static int sah_push(sah_t* s, int first, int count) {
    if (s->nnodes == s->cap) {
        s->cap = s->cap ? 2 * s->cap : 64;
        s->nodes = (bnode_t*)realloc(s->nodes, (size_t)s->cap * sizeof(bnode_t));
    }
    bnode_t n; memset(&n, 0, sizeof n); n.box = box_empty(); n.first = first; n.count = count;
    s->nodes[s->nnodes] = n;
    return s->nnodes++;
}
static inline int sah_bin(float c, float lo, float ext) {
    int b = (int)((c - lo) / ext * 12.0f);
    return b < 11 ? b : 11;
}
static void sah_split(sah_t* s, int ni) {
    aabb_t box = box_empty(), cb = box_empty();
    const int first = s->nodes[ni].first, count = s->nodes[ni].count;
    for (int i = first; i < first + count; ++i) {
        const tri_t* t = &s->tris[s->order[i]];
        box_grow(&box, t->a); box_grow(&box, t->b); box_grow(&box, t->c);
        box_grow(&cb, s->centres[s->order[i]]);
    }
    s->nodes[ni].box = box;
    if (count <= 4) return;
    int bestAxis = -1, bestBin = 0;
    float bestCost = sah_area(&box) * (float)count;
    for (int k = 0; k < 3; ++k) {
        const float lo = v3k(cb.mn, k), ext = v3k(cb.mx, k) - lo;
        if (ext <= 0.0f) continue;
        aabb_t bb[12]; int cnt[12];
        for (int b = 0; b < 12; ++b) { bb[b] = box_empty(); cnt[b] = 0; }
        for (int i = first; i < first + count; ++i) {
            const int o = s->order[i], b = sah_bin(v3k(s->centres[o], k), lo, ext);
            const tri_t* t = &s->tris[o];
            box_grow(&bb[b], t->a); box_grow(&bb[b], t->b); box_grow(&bb[b], t->c); ++cnt[b];
        }
        for (int sp = 1; sp < 12; ++sp) {
            aabb_t l = box_empty(), r = box_empty(); int cl = 0, cr = 0;
            for (int b = 0; b < sp; ++b) if (cnt[b]) { l = box_unite(l, &bb[b]); cl += cnt[b]; }
            for (int b = sp; b < 12; ++b) if (cnt[b]) { r = box_unite(r, &bb[b]); cr += cnt[b]; }
            if (!cl || !cr) continue;
            const float cost = sah_area(&l) * (float)cl + sah_area(&r) * (float)cr;
            if (cost < bestCost) { bestCost = cost; bestAxis = k; bestBin = sp; }
        }
    }
    if (bestAxis < 0) return;
    const float lo = v3k(cb.mn, bestAxis), ext = v3k(cb.mx, bestAxis) - lo;
    /* std::stable_partition: the 'true' elements first, both groups in their old order */
    int* tmp = (int*)malloc((size_t)count * sizeof(int));
    int nl = 0;
    for (int i = first; i < first + count; ++i)
        if (sah_bin(v3k(s->centres[s->order[i]], bestAxis), lo, ext) < bestBin) tmp[nl++] = s->order[i];
    int nr = nl;
    for (int i = first; i < first + count; ++i)
        if (!(sah_bin(v3k(s->centres[s->order[i]], bestAxis), lo, ext) < bestBin)) tmp[nr++] = s->order[i];
    memcpy(s->order + first, tmp, (size_t)count * sizeof(int));
    free(tmp);
    const int left = sah_push(s, first, nl);
    sah_push(s, first + nl, count - nl);
    s->nodes[ni].count = 0;
    s->nodes[ni].first = left;
    s->nodes[ni].right = left + 1;
    sah_split(s, left);
    sah_split(s, left + 1);
}
static void sah_build(sah_t* s, const tri_t* tris, int n) {
    memset(s, 0, sizeof *s);
    s->ntri = n;
    s->tris = (tri_t*)malloc((size_t)(n ? n : 1) * sizeof(tri_t));
    memcpy(s->tris, tris, (size_t)n * sizeof(tri_t));
    s->order = (int*)malloc((size_t)(n ? n : 1) * sizeof(int));
    s->centres = (v3*)malloc((size_t)(n ? n : 1) * sizeof(v3));
    for (int i = 0; i < n; ++i) {
        s->order[i] = i;
        s->centres[i] = mul3(add3(add3(tris[i].a, tris[i].b), tris[i].c), 1.0f / 3.0f);
    }
    sah_push(s, 0, n);
    if (n) sah_split(s, 0);
    tri_t* sorted = (tri_t*)malloc((size_t)(n ? n : 1) * sizeof(tri_t));
    for (int i = 0; i < n; ++i) sorted[i] = s->tris[s->order[i]];
    free(s->tris);
    s->tris = sorted;
}
static void sah_free(sah_t* s) { free(s->tris); free(s->nodes); free(s->order); free(s->centres); }
static inline float finv(float x) { return x != 0.0f ? 1.0f / x : copysignf(INFINITY, x); }
/* bvh.cpp:21-28 */
static inline int sah_entry(const aabb_t* b, v3 o, v3 inv, float tMax) {
    float t0 = 0.0f, t1 = tMax;
    for (int k = 0; k < 3; ++k) {
        const float i = v3k(inv, k), a = (v3k(b->mn, k) - v3k(o, k)) * i, c = (v3k(b->mx, k) - v3k(o, k)) * i;
        t0 = smax(t0, smin(a, c)); t1 = smin(t1, smax(a, c));
    }
    return t0 <= t1 * 1.0000008f;
}
/* bvh.cpp:119-138 */
static int sah_occluded(const sah_t* s, v3 o, v3 d, float tMax) {
    if (!s->nnodes || !s->ntri) return 0;
    const v3 inv = v3m(finv(d.x), finv(d.y), finv(d.z));
    int stack[128], sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const bnode_t* n = &s->nodes[stack[--sp]];
        if (!sah_entry(&n->box, o, inv, tMax)) continue;
        if (n->count) {
            for (int i = n->first; i < n->first + n->count; ++i) {
                float t;
                if (intersect_tri(o, d, &s->tris[i], &t) && t < tMax) return 1;
            }
        } else {
            if (sp > 125) abort();
            stack[sp++] = n->right; stack[sp++] = n->first;
        }
    }
    return 0;
}
/* src/renderer/accel.cpp:31-35: the scan of every triangle, the reference's test oracle. */
static int scan_occluded(const tri_t* tris, int n, v3 o, v3 d, float tMax) {
    for (int i = 0; i < n; ++i) {
        float t;
        if (intersect_tri(o, d, &tris[i], &t) && t < tMax) return 1;
    }
    return 0;
}

/* An occlusion accelerator handle for the Python side: the SAH BVH over a triangle list. */
RNO_API void* rno_accel_build(const float* tris9, int ntri) {
    sah_t* s = (sah_t*)malloc(sizeof(sah_t));
    sah_build(s, (const tri_t*)tris9, ntri);
    return s;
}
RNO_API void rno_accel_free(void* h) { if (h) { sah_free((sah_t*)h); free(h); } }
RNO_API int rno_accel_nodes(void* h) { return ((sah_t*)h)->nnodes; }
RNO_API int rno_occluded(void* h, const float* ray6, float tMax) {
    return sah_occluded((const sah_t*)h, v3m(ray6[0], ray6[1], ray6[2]), v3m(ray6[3], ray6[4], ray6[5]), tMax);
}
RNO_API int rno_occluded_scan(const float* tris9, int ntri, const float* ray6, float tMax) {
    return scan_occluded((const tri_t*)tris9, ntri, v3m(ray6[0], ray6[1], ray6[2]), v3m(ray6[3], ray6[4], ray6[5]), tMax);
}

/* ------------------------------------------------------------------ row-parallel loop
 * raw/core/parallel.hpp:13-31: thread t takes rows t, t+T, ...; output is identical for
 * any thread count because each row is written by one thread from read-only inputs. */
typedef void (*row_fn)(void* ctx, int y);
typedef struct { row_fn fn; void* ctx; int rows, threads, t; } row_job;
static void* row_worker(void* p) {
    row_job* j = (row_job*)p;
    for (int y = j->t; y < j->rows; y += j->threads) j->fn(j->ctx, y);
    return NULL;
}
static void parallel_rows(int rows, int threads, row_fn fn, void* ctx) {
    if (threads > 1 && rows > 1) {
        if (threads > rows) threads = rows;
        pthread_t* th = (pthread_t*)malloc((size_t)threads * sizeof(pthread_t));
        row_job* jobs = (row_job*)malloc((size_t)threads * sizeof(row_job));
        for (int t = 0; t < threads; ++t) {
            jobs[t].fn = fn; jobs[t].ctx = ctx; jobs[t].rows = rows; jobs[t].threads = threads; jobs[t].t = t;
            pthread_create(&th[t], NULL, row_worker, &jobs[t]);
        }
        for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
        free(th); free(jobs);
        return;
    }
    for (int y = 0; y < rows; ++y) fn(ctx, y);
}

/* ------------------------------------------------------------------ ray-traced AO
 * src/renderer/ray_ao.cpp:14-17 (basis) and :20-51 (trace). `row_stride`/`row0` let the
 * benchmark's CPU leg trace a strided subset of rows; both default to every row. */
typedef struct {
    int w, h;
    const float* pos; const float* nrm; const uint8_t* mask;
    const sah_t* bvh; const tri_t* tris; int ntri; int scan;
    int samples; float radius; v3 toLight; int sky, sunForced;
    float* ao; float* skyo; float* sun;
    int row0, row_stride;
} trace_ctx;
static inline int occl(const trace_ctx* c, v3 o, v3 d, float tMax) {
    return c->scan ? scan_occluded(c->tris, c->ntri, o, d, tMax) : sah_occluded(c->bvh, o, d, tMax);
}
static void trace_row(void* p, int yi) {
    const trace_ctx* c = (const trace_ctx*)p;
    const int y = c->row0 + yi * c->row_stride;
    if (y >= c->h) return;
    const float kFar = 1e30f;
    for (int x = 0; x < c->w; ++x) {
        const size_t i = (size_t)y * c->w + x;
        if (!c->mask[i]) {
            c->ao[i] = 1.0f;
            if (c->sky) { c->skyo[i] = 1.0f; c->sun[i] = 1.0f; }
            continue;
        }
        const v3 P = v3m(c->pos[3 * i], c->pos[3 * i + 1], c->pos[3 * i + 2]);
        const v3 n = v3m(c->nrm[3 * i], c->nrm[3 * i + 1], c->nrm[3 * i + 2]);
        const v3 a = fabsf(n.x) > 0.9f ? v3m(0, 1, 0) : v3m(1, 0, 0);
        const v3 t = norm3(cross3(a, n)), b = cross3(n, t);
        const v3 origin = add3(P, mul3(n, 1e-3f));
        int open = 0, freec = 0;
        for (int s = 0; s < c->samples; ++s) {
            const float u1 = hash01((uint32_t)x, (uint32_t)y, (uint32_t)(2 * s));
            const float u2 = hash01((uint32_t)x, (uint32_t)y, (uint32_t)(2 * s + 1));
            const float r = sqrtf(u1), phi = 6.2831853f * u2;
            const float lx = r * cosf(phi), ly = r * sinf(phi);
            const float lz = sqrtf(smax(0.0f, 1.0f - u1));
            const v3 dir = norm3(add3(add3(mul3(t, lx), mul3(b, ly)), mul3(n, lz)));
            if (!occl(c, origin, dir, c->radius)) {
                ++open;
                if (c->sky && !occl(c, origin, dir, kFar)) ++freec;
            }
        }
        c->ao[i] = (float)open / (float)c->samples;
        if (c->sky) {
            c->skyo[i] = (float)freec / (float)c->samples;
            c->sun[i] = (c->sunForced || !occl(c, origin, c->toLight, kFar)) ? 1.0f : 0.0f;
        }
    }
}
/* computeRTAO (ray_ao.cpp:53-58) when sky == NULL, computeRTVisibility (:59-63) otherwise.
 * accel: a handle from rno_accel_build, or NULL to scan every triangle. */
RNO_API void rno_trace(int w, int h, const float* pos, const float* nrm, const uint8_t* mask,
                       void* accel, const float* tris9, int ntri, int samples, float radius,
                       const float* toLight3, int sunForced, float* ao, float* sky, float* sun,
                       int threads, int row0, int row_stride) {
    trace_ctx c;
    memset(&c, 0, sizeof c);
    c.w = w; c.h = h; c.pos = pos; c.nrm = nrm; c.mask = mask;
    c.bvh = (const sah_t*)accel; c.tris = (const tri_t*)tris9; c.ntri = ntri; c.scan = accel == NULL;
    c.samples = samples; c.radius = radius;
    c.toLight = toLight3 ? norm3(v3m(toLight3[0], toLight3[1], toLight3[2])) : v3m(0, 1, 0);
    c.sky = sky != NULL; c.sunForced = sunForced;
    c.ao = ao; c.skyo = sky; c.sun = sun;
    c.row0 = row0 < 0 ? 0 : row0; c.row_stride = row_stride < 1 ? 1 : row_stride;
    const int rows = (h - c.row0 + c.row_stride - 1) / c.row_stride;
    parallel_rows(rows, threads, trace_row, &c);
}

/* ------------------------------------------------------------------ screen-space AO
 * src/renderer/ssao.cpp:11-39. lround: half away from zero. */
typedef struct {
    int w, h; const float* pos; const float* nrm; const uint8_t* mask;
    int samples; float radius; float* ao;
} ssao_ctx;
static void ssao_row(void* p, int y) {
    const ssao_ctx* c = (const ssao_ctx*)p;
    const int R = 6;
    for (int x = 0; x < c->w; ++x) {
        const size_t i = (size_t)y * c->w + x;
        if (!c->mask[i]) { c->ao[i] = 1.0f; continue; }
        const v3 P = v3m(c->pos[3 * i], c->pos[3 * i + 1], c->pos[3 * i + 2]);
        const v3 n = v3m(c->nrm[3 * i], c->nrm[3 * i + 1], c->nrm[3 * i + 2]);
        int occ = 0, used = 0;
        for (int s = 0; s < c->samples; ++s) {
            const float a = hash01((uint32_t)x, (uint32_t)y, (uint32_t)s) * 6.2831853f;
            const float rad = (0.3f + 0.7f * hash01((uint32_t)x, (uint32_t)y, (uint32_t)(s + 97))) * (float)R;
            const int sx = x + (int)lroundf(cosf(a) * rad);
            const int sy = y + (int)lroundf(sinf(a) * rad);
            if (sx < 0 || sy < 0 || sx >= c->w || sy >= c->h) continue;
            const size_t j = (size_t)sy * c->w + sx;
            if (!c->mask[j]) continue;
            ++used;
            const v3 d = sub3(v3m(c->pos[3 * j], c->pos[3 * j + 1], c->pos[3 * j + 2]), P);
            const float dist = len3(d);
            if (dist < 1e-4f || dist > c->radius) continue;
            const float ndl = dot3(n, norm3(d));
            if (ndl > 0.15f) ++occ;
        }
        const float a = used > 0 ? 1.0f - (float)occ / (float)used : 1.0f;
        c->ao[i] = a < 0 ? 0 : a;
    }
}
RNO_API void rno_ssao(int w, int h, const float* pos, const float* nrm, const uint8_t* mask,
                      int samples, float radius, float* ao, int threads) {
    ssao_ctx c = {w, h, pos, nrm, mask, samples, radius, ao};
    parallel_rows(h, threads, ssao_row, &c);
}

/* ------------------------------------------------------------------ reconcile
 * src/cert/reconcile.cpp:4-21: error map, FP64 sum of squares in row-major order, max,
 * count; rmse = (float)sqrt(sum / n); within = rmse <= tolerance. */
RNO_API void rno_reconcile(int w, int h, const float* approx, const float* truth, const uint8_t* mask,
                           float tolerance, float* err, float* rmse, float* maxErr, int* pixels,
                           int* within, double* sumSq) {
    double s = 0; int n = 0; float mx = 0;
    for (int y = 0; y < h; ++y) for (int x = 0; x < w; ++x) {
        const size_t i = (size_t)y * w + x;
        if (!mask[i]) { err[i] = 0; continue; }
        const float e = fabsf(approx[i] - truth[i]);
        err[i] = e;
        if (e > mx) mx = e;
        s += (double)e * e; ++n;
    }
    *pixels = n;
    *rmse = n > 0 ? (float)sqrt(s / n) : 0.0f;
    *maxErr = mx;
    *within = *rmse <= tolerance;
    if (sumSq) *sumSq = s;
}

/* ------------------------------------------------------------------ scene + camera
 * src/scene/scene.cpp:4-32 (buildTestScene), raw/math/mat.hpp:9-35 (mul, perspective,
 * lookAt), raw/scene/scene.hpp:12-17 (Camera: nearZ 0.1, farZ 100). A mesh is flattened
 * into positions (3 f), normals (3 f) and indices; `mesh_of` numbers the triangles. */
typedef struct { float m[16]; } mat4;
static mat4 mat_mul(const mat4* a, const mat4* b) {
    mat4 r; memset(&r, 0, sizeof r);
    for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) {
        float s = 0; for (int k = 0; k < 4; ++k) s += a->m[i * 4 + k] * b->m[k * 4 + j];
        r.m[i * 4 + j] = s;
    }
    return r;
}
static void mat_vec(const mat4* a, const float v[4], float o[4]) {
    for (int r = 0; r < 4; ++r)
        o[r] = a->m[r * 4] * v[0] + a->m[r * 4 + 1] * v[1] + a->m[r * 4 + 2] * v[2] + a->m[r * 4 + 3] * v[3];
}
static mat4 perspective(float fovy, float aspect, float n, float f) {
    const float t = 1.0f / tanf(fovy * 0.5f);
    mat4 r; memset(&r, 0, sizeof r);
    r.m[0] = t / aspect; r.m[5] = t;
    r.m[10] = (f + n) / (n - f); r.m[11] = (2 * f * n) / (n - f);
    r.m[14] = -1;
    return r;
}
static mat4 look_at(v3 eye, v3 center, v3 up) {
    const v3 f = norm3(sub3(center, eye)), s = norm3(cross3(f, up)), u = cross3(s, f);
    mat4 r; memset(&r, 0, sizeof r);
    r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1;
    r.m[0] = s.x; r.m[1] = s.y; r.m[2] = s.z; r.m[3] = -dot3(s, eye);
    r.m[4] = u.x; r.m[5] = u.y; r.m[6] = u.z; r.m[7] = -dot3(u, eye);
    r.m[8] = -f.x; r.m[9] = -f.y; r.m[10] = -f.z; r.m[11] = dot3(f, eye);
    return r;
}
/* The built-in scene: a 10 x 10 plane (2 triangles) and a 2 x 2 x 2 box at (0,1,0)
 * (12 triangles). Writes 14 * 9 positions, 14 * 9 vertex normals (per corner), and the
 * light direction normalize(-0.4,-1,-0.3). Returns the triangle count. */
static int quad(float* P, float* N, int t, v3 a, v3 b, v3 c, v3 d, v3 n) {
    const v3 q[6] = {a, b, c, a, c, d};
    for (int k = 0; k < 6; ++k) {
        P[(t * 3 + k) * 3 + 0] = q[k].x; P[(t * 3 + k) * 3 + 1] = q[k].y; P[(t * 3 + k) * 3 + 2] = q[k].z;
        N[(t * 3 + k) * 3 + 0] = n.x; N[(t * 3 + k) * 3 + 1] = n.y; N[(t * 3 + k) * 3 + 2] = n.z;
    }
    return t + 2;
}
RNO_API int rno_test_scene(float* tris9, float* nrm9, float* light3) {
    int t = 0;
    t = quad(tris9, nrm9, t, v3m(-5, 0, -5), v3m(5, 0, -5), v3m(5, 0, 5), v3m(-5, 0, 5), v3m(0, 1, 0));
    const v3 c = v3m(0, 1, 0); const float h = 1.0f;
    const v3 p0 = v3m(c.x - h, c.y - h, c.z - h), p1 = v3m(c.x + h, c.y + h, c.z + h);
    t = quad(tris9, nrm9, t, v3m(p0.x, p0.y, p1.z), v3m(p1.x, p0.y, p1.z), v3m(p1.x, p1.y, p1.z), v3m(p0.x, p1.y, p1.z), v3m(0, 0, 1));
    t = quad(tris9, nrm9, t, v3m(p1.x, p0.y, p0.z), v3m(p0.x, p0.y, p0.z), v3m(p0.x, p1.y, p0.z), v3m(p1.x, p1.y, p0.z), v3m(0, 0, -1));
    t = quad(tris9, nrm9, t, v3m(p0.x, p1.y, p1.z), v3m(p1.x, p1.y, p1.z), v3m(p1.x, p1.y, p0.z), v3m(p0.x, p1.y, p0.z), v3m(0, 1, 0));
    t = quad(tris9, nrm9, t, v3m(p0.x, p0.y, p0.z), v3m(p1.x, p0.y, p0.z), v3m(p1.x, p0.y, p1.z), v3m(p0.x, p0.y, p1.z), v3m(0, -1, 0));
    t = quad(tris9, nrm9, t, v3m(p1.x, p0.y, p1.z), v3m(p1.x, p0.y, p0.z), v3m(p1.x, p1.y, p0.z), v3m(p1.x, p1.y, p1.z), v3m(1, 0, 0));
    t = quad(tris9, nrm9, t, v3m(p0.x, p0.y, p0.z), v3m(p0.x, p0.y, p1.z), v3m(p0.x, p1.y, p1.z), v3m(p0.x, p1.y, p0.z), v3m(-1, 0, 0));
    if (light3) {
        const v3 l = norm3(v3m(-0.4f, -1.0f, -0.3f));
        light3[0] = l.x; light3[1] = l.y; light3[2] = l.z;
    }
    return t;
}

/* ------------------------------------------------------------------ rasterizer
 * src/renderer/raster.cpp:9-27 (lerp, near clip) and :30-126 (drawTri, rasterize), with
 * the default RasterOptions (no jitter, no snapping, screen-linear depth). Outputs depth,
 * position (3 f), normal (3 f) and mask per pixel. */
typedef struct { float cs[4]; v3 wp, wn; } cvert;
static cvert lerp_vert(const cvert* a, const cvert* b, float t) {
    cvert r;
    for (int k = 0; k < 4; ++k) r.cs[k] = a->cs[k] + (b->cs[k] - a->cs[k]) * t;
    r.wp = v3m(a->wp.x + (b->wp.x - a->wp.x) * t, a->wp.y + (b->wp.y - a->wp.y) * t, a->wp.z + (b->wp.z - a->wp.z) * t);
    r.wn = v3m(a->wn.x + (b->wn.x - a->wn.x) * t, a->wn.y + (b->wn.y - a->wn.y) * t, a->wn.z + (b->wn.z - a->wn.z) * t);
    return r;
}
typedef struct { int w, h; float* depth; float* pos; float* nrm; uint8_t* mask; int32_t* tri; int cur; } rtarget;
static void draw_tri(rtarget* T, const cvert v[3]) {
    const int w = T->w, h = T->h;
    float invw[3]; v3 sp[3];
    for (int k = 0; k < 3; ++k) {
        invw[k] = 1.0f / v[k].cs[3];
        const float nx = v[k].cs[0] * invw[k], ny = v[k].cs[1] * invw[k];
        sp[k].x = (nx * 0.5f + 0.5f) * (float)w;
        sp[k].y = (1.0f - (ny * 0.5f + 0.5f)) * (float)h;
        sp[k].z = v[k].cs[3];
        sp[k].x += 0.0f; sp[k].y += 0.0f;
    }
    const float mnx = smin(smin(sp[0].x, sp[1].x), sp[2].x), mxx = smax(smax(sp[0].x, sp[1].x), sp[2].x);
    const float mny = smin(smin(sp[0].y, sp[1].y), sp[2].y), mxy = smax(smax(sp[0].y, sp[1].y), sp[2].y);
    int minx = (int)floorf(mnx); if (minx < 0) minx = 0;
    int maxx = (int)ceilf(mxx); if (maxx > w - 1) maxx = w - 1;
    int miny = (int)floorf(mny); if (miny < 0) miny = 0;
    int maxy = (int)ceilf(mxy); if (maxy > h - 1) maxy = h - 1;
    const float area = (sp[1].x - sp[0].x) * (sp[2].y - sp[0].y) - (sp[1].y - sp[0].y) * (sp[2].x - sp[0].x);
    if (fabsf(area) < 1e-9f) return;
    for (int y = miny; y <= maxy; ++y) for (int x = minx; x <= maxx; ++x) {
        const float px = (float)x + 0.5f, py = (float)y + 0.5f;
        const float w0 = ((sp[1].x - px) * (sp[2].y - py) - (sp[1].y - py) * (sp[2].x - px)) / area;
        const float w1 = ((sp[2].x - px) * (sp[0].y - py) - (sp[2].y - py) * (sp[0].x - px)) / area;
        const float w2 = 1.0f - w0 - w1;
        if (w0 < 0 || w1 < 0 || w2 < 0) continue;
        const float iw = w0 * invw[0] + w1 * invw[1] + w2 * invw[2];
        const float depth = w0 * sp[0].z + w1 * sp[1].z + w2 * sp[2].z;
        const size_t i = (size_t)y * w + x;
        if (depth >= T->depth[i]) continue;
        const v3* wp = (const v3[3]){v[0].wp, v[1].wp, v[2].wp};
        const v3* wn = (const v3[3]){v[0].wn, v[1].wn, v[2].wn};
        const v3 P = v3m((w0 * wp[0].x * invw[0] + w1 * wp[1].x * invw[1] + w2 * wp[2].x * invw[2]) / iw,
                         (w0 * wp[0].y * invw[0] + w1 * wp[1].y * invw[1] + w2 * wp[2].y * invw[2]) / iw,
                         (w0 * wp[0].z * invw[0] + w1 * wp[1].z * invw[1] + w2 * wp[2].z * invw[2]) / iw);
        const v3 Nn = norm3(v3m((w0 * wn[0].x * invw[0] + w1 * wn[1].x * invw[1] + w2 * wn[2].x * invw[2]) / iw,
                                (w0 * wn[0].y * invw[0] + w1 * wn[1].y * invw[1] + w2 * wn[2].y * invw[2]) / iw,
                                (w0 * wn[0].z * invw[0] + w1 * wn[1].z * invw[1] + w2 * wn[2].z * invw[2]) / iw));
        T->depth[i] = depth;
        T->pos[3 * i] = P.x; T->pos[3 * i + 1] = P.y; T->pos[3 * i + 2] = P.z;
        T->nrm[3 * i] = Nn.x; T->nrm[3 * i + 1] = Nn.y; T->nrm[3 * i + 2] = Nn.z;
        T->mask[i] = 1;
        if (T->tri) T->tri[i] = T->cur;
    }
}
/* cam10: eye(3) center(3) up(3) fovy; aspect = w / h as cameraFromParams
 * (src/tools/cli_params.cpp:12-18) sets it; nearZ 0.1, farZ 100. */
/* tri_out (may be NULL): the index of the triangle each covered pixel shows, -1 elsewhere;
 * a mesh's material albedo is per triangle, so it gives the G-buffer's albedo plane
 * (src/renderer/raster.cpp:76). */
RNO_API void rno_rasterize_ex(const float* tris9, const float* nrm9, int ntri, const float* cam10,
                              int w, int h, float* depth, float* pos, float* nrm, uint8_t* mask, int32_t* tri_out) {
    const size_t np = (size_t)w * h;
    if (tri_out) for (size_t i = 0; i < np; ++i) tri_out[i] = -1;
    for (size_t i = 0; i < np; ++i) { depth[i] = INFINITY; mask[i] = 0; }
    memset(pos, 0, np * 3 * sizeof(float));
    memset(nrm, 0, np * 3 * sizeof(float));
    const v3 eye = v3m(cam10[0], cam10[1], cam10[2]), ctr = v3m(cam10[3], cam10[4], cam10[5]);
    const v3 up = v3m(cam10[6], cam10[7], cam10[8]);
    const float aspect = h > 0 ? (float)w / (float)h : 1.0f, nearZ = 0.1f;
    const mat4 view = look_at(eye, ctr, up), proj = perspective(cam10[9], aspect, nearZ, 100.0f);
    const mat4 vp = mat_mul(&proj, &view);
    rtarget T = {w, h, depth, pos, nrm, mask, tri_out, 0};
    for (int t = 0; t < ntri; ++t) {
        T.cur = t;
        cvert v[3]; int behind = 0;
        for (int k = 0; k < 3; ++k) {
            const float* p = tris9 + (size_t)t * 9 + 3 * k;
            const float* q = nrm9 + (size_t)t * 9 + 3 * k;
            const float hv[4] = {p[0], p[1], p[2], 1};
            mat_vec(&vp, hv, v[k].cs);
            v[k].wp = v3m(p[0], p[1], p[2]); v[k].wn = v3m(q[0], q[1], q[2]);
            behind = behind || v[k].cs[3] <= 1e-6f;
        }
        if (!behind) { draw_tri(&T, v); continue; }
        cvert c[4]; int n = 0;
        for (int k = 0; k < 3; ++k) {
            const cvert* a = &v[k]; const cvert* b = &v[(k + 1) % 3];
            const int ain = a->cs[3] >= nearZ, bin = b->cs[3] >= nearZ;
            if (ain) c[n++] = *a;
            if (ain != bin) c[n++] = lerp_vert(a, b, (nearZ - a->cs[3]) / (b->cs[3] - a->cs[3]));
        }
        for (int k = 1; k + 1 < n; ++k) { const cvert tt[3] = {c[0], c[k], c[k + 1]}; draw_tri(&T, tt); }
    }
}
RNO_API void rno_rasterize(const float* tris9, const float* nrm9, int ntri, const float* cam10,
                           int w, int h, float* depth, float* pos, float* nrm, uint8_t* mask) {
    rno_rasterize_ex(tris9, nrm9, ntri, cam10, w, h, depth, pos, nrm, mask, NULL);
}
/* The built-in scene's albedo per triangle (src/scene/scene.cpp:21-24): the plane's 2 then
 * the box's 12, 3 floats each. */
RNO_API void rno_test_scene_albedo(float* albedo3) {
    for (int t = 0; t < 14; ++t) {
        albedo3[3 * t] = t < 2 ? 0.7f : 0.8f;
        albedo3[3 * t + 1] = t < 2 ? 0.7f : 0.3f;
        albedo3[3 * t + 2] = t < 2 ? 0.7f : 0.2f;
    }
}
/* The camera's view-projection (raw/scene/scene.hpp:21-22 with aspect w / h): 16 floats. */
RNO_API void rno_view_proj(const float* cam10, int w, int h, float* vp16) {
    const v3 eye = v3m(cam10[0], cam10[1], cam10[2]), ctr = v3m(cam10[3], cam10[4], cam10[5]);
    const v3 up = v3m(cam10[6], cam10[7], cam10[8]);
    const float aspect = h > 0 ? (float)w / (float)h : 1.0f;
    const mat4 view = look_at(eye, ctr, up), proj = perspective(cam10[9], aspect, 0.1f, 100.0f);
    const mat4 vp = mat_mul(&proj, &view);
    memcpy(vp16, vp.m, sizeof vp.m);
}

/* ------------------------------------------------------------------ shading and motion
 * src/renderer/composite.cpp:8-42 (radianceAt / radianceV2, shade / shadeV2 and their HDR
 * forms): model 2 lights albedo x (0.2 sky + max(0, n . -l) li sun), model 1 albedo x
 * (0.2 + max(0, n . -l) li) ao; the frame clamps to [0, 1], the HDR view does not; uncovered
 * pixels are 0. src/renderer/motion.cpp:7-32 (projectToUV, computeMotion): current minus
 * previous clip UV of the pixel's world position; returns the valid count. */
RNO_API void rno_shade(int w, int h, const float* nrm, const float* albedo, const uint8_t* mask, int model,
                       const float* a_or_sky, const float* sun, const float* ldir3, float li, float* frame,
                       float* hdr) {
    const v3 nl = mul3(v3m(ldir3[0], ldir3[1], ldir3[2]), -1.0f);
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        float r[3] = {0, 0, 0};
        if (mask[i]) {
            const v3 n = v3m(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
            const float d = dot3(n, nl);
            const float ndl = (d > 0.0f ? d : 0.0f) * li;
            const float lit = model == 2 ? 0.2f * a_or_sky[i] + ndl * sun[i] : (0.2f + ndl) * a_or_sky[i];
            for (int k = 0; k < 3; ++k) r[k] = albedo[3 * i + k] * lit;
        }
        for (int k = 0; k < 3; ++k) {
            hdr[3 * i + k] = r[k];
            frame[3 * i + k] = r[k] < 0.0f ? 0.0f : r[k] > 1.0f ? 1.0f : r[k];
        }
    }
}
static int project_uv(const mat4* vp, const float p[3], float uv[2]) {
    const float hv[4] = {p[0], p[1], p[2], 1.0f};
    float cs[4];
    mat_vec(vp, hv, cs);
    if (cs[3] <= 1e-6f) return 0;
    const float invw = 1.0f / cs[3];
    const float nx = cs[0] * invw, ny = cs[1] * invw;
    uv[0] = nx * 0.5f + 0.5f;
    uv[1] = 1.0f - (ny * 0.5f + 0.5f);
    return 1;
}
RNO_API int rno_motion(int w, int h, const float* pos, const uint8_t* mask, const float* vp16, const float* prev16,
                       float* motion2) {
    mat4 cur, prev;
    memcpy(cur.m, vp16, sizeof cur.m);
    memcpy(prev.m, prev16, sizeof prev.m);
    int valid = 0;
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        motion2[2 * i] = motion2[2 * i + 1] = 0.0f;
        if (!mask[i]) continue;
        float a[2], b[2];
        if (!project_uv(&cur, pos + 3 * i, a) || !project_uv(&prev, pos + 3 * i, b)) continue;
        const float mx = a[0] - b[0], my = a[1] - b[1];
        if (!isfinite(mx) || !isfinite(my)) continue;
        motion2[2 * i] = mx; motion2[2 * i + 1] = my;
        ++valid;
    }
    return valid;
}

/* ------------------------------------------------------------------ PLOC BVH
 * src/renderer/rt_bvh.cpp:83-172 (centroid, pow2Scale, morton3, area, buildPloc).
 * Output nodes: 9 ints each {left, right, tri, bits(lo0), bits(hi0), bits(lo1), ...} in the
 * reference's node order; returns the root and writes the round count. */
typedef struct { float lo[3], hi[3]; int left, right, tri; } pnode;
static uint32_t spread10(uint32_t v) {
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
static float ploc_area(const float* lo, const float* hi) {
    const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return 2.0f * (dy * (dx + dz) + dz * dx);
}
static float pow2_scale(float extent) {
    float s = 1.0f;
    if (!(extent > 0.0f)) return s;
    while (extent * s > 1.0f) s *= 0.5f;
    while (extent * s <= 0.5f) s *= 2.0f;
    return s;
}
static int cmp_u64(const void* a, const void* b) {
    const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : x > y;
}
RNO_API int rno_morton_keys(const float* tris9, int n, uint64_t* keys) {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    float* c = (float*)malloc((size_t)(n ? n : 1) * 3 * sizeof(float));
    const float third = 0.333333343f;
    for (int i = 0; i < n; ++i) {
        const float* t = tris9 + (size_t)i * 9;
        for (int k = 0; k < 3; ++k) {
            c[3 * i + k] = (t[k] + t[3 + k] + t[6 + k]) * third;
            lo[k] = smin(lo[k], c[3 * i + k]); hi[k] = smax(hi[k], c[3 * i + k]);
        }
    }
    const float s = pow2_scale(smax(hi[0] - lo[0], smax(hi[1] - lo[1], hi[2] - lo[2])));
    for (int i = 0; i < n; ++i) {
        uint32_t q[3];
        for (int k = 0; k < 3; ++k) {
            const uint32_t v = (uint32_t)((c[3 * i + k] - lo[k]) * s * 1023.0f);
            q[k] = v < 1023u ? v : 1023u;
        }
        const uint32_t code = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
        keys[i] = ((uint64_t)code << 32) | (uint32_t)i;
    }
    free(c);
    return 0;
}
RNO_API int rno_ploc_build(const float* tris9, int n, int radius, int32_t* out9, uint32_t* rounds) {
    *rounds = 0;
    if (n <= 0) return -1;
    uint64_t* keys = (uint64_t*)malloc((size_t)n * sizeof(uint64_t));
    rno_morton_keys(tris9, n, keys);
    qsort(keys, (size_t)n, sizeof(uint64_t), cmp_u64);
    pnode* N = (pnode*)calloc((size_t)(2 * n - 1), sizeof(pnode));
    for (int i = 0; i < 2 * n - 1; ++i) { N[i].left = N[i].right = N[i].tri = -1; }
    int* cl = (int*)malloc((size_t)n * sizeof(int));
    int* out = (int*)malloc((size_t)n * sizeof(int));
    int* nn = (int*)malloc((size_t)n * sizeof(int));
    for (int i = 0; i < n; ++i) {
        const int t = (int)(uint32_t)keys[i];
        N[i].tri = t;
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) {
                const float x = tris9[(size_t)t * 9 + 3 * k + a];
                N[i].lo[a] = k ? smin(N[i].lo[a], x) : x;
                N[i].hi[a] = k ? smax(N[i].hi[a], x) : x;
            }
        cl[i] = i;
    }
    int next = n, m = n;
    while (m > 1) {
        for (int i = 0; i < m; ++i) {
            float best = FLT_MAX; nn[i] = -1;
            const int j0 = i - radius > 0 ? i - radius : 0, j1 = i + radius < m - 1 ? i + radius : m - 1;
            for (int j = j0; j <= j1; ++j) {
                if (j == i) continue;
                float lo[3], hi[3];
                for (int k = 0; k < 3; ++k) {
                    lo[k] = smin(N[cl[i]].lo[k], N[cl[j]].lo[k]);
                    hi[k] = smax(N[cl[i]].hi[k], N[cl[j]].hi[k]);
                }
                const float d = ploc_area(lo, hi);
                if (d < best) { best = d; nn[i] = j; }
            }
        }
        int mo = 0;
        for (int i = 0; i < m; ++i) {
            const int j = nn[i];
            const int mutual = nn[j] == i;
            if (mutual && i > j) continue;
            if (!mutual) { out[mo++] = cl[i]; continue; }
            pnode* X = &N[next];
            for (int k = 0; k < 3; ++k) {
                X->lo[k] = smin(N[cl[i]].lo[k], N[cl[j]].lo[k]);
                X->hi[k] = smax(N[cl[i]].hi[k], N[cl[j]].hi[k]);
            }
            X->left = cl[i]; X->right = cl[j];
            out[mo++] = next++;
        }
        int* sw = cl; cl = out; out = sw;
        m = mo;
        ++*rounds;
    }
    const int root = cl[0];
    for (int i = 0; i < 2 * n - 1; ++i) {
        int32_t* o = out9 + (size_t)i * 9;
        o[0] = N[i].left; o[1] = N[i].right; o[2] = N[i].tri;
        for (int k = 0; k < 3; ++k) { memcpy(&o[3 + 2 * k], &N[i].lo[k], 4); memcpy(&o[4 + 2 * k], &N[i].hi[k], 4); }
    }
    free(keys); free(N); free(cl); free(out); free(nn);
    return root;
}
/* FNV-1a over every node's fields: src/renderer/gpu/rt_bvh_parity.cpp:49-58. Node layout
 * as rno_ploc_build writes it. */
RNO_API uint64_t rno_tree_hash(const int32_t* nodes9, int count) {
    uint64_t h = 1469598103934665603ull;
    for (int i = 0; i < count; ++i)
        for (int f = 0; f < 9; ++f) {
            const uint32_t v = (uint32_t)nodes9[(size_t)i * 9 + f];
            for (int b = 0; b < 4; ++b) { h ^= (v >> (8 * b)) & 255u; h *= 1099511628211ull; }
        }
    return h;
}
/* src/renderer/rt_scenes.cpp:7-11 (hash, unit) and :52-63 (soup): seeded random triangles
 * in a cube, the reference's BVH check scene. */
static uint32_t soup_hash(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}
RNO_API void rno_soup(int count, uint64_t seed, float* tris9) {
    uint32_t r = (uint32_t)(seed * 2654435761ull + 1ull);
    for (int i = 0; i < count; ++i) {
        float v[12];
        for (int k = 0; k < 12; ++k) { r = soup_hash(r + 0x9e3779b9u); v[k] = (float)(r >> 8) / 16777216.0f; }
        const v3 c = v3m(24.0f * v[0] - 12.0f, 24.0f * v[1] - 12.0f, 24.0f * v[2] - 12.0f);
        const v3 a = add3(c, v3m(2.0f * v[3] - 1.0f, 2.0f * v[4] - 1.0f, 2.0f * v[5] - 1.0f));
        const v3 b = add3(c, v3m(2.0f * v[6] - 1.0f, 2.0f * v[7] - 1.0f, 2.0f * v[8] - 1.0f));
        const v3 d = add3(c, v3m(2.0f * v[9] - 1.0f, 2.0f * v[10] - 1.0f, 2.0f * v[11] - 1.0f));
        float* o = tris9 + (size_t)i * 9;
        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = b.x; o[4] = b.y; o[5] = b.z; o[6] = d.x; o[7] = d.y; o[8] = d.z;
    }
}

/* Any-hit scan for a batch of rays (accel.cpp:31-35 per ray), rows of `threads` workers. */
typedef struct { const tri_t* tris; int ntri; const float* rays; const float* tmax; uint8_t* hit; int n; } scan_ctx;
static void scan_row(void* p, int i) {
    const scan_ctx* c = (const scan_ctx*)p;
    const float* r = c->rays + (size_t)i * 6;
    c->hit[i] = (uint8_t)scan_occluded(c->tris, c->ntri, v3m(r[0], r[1], r[2]), v3m(r[3], r[4], r[5]), c->tmax[i]);
}
RNO_API void rno_occluded_scan_batch(const float* tris9, int ntri, const float* rays6, const float* tmax, int n,
                                     uint8_t* hit, int threads) {
    scan_ctx c = {(const tri_t*)tris9, ntri, rays6, tmax, hit, n};
    parallel_rows(n, threads, scan_row, &c);
}

/* ------------------------------------------------------------------ closest hit, hybrid
 * rt::closest (src/renderer/rt_bvh.cpp:125-152) by its definition: the smallest t of the
 * watertight test below tMax, ties to the lowest triangle index (the rule its walk keeps:
 * tt < best, or tt == best with a lower index); here by scanning every triangle in index
 * order, as the reference's own hybrid check does (src/renderer/gpu/rt_hybrid_parity.cpp:66-71). */
static int scan_closest(const tri_t* tris, int ntri, v3 o, v3 d, float tmax, float* tout) {
    int best_tri = -1;
    float best = tmax;
    for (int i = 0; i < ntri; ++i) {
        float t;
        if (!intersect_tri(o, d, &tris[i], &t)) continue;
        if (t < best) { best = t; best_tri = i; }      /* in index order a tie keeps the lower index */
    }
    *tout = best;
    return best_tri;
}
typedef struct { const tri_t* tris; int ntri; const float* rays; const float* tmax; int32_t* tri; float* t; } closest_ctx;
static void closest_row(void* p, int i) {
    const closest_ctx* c = (const closest_ctx*)p;
    const float* r = c->rays + (size_t)i * 6;
    float t;
    const int id = scan_closest(c->tris, c->ntri, v3m(r[0], r[1], r[2]), v3m(r[3], r[4], r[5]), c->tmax[i], &t);
    c->tri[i] = id;
    c->t[i] = id >= 0 ? t : -1.0f;
}
RNO_API void rno_closest_scan_batch(const float* tris9, int ntri, const float* rays6, const float* tmax, int n,
                                    int32_t* tri, float* t, int threads) {
    closest_ctx c = {(const tri_t*)tris9, ntri, rays6, tmax, tri, t};
    parallel_rows(n, threads, closest_row, &c);
}

/* The hybrid pass's per-pixel rule (src/renderer/gpu/rt_hybrid_parity.cpp:35-41, 57-80) over
 * a G-buffer: d = normalize(pos - eye); the geometric normal (a plane of its own, or the
 * G-buffer normal when none is given) turned to face the viewer, the shading normal (the
 * G-buffer normal) turned to its side; origins pushed off by 2e-4 (1 + max |pos|) along the
 * geometric normal toward each ray; lit = no hit toward normalize(sun) below 1e30 (1, else
 * 0); the mirror ray d - n (2 d.n) and its nearest hit below 1e30. Uncovered: -1. */
typedef struct {
    int w; const float* pos; const float* nrm; const float* ng; const uint8_t* mask; const tri_t* tris; int ntri;
    v3 eye, sun; float* lit; int32_t* tri; float* t;
} hybrid_ctx;
static v3 offset_of(v3 p, v3 n, v3 dir) {
    const float e = 2e-4f * (1.0f + smax(fabsf(p.x), smax(fabsf(p.y), fabsf(p.z))));
    return add3(p, mul3(n, dot3(n, dir) > 0.0f ? e : -e));
}
static void hybrid_row(void* p, int y) {
    const hybrid_ctx* c = (const hybrid_ctx*)p;
    for (int x = 0; x < c->w; ++x) {
        const size_t i = (size_t)y * c->w + x;
        if (!c->mask[i]) { c->lit[i] = -1.0f; c->tri[i] = -1; c->t[i] = -1.0f; continue; }
        const v3 pos = v3m(c->pos[3 * i], c->pos[3 * i + 1], c->pos[3 * i + 2]);
        v3 n = v3m(c->nrm[3 * i], c->nrm[3 * i + 1], c->nrm[3 * i + 2]);
        v3 ng = c->ng ? v3m(c->ng[3 * i], c->ng[3 * i + 1], c->ng[3 * i + 2]) : n;
        const v3 d = norm3(sub3(pos, c->eye));
        if (dot3(ng, d) > 0.0f) ng = mul3(ng, -1.0f);
        if (dot3(n, ng) < 0.0f) n = mul3(n, -1.0f);
        const v3 l = norm3(c->sun);
        c->lit[i] = scan_occluded(c->tris, c->ntri, offset_of(pos, ng, l), l, 1e30f) ? 0.0f : 1.0f;
        const v3 r = sub3(d, mul3(n, 2.0f * dot3(d, n)));
        float t;
        const int id = scan_closest(c->tris, c->ntri, offset_of(pos, ng, r), r, 1e30f, &t);
        c->tri[i] = id;
        c->t[i] = id >= 0 ? t : -1.0f;
    }
}
RNO_API void rno_hybrid(int w, int h, const float* pos, const float* nrm, const float* ng, const uint8_t* mask,
                        const float* tris9, int ntri, const float* eye3, const float* sun3, float* lit, int32_t* tri,
                        float* t, int threads) {
    hybrid_ctx c = {w, pos, nrm, ng, mask, (const tri_t*)tris9, ntri, v3m(eye3[0], eye3[1], eye3[2]),
                    v3m(sun3[0], sun3[1], sun3[2]), lit, tri, t};
    parallel_rows(h, threads, hybrid_row, &c);
}

/* ------------------------------------------------------------------ GTAO (raw::post)
 * The view-space G-buffer (src/renderer/post_gtao.cpp:36-53, in float as there), the screen
 * projection (:55-61), the depth sample between pixel centres (:14-33) and GTAO itself
 * (:64-135: Jimenez et al. 2016, per slice the two horizon angles clamped to the projected
 * normal's hemisphere, integrated against the cosine), all in double as the reference. The
 * view depth is negative where nothing was drawn. cam10 as rno_rasterize. */
RNO_API void rno_view_gbuffer(int w, int h, const float* pos, const float* nrm, const uint8_t* mask, const float* cam10,
                              float* vpos, float* vnrm, float* vdepth) {
    const v3 eye = v3m(cam10[0], cam10[1], cam10[2]), ctr = v3m(cam10[3], cam10[4], cam10[5]);
    const v3 up = v3m(cam10[6], cam10[7], cam10[8]);
    const mat4 view = look_at(eye, ctr, up);
    const size_t n = (size_t)w * h;
    for (size_t i = 0; i < n; ++i) {
        vpos[3 * i] = vpos[3 * i + 1] = vpos[3 * i + 2] = 0.0f;
        vnrm[3 * i] = vnrm[3 * i + 1] = vnrm[3 * i + 2] = 0.0f;
        vdepth[i] = -1.0f;
        if (!mask[i]) continue;
        const float p4[4] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], 1.0f};
        const float n4[4] = {nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2], 0.0f};
        float pv[4], nv[4];
        mat_vec(&view, p4, pv);
        mat_vec(&view, n4, nv);
        const v3 nn = norm3(v3m(nv[0], nv[1], nv[2]));
        vpos[3 * i] = pv[0]; vpos[3 * i + 1] = pv[1]; vpos[3 * i + 2] = pv[2];
        vnrm[3 * i] = nn.x; vnrm[3 * i + 1] = nn.y; vnrm[3 * i + 2] = nn.z;
        vdepth[i] = -pv[2];
    }
}

typedef struct { int w, h; double tanHalf, aspect; const float *pos, *nrm, *depth; } vgb;
static int vgb_valid(const vgb* v, int x, int y) {
    return x >= 0 && y >= 0 && x < v->w && y < v->h && v->depth[(size_t)y * v->w + x] >= 0.0f;
}
static double d3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static double gt_sample_depth(const vgb* v, double fx, double fy, int sx, int sy) {
    const double nearest = v->depth[(size_t)sy * v->w + sx];
    const int x0 = (int)floor(fx - 0.5), y0 = (int)floor(fy - 0.5);
    const double ax = fx - 0.5 - x0, ay = fy - 0.5 - y0;
    double k[4], lo = 1e30, hi = 0.0;
    for (int q = 0; q < 4; ++q) {
        const int qx = x0 + (q & 1), qy = y0 + (q >> 1);
        if (!vgb_valid(v, qx, qy)) return nearest;
        const double d = v->depth[(size_t)qy * v->w + qx];
        lo = d < lo ? d : lo; hi = d > hi ? d : hi;
        k[q] = 1.0 / d;
    }
    if (hi > 1.1 * lo) return nearest;
    const double inv = (k[0] * (1 - ax) + k[1] * ax) * (1 - ay) + (k[2] * (1 - ax) + k[3] * ax) * ay;
    return 1.0 / inv;
}
static int gt_project(const vgb* v, const double p[3], double* sx, double* sy) {
    if (p[2] >= -1e-6) return 0;
    const double w = -p[2];
    *sx = (p[0] / (w * v->tanHalf * v->aspect) * 0.5 + 0.5) * v->w;
    *sy = (1.0 - (p[1] / (w * v->tanHalf) * 0.5 + 0.5)) * v->h;
    return 1;
}
static double clampd(double x, double lo, double hi) { return x < lo ? lo : x > hi ? hi : x; }

/* tanHalf = tan(0.5 * (double)fovy), aspect = (double)(float)(w / h) as the Camera holds it. */
RNO_API void rno_gtao(int w, int h, const float* vpos, const float* vnrm, const float* vdepth, double tanHalf,
                      double aspect, double radius, int slices, int steps, double* out) {
    const double kPi = 3.14159265358979323846;
    const vgb V0 = {w, h, tanHalf, aspect, vpos, vnrm, vdepth};
    const vgb* v = &V0;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const size_t i = (size_t)y * w + x;
            out[i] = 1.0;
            if (vdepth[i] < 0.0f) continue;
            const double P[3] = {vpos[3 * i], vpos[3 * i + 1], vpos[3 * i + 2]};
            const double N[3] = {vnrm[3 * i], vnrm[3 * i + 1], vnrm[3 * i + 2]};
            const double pl = sqrt(d3(P, P));
            const double Vv[3] = {-P[0] / pl, -P[1] / pl, -P[2] / pl};
            const double rpx = radius * h / (2.0 * tanHalf * vdepth[i]);
            double T[3] = {1.0 - Vv[0] * Vv[0], -Vv[0] * Vv[1], -Vv[0] * Vv[2]};
            const double tl = sqrt(d3(T, T));
            T[0] /= tl; T[1] /= tl; T[2] /= tl;
            const double B[3] = {Vv[1] * T[2] - Vv[2] * T[1], Vv[2] * T[0] - Vv[0] * T[2], Vv[0] * T[1] - Vv[1] * T[0]};
            double sx0 = 0, sy0 = 0;
            gt_project(v, P, &sx0, &sy0);
            double sum = 0.0;
            for (int s = 0; s < slices; ++s) {
                const double phi = kPi * (s + 0.5) / slices, cp = cos(phi), sp = sin(phi);
                const double dir[3] = {cp * T[0] + sp * B[0], cp * T[1] + sp * B[1], cp * T[2] + sp * B[2]};
                const double e = 1e-3 * vdepth[i];
                const double Q[3] = {P[0] + dir[0] * e, P[1] + dir[1] * e, P[2] + dir[2] * e};
                double sx1 = 0, sy1 = 0;
                gt_project(v, Q, &sx1, &sy1);
                const double ddl = hypot(sx1 - sx0, sy1 - sy0);
                if (ddl < 1e-12) continue;
                const double c = (sx1 - sx0) / ddl, sn = (sy1 - sy0) / ddl;
                const double dv = d3(dir, Vv);
                const double od[3] = {dir[0] - dv * Vv[0], dir[1] - dv * Vv[1], dir[2] - dv * Vv[2]};
                double ax[3] = {od[1] * Vv[2] - od[2] * Vv[1], od[2] * Vv[0] - od[0] * Vv[2], od[0] * Vv[1] - od[1] * Vv[0]};
                const double al = sqrt(d3(ax, ax));
                ax[0] /= al; ax[1] /= al; ax[2] /= al;
                const double na = d3(N, ax);
                const double pn[3] = {N[0] - ax[0] * na, N[1] - ax[1] * na, N[2] - ax[2] * na};
                const double pnl = sqrt(d3(pn, pn));
                if (pnl < 1e-9) continue;
                const double sgn = d3(od, pn) >= 0.0 ? 1.0 : -1.0;
                const double cn = clampd(d3(pn, Vv) / pnl, 0.0, 1.0), nang = sgn * acos(cn);
                double hc[2] = {cos(nang + kPi / 2), cos(nang - kPi / 2)};
                for (int side = 0; side < 2; ++side) {
                    const double sd = side == 0 ? 1.0 : -1.0;
                    for (int k = 1; k <= steps; ++k) {
                        const double off = sd * rpx * k / steps;
                        const double fx = x + 0.5 + off * c, fy = y + 0.5 + off * sn;
                        const int sx = (int)floor(fx), sy = (int)floor(fy);
                        if (!vgb_valid(v, sx, sy) || (sx == x && sy == y)) continue;
                        const double D = gt_sample_depth(v, fx, fy, sx, sy);
                        const double S[3] = {(fx / w * 2.0 - 1.0) * D * tanHalf * aspect, (1.0 - fy / h * 2.0) * D * tanHalf, -D};
                        const double dd[3] = {S[0] - P[0], S[1] - P[1], S[2] - P[2]}, dl = sqrt(d3(dd, dd));
                        if (dl < 1e-9 || dl > radius) continue;
                        const double cosh_ = d3(dd, Vv) / dl;
                        hc[side] = cosh_ > hc[side] ? cosh_ : hc[side];
                    }
                }
                const double m1 = acos(clampd(hc[0], -1.0, 1.0)) - nang, m0 = -acos(clampd(hc[1], -1.0, 1.0)) - nang;
                const double h1 = nang + (m1 < kPi / 2 ? m1 : kPi / 2);
                const double h0 = nang + (m0 > -kPi / 2 ? m0 : -kPi / 2);
                const double sn2 = sin(nang);
                const double a0 = (cn + 2.0 * h0 * sn2 - cos(2.0 * h0 - nang)) / 4.0;
                const double a1 = (cn + 2.0 * h1 * sn2 - cos(2.0 * h1 - nang)) / 4.0;
                sum += pnl * (a0 + a1);
            }
            out[i] = sum / slices;
        }
}

/* ------------------------------------------------------------------ the path tracer
 * raw::rt::pathTraceCpu (interface v4, v2 scenes): in its own file, built into this library. */
#include "rn_oracle_pt.c"
