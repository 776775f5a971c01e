// ploc.cu -- the GPU BVH builder: PLOC (Meister and Bittner, TVCG 2018) as raw-native's
// CPU reference defines it (src/renderer/rt_bvh.cpp:83-172), built node for node on the
// device, then collapsed into 4-wide nodes for the AO traversal.
//
//   1. centroids (a + b + c) * 0.333333343f and their bounds      (one pass, atomics on
//      order-preserving integer images of the floats: min/max are exact and order-free)
//   2. 30-bit Morton codes after the power-of-two scale            (one pass)
//   3. stable LSD radix sort of (code, index), 8-bit digits        (4 x histogram/scan/scatter)
//   4. leaves in sorted order                                       (one pass)
//   5. rounds: nearest neighbour within +-radius positions by the factored union area (ties to
//      the lower position), merge mutual pairs into nodes numbered by a prefix sum in position
//      order, compact the survivors. The round count lives on the device: the host launches
//      rounds in batches and reads the survivor count once per batch, not once per round.
//   6. collapse: subtree sizes bottom-up, then level by level each 4-wide node takes the
//      binary node's children and opens the largest-area interior child until it has 4;
//      subtrees of at most leaf_max (<= 8) triangles become leaves with their triangles copied
//      contiguously (48-byte records).
#include "rn_internal.h"
#include "rn_device.cuh"
#include <cooperative_groups.h>
#include <cfloat>
#include <cstring>
#include <vector>

namespace rn {
namespace {
namespace cg = cooperative_groups;

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;     // elements per block in scans and sorts

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ------------------------------------------------------------------ block scan helpers
// Exclusive scan of one value per thread across the block; returns the block total too.
template <typename T>
__device__ T block_exclusive_scan(T v, T& total) {
    __shared__ T warp_tot[kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x = v;
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T w = lane < kThreads / 32 ? warp_tot[lane] : T(0);
        for (int o = 1; o < kThreads / 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kThreads / 32) warp_tot[lane] = w;
    }
    __syncthreads();
    const T before = warp == 0 ? T(0) : warp_tot[warp - 1];
    total = warp_tot[kThreads / 32 - 1];
    __syncthreads();
    return before + x - v;
}

// ------------------------------------------------------------------ generic u32 scan
__global__ void scan_reduce_u32(const uint32_t* __restrict__ in, uint32_t n, uint32_t* __restrict__ bsum) {
    const uint32_t base = blockIdx.x * kTile + threadIdx.x * kItems;
    uint32_t s = 0;
    for (int k = 0; k < kItems; ++k) if (base + k < n) s += in[base + k];
    uint32_t tot;
    block_exclusive_scan<uint32_t>(s, tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}
// One block scans `count` block sums in place (exclusive), chunk by chunk with a carry.
__global__ void scan_top_u32(uint32_t* __restrict__ bsum, uint32_t count, uint32_t* total) {
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t c0 = 0; c0 < count; c0 += kThreads) {
        const uint32_t i = c0 + threadIdx.x;
        const uint32_t v = i < count ? bsum[i] : 0;
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan<uint32_t>(v, tot);
        if (i < count) bsum[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total) *total = carry;
}
__global__ void scan_down_u32(const uint32_t* __restrict__ in, uint32_t n, const uint32_t* __restrict__ bsum,
                              uint32_t* __restrict__ out) {
    const uint32_t base = blockIdx.x * kTile + threadIdx.x * kItems;
    uint32_t v[kItems], s = 0;
    for (int k = 0; k < kItems; ++k) { v[k] = base + k < n ? in[base + k] : 0; s += v[k]; }
    uint32_t tot;
    uint32_t run = block_exclusive_scan<uint32_t>(s, tot) + bsum[blockIdx.x];
    for (int k = 0; k < kItems; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
}
// ------------------------------------------------------------------ centroids and codes
struct Bounds { unsigned lo[3], hi[3]; };

__global__ void init_bounds(Bounds* b) {
    if (threadIdx.x < 3) { b->lo[threadIdx.x] = f2ord(FLT_MAX); b->hi[threadIdx.x] = f2ord(-FLT_MAX); }
}
// rt_bvh.cpp:92-95 (centroid) and :116-122 (centroid bounds).
__global__ void centroid_bounds(const float* __restrict__ tris, uint32_t n, float* __restrict__ cent, Bounds* b) {
    __shared__ unsigned slo[3], shi[3];
    if (threadIdx.x < 3) { slo[threadIdx.x] = f2ord(FLT_MAX); shi[threadIdx.x] = f2ord(-FLT_MAX); }
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const float* t = tris + (size_t)i * 9;
        const float third = 0.333333343f;
        for (int k = 0; k < 3; ++k) {
            const float c = fmul(fadd(fadd(t[k], t[3 + k]), t[6 + k]), third);
            cent[(size_t)i * 3 + k] = c;
            atomicMin(&slo[k], f2ord(c));
            atomicMax(&shi[k], f2ord(c));
        }
    }
    __syncthreads();
    if (threadIdx.x < 3) { atomicMin(&b->lo[threadIdx.x], slo[threadIdx.x]); atomicMax(&b->hi[threadIdx.x], shi[threadIdx.x]); }
}
// rt_bvh.cpp:96-102: the power of two that maps the extent into (0.5, 1]; 1 for none.
__device__ float pow2_scale(float extent) {
    float s = 1.0f;
    if (!(extent > 0.0f)) return s;
    for (int g = 0; g < 600 && fmul(extent, s) > 1.0f; ++g) s = fmul(s, 0.5f);
    for (int g = 0; g < 600 && fmul(extent, s) <= 0.5f; ++g) s = fmul(s, 2.0f);
    return s;
}
__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
// rt_bvh.cpp:123-130: 10-bit quantization min(1023, (x - lo) * s * 1023), code = morton3.
__global__ void morton_codes(const float* __restrict__ cent, uint32_t n, const Bounds* __restrict__ b,
                             uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    __shared__ float slo[3], sscale;
    if (threadIdx.x == 0) {
        float lo[3], hi[3];
        for (int k = 0; k < 3; ++k) { lo[k] = ord2f(b->lo[k]); hi[k] = ord2f(b->hi[k]); slo[k] = lo[k]; }
        sscale = pow2_scale(smax(fsub(hi[0], lo[0]), smax(fsub(hi[1], lo[1]), fsub(hi[2], lo[2]))));
    }
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t q[3];
    for (int k = 0; k < 3; ++k) {
        const uint32_t v = (uint32_t)fmul(fmul(fsub(cent[(size_t)i * 3 + k], slo[k]), sscale), 1023.0f);
        q[k] = v < 1023u ? v : 1023u;
    }
    keys[i] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
    vals[i] = i;
}

// ------------------------------------------------------------------ radix sort
__global__ void rs_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift, uint32_t nb,
                        uint32_t* __restrict__ hist) {
    __shared__ uint32_t cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    for (int j = 0; j < kItems; ++j) {
        const uint32_t e = blockIdx.x * kTile + j * kThreads + threadIdx.x;
        if (e < n) atomicAdd(&cnt[(keys[e] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nb + blockIdx.x] = cnt[threadIdx.x];
}
// Stable scatter: elements of a tile keep their order within each digit (tile order =
// element order, striped across threads so each pass over j covers 256 consecutive keys).
__global__ void rs_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint32_t n,
                           int shift, uint32_t nb, const uint32_t* __restrict__ offs,
                           uint32_t* __restrict__ kout, uint32_t* __restrict__ vout) {
    __shared__ uint32_t wcnt[kThreads / 32][256];
    __shared__ uint32_t running[256];
    __shared__ uint32_t base[256];
    const int tid = threadIdx.x, warp = tid >> 5;
    base[tid] = offs[tid * nb + blockIdx.x];
    running[tid] = 0;
    for (int j = 0; j < kItems; ++j) {
        for (int q = tid; q < (kThreads / 32) * 256; q += kThreads) (&wcnt[0][0])[q] = 0;
        __syncthreads();
        const uint32_t e = blockIdx.x * kTile + j * kThreads + tid;
        const bool valid = e < n;
        const uint32_t k = valid ? kin[e] : 0u, v = valid ? vin[e] : 0u;
        const uint32_t d = (k >> shift) & 255u;
        const unsigned peers = __match_any_sync(0xffffffffu, valid ? d : 0xFFFFFFFFu);
        const uint32_t r = __popc(peers & lanemask_lt());
        if (valid && r == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t off = running[d];
            for (int w = 0; w < warp; ++w) off += wcnt[w][d];
            const uint32_t pos = base[d] + off + r;
            kout[pos] = k;
            vout[pos] = v;
        }
        __syncthreads();
        uint32_t add = 0;
        for (int w = 0; w < kThreads / 32; ++w) add += wcnt[w][tid];
        running[tid] += add;
        __syncthreads();
    }
}

// ------------------------------------------------------------------ leaves
// rt_bvh.cpp:68-77 (leafBox) and :134-139.
__global__ void make_leaves(const float* __restrict__ tris, const uint32_t* __restrict__ order, uint32_t n,
                            float* __restrict__ box, int32_t* __restrict__ left, int32_t* __restrict__ right,
                            int32_t* __restrict__ tri, float* __restrict__ cbox, int32_t* __restrict__ cl) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t t = order[i];
    const float* v = tris + (size_t)t * 9;
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) { lo[a] = v[a]; hi[a] = v[a]; }
    for (int k = 1; k < 3; ++k)
        for (int a = 0; a < 3; ++a) { lo[a] = smin(lo[a], v[3 * k + a]); hi[a] = smax(hi[a], v[3 * k + a]); }
    for (int a = 0; a < 3; ++a) {
        box[(size_t)i * 6 + a] = lo[a]; box[(size_t)i * 6 + 3 + a] = hi[a];
        cbox[(size_t)i * 6 + a] = lo[a]; cbox[(size_t)i * 6 + 3 + a] = hi[a];
    }
    left[i] = -1; right[i] = -1; tri[i] = (int32_t)t;
    cl[i] = (int32_t)i;
}
__global__ void init_internal(uint32_t n, float* __restrict__ box, int32_t* __restrict__ left,
                              int32_t* __restrict__ right, int32_t* __restrict__ tri) {
    const uint32_t i = n + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * n - 1) return;
    for (int a = 0; a < 6; ++a) box[(size_t)i * 6 + a] = 0.0f;
    left[i] = -1; right[i] = -1; tri[i] = -1;
}

// ------------------------------------------------------------------ PLOC rounds
struct RoundState {
    uint32_t m;          // clusters in the current round
    uint32_t next;       // id of the next internal node
    uint32_t parity;     // which cluster buffer is current
    uint32_t rounds;     // rounds done
    uint32_t m_next;     // survivors after this round (written by the top scan)
    uint32_t merges;     // merges in this round
    uint32_t error;      // DEV_PLOC_NO_MERGE when a round merged nothing
    int32_t root;        // the last cluster, written by the tail kernels when one is left
    uint32_t stop;       // the launched rounds do nothing once m <= stop (the tail's threshold, or 1)
};

// rt_bvh.cpp:104-110: 2 (dy (dx + dz) + dz dx), operation for operation.
__device__ __forceinline__ float ploc_area(float lx, float ly, float lz, float hx, float hy, float hz) {
    const float dx = fsub(hx, lx), dy = fsub(hy, ly), dz = fsub(hz, lz);
    return fmul(2.0f, fadd(fmul(dy, fadd(dx, dz)), fmul(dz, dx)));
}

// rt_bvh.cpp:143-152: nearest neighbour of each cluster within +-radius positions.
template <int R>
__global__ void ploc_nn(const RoundState* __restrict__ st, const float* __restrict__ cbox0,
                        const float* __restrict__ cbox1, int32_t* __restrict__ nn) {
    __shared__ float sb[6][kThreads + 2 * R];
    const uint32_t m = st->m;
    const float* cbox = st->parity ? cbox1 : cbox0;
    const int base = blockIdx.x * kThreads;
    if (m <= st->stop || (uint32_t)base >= m) return;
    for (int q = threadIdx.x; q < kThreads + 2 * R; q += kThreads) {
        const int j = base - R + q;
        if (j >= 0 && (uint32_t)j < m)
            for (int a = 0; a < 6; ++a) sb[a][q] = cbox[(size_t)j * 6 + a];
    }
    __syncthreads();
    const int i = base + threadIdx.x;
    if ((uint32_t)i >= m) return;
    const int li = threadIdx.x + R;
    const float alx = sb[0][li], aly = sb[1][li], alz = sb[2][li], ahx = sb[3][li], ahy = sb[4][li], ahz = sb[5][li];
    const int j0 = i - R > 0 ? i - R : 0, j1 = i + R < (int)m - 1 ? i + R : (int)m - 1;
    float best = FLT_MAX;
    int arg = -1;
    for (int j = j0; j <= j1; ++j) {
        if (j == i) continue;
        const int lj = j - base + R;
        const float d = ploc_area(smin(alx, sb[0][lj]), smin(aly, sb[1][lj]), smin(alz, sb[2][lj]),
                                  smax(ahx, sb[3][lj]), smax(ahy, sb[4][lj]), smax(ahz, sb[5][lj]));
        if (d < best) { best = d; arg = j; }
    }
    nn[i] = arg;
}
// Generic-radius fallback (a radius other than 8, 16 or 32): reads neighbours from global memory.
__global__ void ploc_nn_any(const RoundState* __restrict__ st, const float* __restrict__ cbox0,
                            const float* __restrict__ cbox1, int32_t* __restrict__ nn, int R) {
    const uint32_t m = st->m;
    const float* cbox = st->parity ? cbox1 : cbox0;
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (m <= st->stop || (uint32_t)i >= m) return;
    const float* A = cbox + (size_t)i * 6;
    const int j0 = i - R > 0 ? i - R : 0, j1 = i + R < (int)m - 1 ? i + R : (int)m - 1;
    float best = FLT_MAX;
    int arg = -1;
    for (int j = j0; j <= j1; ++j) {
        if (j == i) continue;
        const float* B = cbox + (size_t)j * 6;
        const float d = ploc_area(smin(A[0], B[0]), smin(A[1], B[1]), smin(A[2], B[2]),
                                  smax(A[3], B[3]), smax(A[4], B[4]), smax(A[5], B[5]));
        if (d < best) { best = d; arg = j; }
    }
    nn[i] = arg;
}

// Flags of position i (rt_bvh.cpp:155-159): a mutual pair is kept by its lower position,
// which makes the node; a cluster without a mutual neighbour survives as it is.
__device__ __forceinline__ void ploc_flags(const int32_t* __restrict__ nn, uint32_t i, uint32_t& out, uint32_t& merge) {
    const int32_t j = nn[i];
    const bool mutual = j >= 0 && nn[j] == (int32_t)i;
    out = (!mutual || (int32_t)i < j) ? 1u : 0u;
    merge = (mutual && (int32_t)i < j) ? 1u : 0u;
}
__global__ void ploc_count(const RoundState* __restrict__ st, const int32_t* __restrict__ nn,
                           unsigned long long* __restrict__ bsum) {
    const uint32_t m = st->m;
    if (m <= st->stop || blockIdx.x * (uint32_t)kTile >= m) return;
    const uint32_t base = blockIdx.x * kTile + threadIdx.x * kItems;
    unsigned long long s = 0;
    for (int k = 0; k < kItems; ++k)
        if (base + k < m) {
            uint32_t o, g;
            ploc_flags(nn, base + k, o, g);
            s += (unsigned long long)o | ((unsigned long long)g << 32);
        }
    unsigned long long tot;
    block_exclusive_scan<unsigned long long>(s, tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}
__global__ void ploc_top(RoundState* st, unsigned long long* __restrict__ bsum) {
    __shared__ unsigned long long carry;
    const uint32_t m = st->m;
    if (m <= st->stop) return;
    const uint32_t nb = (m + kTile - 1) / kTile;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t c0 = 0; c0 < nb; c0 += kThreads) {
        const uint32_t i = c0 + threadIdx.x;
        const unsigned long long v = i < nb ? bsum[i] : 0ull;
        unsigned long long tot;
        const unsigned long long ex = block_exclusive_scan<unsigned long long>(v, tot);
        if (i < nb) bsum[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        st->m_next = (uint32_t)(carry & 0xFFFFFFFFull);
        st->merges = (uint32_t)(carry >> 32);
        if (st->merges == 0) st->error |= DEV_PLOC_NO_MERGE;
    }
}
// rt_bvh.cpp:155-167: write merged nodes (box = min/max of the pair, left = lower position)
// and the compacted cluster list.
__global__ void ploc_scatter(const RoundState* __restrict__ st, const int32_t* __restrict__ nn,
                             const unsigned long long* __restrict__ bsum,
                             const int32_t* __restrict__ cl0, const int32_t* __restrict__ cl1,
                             int32_t* __restrict__ clo0, int32_t* __restrict__ clo1,
                             const float* __restrict__ cb0, const float* __restrict__ cb1,
                             float* __restrict__ cbo0, float* __restrict__ cbo1,
                             float* __restrict__ box, int32_t* __restrict__ left, int32_t* __restrict__ right) {
    const uint32_t m = st->m;
    if (m <= st->stop || st->merges == 0 || blockIdx.x * (uint32_t)kTile >= m) return;
    const bool p = st->parity != 0;
    const int32_t* cl = p ? cl1 : cl0;
    int32_t* clo = p ? clo0 : clo1;        // the other buffer of the pair
    const float* cb = p ? cb1 : cb0;
    float* cbo = p ? cbo0 : cbo1;
    const uint32_t next = st->next;
    const uint32_t base = blockIdx.x * kTile + threadIdx.x * kItems;
    uint32_t o[kItems], g[kItems];
    unsigned long long s = 0;
    for (int k = 0; k < kItems; ++k) {
        o[k] = g[k] = 0;
        if (base + k < m) ploc_flags(nn, base + k, o[k], g[k]);
        s += (unsigned long long)o[k] | ((unsigned long long)g[k] << 32);
    }
    unsigned long long tot;
    unsigned long long run = block_exclusive_scan<unsigned long long>(s, tot) + bsum[blockIdx.x];
    for (int k = 0; k < kItems; ++k) {
        const uint32_t i = base + k;
        if (i < m && o[k]) {
            const uint32_t pos = (uint32_t)(run & 0xFFFFFFFFull);
            if (g[k]) {
                const uint32_t id = next + (uint32_t)(run >> 32);
                const int32_t j = nn[i];
                const float* A = cb + (size_t)i * 6;
                const float* B = cb + (size_t)j * 6;
                float nb6[6];
                for (int a = 0; a < 3; ++a) { nb6[a] = smin(A[a], B[a]); nb6[3 + a] = smax(A[3 + a], B[3 + a]); }
                for (int a = 0; a < 6; ++a) { box[(size_t)id * 6 + a] = nb6[a]; cbo[(size_t)pos * 6 + a] = nb6[a]; }
                left[id] = cl[i];
                right[id] = cl[j];
                clo[pos] = (int32_t)id;
            } else {
                for (int a = 0; a < 6; ++a) cbo[(size_t)pos * 6 + a] = cb[(size_t)i * 6 + a];
                clo[pos] = cl[i];
            }
        }
        run += (unsigned long long)o[k] | ((unsigned long long)g[k] << 32);
    }
}
// The round's flags, their prefix sum and the scatter in one launch (ploc_count + ploc_top +
// ploc_scatter + ploc_commit): a tile of kTile positions per block, tiles handed out by a
// ticket so that every tile a block waits on is already running, and the prefix across tiles
// by decoupled look-back (Merrill and Garland, 2016): each tile publishes its total, then
// adds its predecessors' totals back to the first one that published its inclusive prefix.
// A status word packs the round (6 bits), the kind (aggregate 1, inclusive prefix 2) and
// the two sums (survivors, merges: 28 bits each; n < 2^28). The tile that ends the round
// commits the state (ploc_commit's update) and clears the next launch's ticket (tickets are
// counted per launch, `launch` numbering this build's merge launches: a block that starts
// after the commit takes a ticket past the round's tiles and leaves). Every wait is bounded:
// a tile that gives up sets DEV_GUARD and publishes anyway, and the build fails.
constexpr uint64_t kLookOut = (1ull << 28) - 1;
constexpr int kLookSpin = 1 << 22;
__device__ __forceinline__ uint64_t look_load(const unsigned long long* p) {
    uint64_t v;
    asm volatile("ld.global.acquire.gpu.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void look_store(unsigned long long* p, uint64_t v) {
    asm volatile("st.global.release.gpu.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__global__ void ploc_merge(RoundState* st, const int32_t* __restrict__ nn, unsigned long long* look, uint32_t* ticket,
                           uint32_t launch, int32_t* __restrict__ cl0, int32_t* __restrict__ cl1, float* __restrict__ cb0,
                           float* __restrict__ cb1, float* __restrict__ box, int32_t* __restrict__ left,
                           int32_t* __restrict__ right) {
    __shared__ uint32_t s_m, s_next, s_parity, s_rounds, s_stop, s_tile;
    __shared__ unsigned long long s_prefix;
    if (threadIdx.x == 0) {
        s_m = st->m; s_next = st->next; s_parity = st->parity; s_rounds = st->rounds; s_stop = st->stop;
        __threadfence();                         // the state is read before the ticket is taken
        s_tile = s_m <= s_stop ? 0xFFFFFFFFu : atomicAdd(ticket + (launch & 1u), 1u);
    }
    __syncthreads();
    const uint32_t m = s_m, tile = s_tile;
    const uint32_t ntiles = (m + kTile - 1) / kTile;
    if (m <= s_stop || tile >= ntiles) return;
    const bool p = s_parity != 0;
    const int32_t* cl = p ? cl1 : cl0;
    int32_t* clo = p ? cl0 : cl1;
    const float* cb = p ? cb1 : cb0;
    float* cbo = p ? cb0 : cb1;
    const uint32_t base = tile * kTile + threadIdx.x * kItems;
    uint32_t o[kItems], g[kItems];
    unsigned long long s = 0;
    for (int k = 0; k < kItems; ++k) {
        o[k] = g[k] = 0;
        if (base + k < m) ploc_flags(nn, base + k, o[k], g[k]);
        s += (unsigned long long)o[k] | ((unsigned long long)g[k] << 32);
    }
    unsigned long long tot;
    const unsigned long long ex = block_exclusive_scan<unsigned long long>(s, tot);
    if (threadIdx.x == 0) {
        const uint64_t tag = (uint64_t)(s_rounds & 63u) << 58;
        const uint64_t agg = (tot & 0xFFFFFFFFull) | ((tot >> 32) << 28);
        uint64_t prefix = 0;
        if (tile == 0) {
            look_store(look, tag | (2ull << 56) | agg);
        } else {
            look_store(look + tile, tag | (1ull << 56) | agg);
            bool ok = true;
            for (int k = (int)tile - 1; k >= 0;) {
                uint64_t w = 0;
                int spin = 0;
                for (; spin < kLookSpin; ++spin) {
                    w = look_load(look + k);
                    if ((w >> 58) == (tag >> 58) && ((w >> 56) & 3u) != 0) break;
                    if (spin > 64) __nanosleep(64);
                }
                if (spin == kLookSpin) { ok = false; break; }
                prefix += w & ((1ull << 56) - 1);
                if (((w >> 56) & 3u) == 2u) break;
                --k;
            }
            if (!ok) atomicOr(&st->error, DEV_GUARD);
            look_store(look + tile, tag | (2ull << 56) | ((prefix + agg) & ((1ull << 56) - 1)));
        }
        // back to the block's form: survivors in the low half, merges in the high half
        s_prefix = (prefix & kLookOut) | ((prefix >> 28) << 32);
        if (tile == ntiles - 1) {
            const uint64_t total = prefix + agg;
            const uint32_t m_next = (uint32_t)(total & kLookOut), merges = (uint32_t)(total >> 28);
            st->m_next = m_next;
            st->merges = merges;
            if (merges == 0) {
                atomicOr(&st->error, DEV_PLOC_NO_MERGE);
            } else {
                ticket[(launch + 1) & 1u] = 0;
                st->next = s_next + merges;
                st->m = m_next;
                st->parity = s_parity ^ 1u;
                st->rounds = s_rounds + 1;
            }
        }
    }
    __syncthreads();
    unsigned long long run = ex + s_prefix;
    const uint32_t next = s_next;
    for (int k = 0; k < kItems; ++k) {
        const uint32_t i = base + k;
        if (i < m && o[k]) {
            const uint32_t pos = (uint32_t)(run & 0xFFFFFFFFull);
            if (g[k]) {
                const uint32_t id = next + (uint32_t)(run >> 32);
                const int32_t j = nn[i];
                const float* A = cb + (size_t)i * 6;
                const float* B = cb + (size_t)j * 6;
                float nb6[6];
                for (int a = 0; a < 3; ++a) { nb6[a] = smin(A[a], B[a]); nb6[3 + a] = smax(A[3 + a], B[3 + a]); }
                for (int a = 0; a < 6; ++a) { box[(size_t)id * 6 + a] = nb6[a]; cbo[(size_t)pos * 6 + a] = nb6[a]; }
                left[id] = cl[i];
                right[id] = cl[j];
                clo[pos] = (int32_t)id;
            } else {
                for (int a = 0; a < 6; ++a) cbo[(size_t)pos * 6 + a] = cb[(size_t)i * 6 + a];
                clo[pos] = cl[i];
            }
        }
        run += (unsigned long long)o[k] | ((unsigned long long)g[k] << 32);
    }
}

// The remaining rounds in one block, once few clusters are left: the round's three steps
// (nearest neighbours, the flags' prefix sum, the scatter) are separated by block barriers
// instead of kernel launches, and the round state lives in shared memory. Each thread takes
// a contiguous run of positions, so the prefix sum runs in position order and node ids,
// cluster order and boxes are ploc_nn / ploc_scatter's exactly. At most max_rounds rounds
// (a bound, not a wait: every round either merges or sets DEV_PLOC_NO_MERGE and stops).
constexpr int kTailThreads = 1024;
__global__ void __launch_bounds__(kTailThreads) ploc_tail(RoundState* st, int32_t* __restrict__ cl0,
                                                          int32_t* __restrict__ cl1, float* __restrict__ cb0,
                                                          float* __restrict__ cb1, int32_t* __restrict__ nn,
                                                          float* __restrict__ box, int32_t* __restrict__ left,
                                                          int32_t* __restrict__ right, int R, uint32_t max_rounds,
                                                          uint32_t tail_max) {
    __shared__ uint32_t s_m, s_next, s_parity, s_rounds, s_error;
    __shared__ unsigned long long warp_tot[kTailThreads / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) { s_m = st->m; s_next = st->next; s_parity = st->parity; s_rounds = st->rounds; s_error = 0; }
    __syncthreads();
    // launched after every batch of rounds: nothing to do until the rounds reach the threshold
    if (s_m <= 1 || s_m > tail_max) return;
    for (uint32_t guard = 0; guard < max_rounds; ++guard) {
        const uint32_t m = s_m;
        if (m <= 1 || s_error) break;
        const bool p = s_parity != 0;
        const float* cb = p ? cb1 : cb0;
        float* cbo = p ? cb0 : cb1;
        const int32_t* cl = p ? cl1 : cl0;
        int32_t* clo = p ? cl0 : cl1;
        // nearest neighbours (ploc_nn_any)
        for (uint32_t i = tid; i < m; i += kTailThreads) {
            const float* A = cb + (size_t)i * 6;
            const int ii = (int)i;
            const int j0 = ii - R > 0 ? ii - R : 0, j1 = ii + R < (int)m - 1 ? ii + R : (int)m - 1;
            float best = FLT_MAX;
            int arg = -1;
            for (int j = j0; j <= j1; ++j) {
                if (j == ii) continue;
                const float* B = cb + (size_t)j * 6;
                const float d = ploc_area(smin(A[0], B[0]), smin(A[1], B[1]), smin(A[2], B[2]),
                                          smax(A[3], B[3]), smax(A[4], B[4]), smax(A[5], B[5]));
                if (d < best) { best = d; arg = j; }
            }
            nn[i] = arg;
        }
        __syncthreads();
        // flags of this thread's run of positions, then their prefix sum in position order
        const uint32_t chunk = (m + kTailThreads - 1) / kTailThreads;
        const uint32_t b0 = min(m, (uint32_t)tid * chunk), b1 = min(m, b0 + chunk);
        unsigned long long s = 0;
        for (uint32_t i = b0; i < b1; ++i) {
            uint32_t o, g;
            ploc_flags(nn, i, o, g);
            s += (unsigned long long)o | ((unsigned long long)g << 32);
        }
        unsigned long long x = s;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[warp] = x;
        __syncthreads();
        if (warp == 0) {
            unsigned long long w = warp_tot[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            warp_tot[lane] = w;
        }
        __syncthreads();
        const unsigned long long total = warp_tot[kTailThreads / 32 - 1];
        const uint32_t merges = (uint32_t)(total >> 32);
        if (merges == 0) {
            if (tid == 0) s_error = DEV_PLOC_NO_MERGE;
            __syncthreads();
            break;
        }
        unsigned long long run = (warp == 0 ? 0ull : warp_tot[warp - 1]) + x - s;
        const uint32_t next = s_next;
        for (uint32_t i = b0; i < b1; ++i) {
            uint32_t o, g;
            ploc_flags(nn, i, o, g);
            if (o) {
                const uint32_t pos = (uint32_t)(run & 0xFFFFFFFFull);
                if (g) {
                    const uint32_t id = next + (uint32_t)(run >> 32);
                    const int32_t j = nn[i];
                    const float* A = cb + (size_t)i * 6;
                    const float* B = cb + (size_t)j * 6;
                    float nb6[6];
                    for (int a = 0; a < 3; ++a) { nb6[a] = smin(A[a], B[a]); nb6[3 + a] = smax(A[3 + a], B[3 + a]); }
                    for (int a = 0; a < 6; ++a) { box[(size_t)id * 6 + a] = nb6[a]; cbo[(size_t)pos * 6 + a] = nb6[a]; }
                    left[id] = cl[i];
                    right[id] = cl[j];
                    clo[pos] = (int32_t)id;
                } else {
                    for (int a = 0; a < 6; ++a) cbo[(size_t)pos * 6 + a] = cb[(size_t)i * 6 + a];
                    clo[pos] = cl[i];
                }
            }
            run += (unsigned long long)o | ((unsigned long long)g << 32);
        }
        __syncthreads();
        if (tid == 0) {
            s_next = next + merges;
            s_m = (uint32_t)(total & 0xFFFFFFFFull);
            s_parity ^= 1u;
            s_rounds += 1;
        }
        __syncthreads();
    }
    if (tid == 0) {
        st->m = s_m; st->next = s_next; st->parity = s_parity; st->rounds = s_rounds;
        st->root = s_m == 1 ? (s_parity ? cl1 : cl0)[0] : -1;
        if (s_error) st->error |= s_error;
        else if (s_m > 1) st->error |= DEV_GUARD;
    }
}

// The remaining rounds in one thread-block cluster of C CTAs (C x 1024 threads on C SMs),
// for more clusters than one block takes well: ploc_tail's rounds with the steps separated by
// cluster barriers (barrier.cluster, release/acquire: each step's global writes are seen by
// every CTA of the cluster after it), the CTAs' flag totals exchanged through distributed
// shared memory, and the round state kept, identical, in every CTA's shared memory. Global
// thread g = rank x 1024 + tid takes a contiguous run of positions, so the prefix sum still
// runs in position order and node ids, cluster order and boxes are ploc_nn / ploc_scatter's
// exactly. Data another CTA wrote in this launch is read through L2 (ld.global.cg).
template <int C>
__global__ void __launch_bounds__(kTailThreads) ploc_tail_cluster(RoundState* st, int32_t* __restrict__ cl0,
                                                                  int32_t* __restrict__ cl1, float* __restrict__ cb0,
                                                                  float* __restrict__ cb1, int32_t* __restrict__ nn,
                                                                  float* __restrict__ box, int32_t* __restrict__ left,
                                                                  int32_t* __restrict__ right, int R,
                                                                  uint32_t max_rounds, uint32_t tail_max) {
    cg::cluster_group cluster = cg::this_cluster();
    __shared__ uint32_t s_m, s_next, s_parity, s_rounds, s_error;
    __shared__ unsigned long long warp_tot[kTailThreads / 32];
    __shared__ unsigned long long s_cta_tot;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t rank = cluster.block_rank();
    const uint32_t g = rank * kTailThreads + (uint32_t)tid, G = (uint32_t)C * kTailThreads;
    if (tid == 0) {
        s_m = __ldcg(&st->m); s_next = __ldcg(&st->next); s_parity = __ldcg(&st->parity);
        s_rounds = __ldcg(&st->rounds); s_error = 0;
    }
    __syncthreads();
    // launched after every batch of rounds: nothing to do until the rounds reach the threshold
    // (every CTA reads the same state, so all leave together, before any cluster barrier)
    if (s_m <= 1 || s_m > tail_max) return;
    for (uint32_t guard = 0; guard < max_rounds; ++guard) {
        const uint32_t m = s_m;
        if (m <= 1 || s_error) break;            // the same in every CTA
        const bool p = s_parity != 0;
        const float* cb = p ? cb1 : cb0;
        float* cbo = p ? cb0 : cb1;
        const int32_t* cl = p ? cl1 : cl0;
        int32_t* clo = p ? cl0 : cl1;
        // nearest neighbours (ploc_nn_any)
        for (uint32_t i = g; i < m; i += G) {
            const float* A = cb + (size_t)i * 6;
            const float a0 = __ldcg(A), a1 = __ldcg(A + 1), a2 = __ldcg(A + 2), a3 = __ldcg(A + 3), a4 = __ldcg(A + 4),
                        a5 = __ldcg(A + 5);
            const int ii = (int)i;
            const int j0 = ii - R > 0 ? ii - R : 0, j1 = ii + R < (int)m - 1 ? ii + R : (int)m - 1;
            float best = FLT_MAX;
            int arg = -1;
            for (int j = j0; j <= j1; ++j) {
                if (j == ii) continue;
                const float* B = cb + (size_t)j * 6;
                const float d = ploc_area(smin(a0, __ldcg(B)), smin(a1, __ldcg(B + 1)), smin(a2, __ldcg(B + 2)),
                                          smax(a3, __ldcg(B + 3)), smax(a4, __ldcg(B + 4)), smax(a5, __ldcg(B + 5)));
                if (d < best) { best = d; arg = j; }
            }
            nn[i] = arg;
        }
        cluster.sync();
        // flags of this thread's run of positions, then their prefix sum in position order:
        // within the CTA by warp shuffles, across the CTAs by their totals
        const uint32_t chunk = (m + G - 1) / G;
        const uint32_t b0 = min(m, g * chunk), b1 = min(m, b0 + chunk);
        unsigned long long s = 0;
        for (uint32_t i = b0; i < b1; ++i) {
            const int32_t j = __ldcg(nn + i);
            const bool mutual = j >= 0 && __ldcg(nn + j) == (int32_t)i;
            const uint32_t o = (!mutual || (int32_t)i < j) ? 1u : 0u, gm = (mutual && (int32_t)i < j) ? 1u : 0u;
            s += (unsigned long long)o | ((unsigned long long)gm << 32);
        }
        unsigned long long x = s;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[warp] = x;
        __syncthreads();
        if (warp == 0) {
            unsigned long long w = warp_tot[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            warp_tot[lane] = w;
            if (lane == 31) s_cta_tot = w;
        }
        cluster.sync();
        unsigned long long before = 0, total = 0;
        for (uint32_t r = 0; r < (uint32_t)C; ++r) {
            const unsigned long long v = *cluster.map_shared_rank(&s_cta_tot, r);
            if (r < rank) before += v;
            total += v;
        }
        const uint32_t merges = (uint32_t)(total >> 32);
        if (merges == 0) {
            if (tid == 0) s_error = DEV_PLOC_NO_MERGE;
            __syncthreads();
            break;
        }
        unsigned long long run = before + (warp == 0 ? 0ull : warp_tot[warp - 1]) + x - s;
        const uint32_t next = s_next;
        for (uint32_t i = b0; i < b1; ++i) {
            const int32_t j = __ldcg(nn + i);
            const bool mutual = j >= 0 && __ldcg(nn + j) == (int32_t)i;
            const uint32_t o = (!mutual || (int32_t)i < j) ? 1u : 0u, gm = (mutual && (int32_t)i < j) ? 1u : 0u;
            if (o) {
                const uint32_t pos = (uint32_t)(run & 0xFFFFFFFFull);
                if (gm) {
                    const uint32_t id = next + (uint32_t)(run >> 32);
                    const float* A = cb + (size_t)i * 6;
                    const float* B = cb + (size_t)j * 6;
                    float nb6[6];
                    for (int a = 0; a < 3; ++a) {
                        nb6[a] = smin(__ldcg(A + a), __ldcg(B + a));
                        nb6[3 + a] = smax(__ldcg(A + 3 + a), __ldcg(B + 3 + a));
                    }
                    for (int a = 0; a < 6; ++a) { box[(size_t)id * 6 + a] = nb6[a]; cbo[(size_t)pos * 6 + a] = nb6[a]; }
                    left[id] = __ldcg(cl + i);
                    right[id] = __ldcg(cl + j);
                    clo[pos] = (int32_t)id;
                } else {
                    for (int a = 0; a < 6; ++a) cbo[(size_t)pos * 6 + a] = __ldcg(cb + (size_t)i * 6 + a);
                    clo[pos] = __ldcg(cl + i);
                }
            }
            run += (unsigned long long)o | ((unsigned long long)gm << 32);
        }
        __syncthreads();
        if (tid == 0) {
            s_next = next + merges;
            s_m = (uint32_t)(total & 0xFFFFFFFFull);
            s_parity ^= 1u;
            s_rounds += 1;
        }
        cluster.sync();
    }
    cluster.sync();                              // no CTA leaves while another reads its shared memory
    if (rank == 0 && tid == 0) {
        st->m = s_m; st->next = s_next; st->parity = s_parity; st->rounds = s_rounds;
        st->root = s_m == 1 ? __ldcg((s_parity ? cl1 : cl0)) : -1;
        if (s_error) st->error |= s_error;
        else if (s_m > 1) st->error |= DEV_GUARD;
    }
}

template <int C>
cudaError_t launch_tail_cluster(cudaStream_t s, RoundState* st, int32_t* cl0, int32_t* cl1, float* cb0, float* cb1,
                                int32_t* nn, float* box, int32_t* left, int32_t* right, int R, uint32_t max_rounds,
                                uint32_t tail_max) {
    if (C > 8) {
        const cudaError_t e = cudaFuncSetAttribute(ploc_tail_cluster<C>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(kTailThreads);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, ploc_tail_cluster<C>, st, cl0, cl1, cb0, cb1, nn, box, left, right, R, max_rounds,
                              tail_max);
}

__global__ void ploc_commit(RoundState* st) {
    if (st->m <= st->stop || st->merges == 0) return;
    st->next += st->merges;
    st->m = st->m_next;
    st->parity ^= 1u;
    st->rounds += 1;
}

// ------------------------------------------------------------------ export
__global__ void export_nodes9(uint32_t count, const float* __restrict__ box, const int32_t* __restrict__ left,
                              const int32_t* __restrict__ right, const int32_t* __restrict__ tri,
                              int32_t* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    int32_t* o = out + (size_t)i * 9;
    o[0] = left[i]; o[1] = right[i]; o[2] = tri[i];
    for (int k = 0; k < 3; ++k) {
        o[3 + 2 * k] = __float_as_int(box[(size_t)i * 6 + k]);
        o[4 + 2 * k] = __float_as_int(box[(size_t)i * 6 + 3 + k]);
    }
}

// ------------------------------------------------------------------ collapse to 4-wide
__global__ void set_parents(uint32_t n, const int32_t* __restrict__ left, const int32_t* __restrict__ right,
                            int32_t* __restrict__ parent) {
    const uint32_t i = n + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * n - 1) return;
    parent[left[i]] = (int32_t)i;
    parent[right[i]] = (int32_t)i;
}
// Subtree leaf counts, bottom-up: the second child to arrive at a node computes it.
__global__ void subtree_counts(uint32_t n, const int32_t* __restrict__ left, const int32_t* __restrict__ right,
                               const int32_t* __restrict__ parent, uint32_t* __restrict__ visits,
                               uint32_t* count, uint32_t* err) {
    const uint32_t leaf = blockIdx.x * blockDim.x + threadIdx.x;
    if (leaf >= n) return;
    volatile uint32_t* vcount = count;
    vcount[leaf] = 1;
    int32_t c = (int32_t)leaf;
    for (uint32_t guard = 0; guard < 2 * n; ++guard) {
        const int32_t p = parent[c];
        if (p < 0) return;
        __threadfence();
        if (atomicAdd(&visits[p], 1u) == 0) return;   // the sibling is not done yet
        __threadfence();
        vcount[p] = vcount[left[p]] + vcount[right[p]];
        c = p;
    }
    atomicOr(err, DEV_GUARD);
}

struct Task { int32_t bnode, wnode; };

__device__ __forceinline__ float box_area(const float* b) {
    const float dx = b[3] - b[0], dy = b[4] - b[1], dz = b[5] - b[2];
    return dx * dy + dy * dz + dz * dx;
}
// Outward padding of a child box: the slab test must never cull a box whose triangle the
// watertight test accepts; 2^-19 of the coordinate plus 1e-6 of the extent covers the
// rounding of both tests with margin (the traversal also widens the slab exit, Ize 2013).
__device__ __forceinline__ void padded(const float* b, float* lo, float* hi) {
    for (int a = 0; a < 3; ++a) {
        const float ext = b[3 + a] - b[a];
        const float mag = fmaxf(fabsf(b[a]), fabsf(b[3 + a]));
        const float pad = ext * 1e-6f + mag * 1.9073486e-6f + 1e-30f;
        lo[a] = b[a] - pad;
        hi[a] = b[3 + a] + pad;
    }
}

// Reserve `n` consecutive slots of a global counter for each lane of the warp (every lane
// calls it; `am` is the full warp) with one atomic for the warp: returns the lane's first
// slot. The counters hand out node ids, queue positions and leaf
// triangle ranges; their order does not matter to any answer (the tree is the same), and
// one atomic per warp instead of one per child keeps a level of millions of tasks from
// queueing on three addresses.
__device__ __forceinline__ uint32_t warp_reserve(uint32_t* ctr, uint32_t n, unsigned am) {
    const int lane = threadIdx.x & 31;
    uint32_t incl = n;
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(am, incl, off);
        if (lane >= off) incl += y;
    }
    const int last = 31 - __clz(am);
    const uint32_t total = __shfl_sync(am, incl, last);
    uint32_t base = 0;
    if (lane == last && total) base = atomicAdd(ctr, total);
    base = __shfl_sync(am, base, last);
    return base + incl - n;
}

// One level's tasks in[0, m), strided: this thread's warp takes bases first, first + step, ...
// (first and step warp-uniform), so whole warps step together and every lane takes part in
// the reservations; lanes past the end reserve nothing. `in` and `out` carry no __restrict__:
// the single-block form reads in one level what it wrote in the previous one.
__device__ __forceinline__ void collapse_tasks(const Task* in, uint32_t m, uint32_t first, uint32_t step, Task* out,
                                               uint32_t* nout, uint32_t out_cap, uint32_t* node_ctr,
                                               uint32_t node_cap, uint32_t* tri_ctr,
                                               const float* __restrict__ box, const int32_t* __restrict__ left,
                                               const int32_t* __restrict__ right, const int32_t* __restrict__ tri,
                                               const uint32_t* __restrict__ count, const float* __restrict__ tris,
                                               Node4* __restrict__ nodes, LeafTri* __restrict__ leaf,
                                               uint32_t leaf_max, uint32_t* err) {
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t base = first; base < m; base += step) {
        const uint32_t t = base + lane;
        const bool valid = t < m;
        const Task task = valid ? in[t] : Task{0, 0};
        int32_t C[4];
        int nc = 0;
        const int32_t b = task.bnode;
        if (!valid) {
            nc = 0;
        } else if (tri[b] >= 0 || count[b] <= leaf_max) {
            C[nc++] = b;
        } else {
            C[nc++] = left[b];
            C[nc++] = right[b];
            while (nc < 4) {
                int pick = -1;
                float best = -1.0f;
                for (int k = 0; k < nc; ++k) {
                    const int32_t c = C[k];
                    if (tri[c] >= 0 || count[c] <= leaf_max) continue;
                    const float a = box_area(box + (size_t)c * 6);
                    if (a > best) { best = a; pick = k; }
                }
                if (pick < 0) break;
                const int32_t c = C[pick];
                C[pick] = left[c];
                C[nc++] = right[c];
            }
        }
        // this task's leaf triangles and interior children, reserved for the warp at once
        uint32_t ntri = 0, nint = 0;
        for (int k = 0; k < nc; ++k) {
            const int32_t c = C[k];
            if (tri[c] >= 0 || count[c] <= leaf_max) ntri += count[c];
            else ++nint;
        }
        uint32_t tri_next = warp_reserve(tri_ctr, ntri, 0xffffffffu);
        uint32_t id_next = warp_reserve(node_ctr, nint, 0xffffffffu);
        uint32_t q_next = warp_reserve(nout, nint, 0xffffffffu);
        if (!valid) continue;
        Node4 nd;
        for (int k = 0; k < 4; ++k) {
            nd.lox[k] = nd.loy[k] = nd.loz[k] = 1e30f;
            nd.hix[k] = nd.hiy[k] = nd.hiz[k] = -1e30f;
            nd.child[k] = 0;
            nd.meta[k] = 0;
        }
        nd.meta[0] = nc;
        for (int k = 0; k < nc; ++k) {
            const int32_t c = C[k];
            float lo[3], hi[3];
            padded(box + (size_t)c * 6, lo, hi);
            nd.lox[k] = lo[0]; nd.loy[k] = lo[1]; nd.loz[k] = lo[2];
            nd.hix[k] = hi[0]; nd.hiy[k] = hi[1]; nd.hiz[k] = hi[2];
            if (tri[c] >= 0 || count[c] <= leaf_max) {
                const uint32_t cnt = count[c];
                const uint32_t first = tri_next;
                tri_next += cnt;
                // the subtree's leaves, left to right
                int32_t stack[2 * kLeafCap];
                int sp = 0, w = 0;
                stack[sp++] = c;
                while (sp > 0) {
                    const int32_t x = stack[--sp];
                    if (tri[x] >= 0) {
                        const float* v = tris + (size_t)tri[x] * 9;
                        LeafTri lt;
                        lt.ax = v[0]; lt.ay = v[1]; lt.az = v[2]; lt.id = __int_as_float(tri[x]);
                        lt.bx = v[3]; lt.by = v[4]; lt.bz = v[5]; lt.pad0 = 0.0f;
                        lt.cx = v[6]; lt.cy = v[7]; lt.cz = v[8]; lt.pad1 = 0.0f;
                        leaf[first + w++] = lt;
                    } else if (sp + 2 <= 2 * kLeafCap) {
                        stack[sp++] = right[x];
                        stack[sp++] = left[x];
                    } else {
                        atomicOr(err, DEV_STACK_OVERFLOW);
                    }
                }
                nd.child[k] = ~(int32_t)((first << 3) | (cnt - 1));
            } else {
                const uint32_t id = id_next++;
                const uint32_t q = q_next++;
                if (id >= node_cap || q >= out_cap) { atomicOr(err, DEV_QUEUE_OVERFLOW); nd.child[k] = 0; continue; }
                out[q] = Task{c, (int32_t)id};
                nd.child[k] = (int32_t)id;
            }
        }
        nodes[task.wnode] = nd;
    }
}

// One level over the whole grid: a fixed grid strides over the level's tasks, whose count
// is read on the device.
__global__ void collapse_level(const Task* in, const uint32_t* __restrict__ nin, Task* out,
                               uint32_t* __restrict__ nout, uint32_t out_cap, uint32_t* __restrict__ node_ctr,
                               uint32_t node_cap, uint32_t* __restrict__ tri_ctr,
                               const float* __restrict__ box, const int32_t* __restrict__ left,
                               const int32_t* __restrict__ right, const int32_t* __restrict__ tri,
                               const uint32_t* __restrict__ count, const float* __restrict__ tris,
                               Node4* __restrict__ nodes, LeafTri* __restrict__ leaf, uint32_t leaf_max,
                               uint32_t* err) {
    collapse_tasks(in, *nin, blockIdx.x * blockDim.x + (threadIdx.x & ~31u), gridDim.x * blockDim.x, out, nout,
                   out_cap, node_ctr, node_cap, tri_ctr, box, left, right, tri, count, tris, nodes, leaf, leaf_max,
                   err);
}

// Between two levels: count the level just processed if it had tasks (ctr[5], the 4-wide
// depth), make its output the next input (ctr[0] = ctr[1]) and restart the output count.
__device__ __forceinline__ void collapse_advance(uint32_t* ctr) {
    if (ctr[0] > 0) ++ctr[5];
    ctr[0] = ctr[1];
    ctr[1] = 0;
}
__global__ void collapse_next(uint32_t* ctr) { collapse_advance(ctr); }

// The whole collapse in one block, for small trees: the levels are separated by block
// barriers instead of launches and host reads (the same tasks, reservations and nodes as
// collapse_level / collapse_next). At most max_levels levels (a bound: a level left over
// shows as a task count above zero, which the host reports).
constexpr int kCollapseThreads = 1024;
__global__ void __launch_bounds__(kCollapseThreads) collapse_block(Task* q0, Task* q1, uint32_t* ctr, uint32_t out_cap,
                                                                   uint32_t node_cap, const float* __restrict__ box,
                                                                   const int32_t* __restrict__ left,
                                                                   const int32_t* __restrict__ right,
                                                                   const int32_t* __restrict__ tri,
                                                                   const uint32_t* __restrict__ count,
                                                                   const float* __restrict__ tris,
                                                                   Node4* __restrict__ nodes, LeafTri* __restrict__ leaf,
                                                                   uint32_t leaf_max, uint32_t max_levels) {
    volatile uint32_t* vctr = ctr;
    for (uint32_t lv = 0; lv < max_levels; ++lv) {
        const uint32_t m = vctr[0];
        if (m == 0) break;                       // every thread read the same count after the barrier
        const Task* in = (lv & 1) ? q1 : q0;
        Task* out = (lv & 1) ? q0 : q1;
        collapse_tasks(in, m, threadIdx.x & ~31u, kCollapseThreads, out, ctr + 1, out_cap, ctr + 2, node_cap, ctr + 3,
                       box, left, right, tri, count, tris, nodes, leaf, leaf_max, ctr + 4);
        __syncthreads();
        if (threadIdx.x == 0) collapse_advance(ctr);
        __syncthreads();
    }
}

inline uint32_t cdiv(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

}  // namespace

// Exclusive prefix sum of n u32 values (three launches: block sums, one-block scan of the
// sums, block scans plus offsets); `total` (device) receives the sum when not null.
int scan_exclusive_u32(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* bsum, uint32_t* total,
                       cudaStream_t s) {
    const uint32_t nb = (n + kTile - 1) / kTile;
    if (nb == 0) return RN_OK;
    scan_reduce_u32<<<nb, kThreads, 0, s>>>(in, n, bsum);
    scan_top_u32<<<1, kThreads, 0, s>>>(bsum, nb, total);
    scan_down_u32<<<nb, kThreads, 0, s>>>(in, n, bsum, out);
    return RN_OK;
}

// ------------------------------------------------------------------ host drivers
int ploc_build(const float* d_tris, uint32_t n, int radius, PlocTree* out, cudaStream_t s, rn_status* st) {
    *out = PlocTree{};
    out->n = n;
    if (n == 0) return ok(st);
    if (radius < 1 || radius > 1024) return fail(st, RN_ERR_INVALID, "PLOC radius %d outside [1, 1024]", radius);
    const size_t N = 2 * (size_t)n - 1;
    const uint32_t nbs = cdiv(n, kTile);
    // one workspace block for everything the build needs (grow-only: repeated builds allocate
    // nothing; the tree's arrays live there until the next build)
    size_t off = 0;
    auto take = [&](size_t bytes) { const size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
    const size_t o_box = take(N * 6 * 4), o_left = take(N * 4), o_right = take(N * 4), o_tri = take(N * 4);
    const size_t o_cent = take((size_t)n * 12), o_k0 = take((size_t)n * 4), o_v0 = take((size_t)n * 4);
    const size_t o_k1 = take((size_t)n * 4), o_v1 = take((size_t)n * 4);
    const size_t o_hist = take((size_t)256 * nbs * 4), o_offs = take((size_t)256 * nbs * 4);
    const size_t o_bsum = take((size_t)(cdiv(256 * nbs, kTile) + 1) * 8);
    const size_t o_cl0 = take((size_t)n * 4), o_cl1 = take((size_t)n * 4);
    const size_t o_cb0 = take((size_t)n * 24), o_cb1 = take((size_t)n * 24);
    const size_t o_nn = take((size_t)n * 4), o_bs64 = take((size_t)(nbs + 1) * 8);
    const size_t o_look = take((size_t)(nbs + 1) * 8), o_ticket = take(8);
    const size_t o_bounds = take(sizeof(Bounds)), o_state = take(sizeof(RoundState));
    char* mem = nullptr;
    RN_TRY(ws_get(WS_PLOC, off, (void**)&mem, st));
    out->mem = mem;
    out->box = (float*)(mem + o_box);
    out->left = (int32_t*)(mem + o_left);
    out->right = (int32_t*)(mem + o_right);
    out->tri = (int32_t*)(mem + o_tri);
    float* cent = (float*)(mem + o_cent);
    uint32_t *k0 = (uint32_t*)(mem + o_k0), *v0 = (uint32_t*)(mem + o_v0);
    uint32_t *k1 = (uint32_t*)(mem + o_k1), *v1 = (uint32_t*)(mem + o_v1);
    uint32_t* hist = (uint32_t*)(mem + o_hist);
    uint32_t* offs = (uint32_t*)(mem + o_offs);
    uint32_t* bsum = (uint32_t*)(mem + o_bsum);
    int32_t *cl0 = (int32_t*)(mem + o_cl0), *cl1 = (int32_t*)(mem + o_cl1);
    float *cb0 = (float*)(mem + o_cb0), *cb1 = (float*)(mem + o_cb1);
    int32_t* nn = (int32_t*)(mem + o_nn);
    unsigned long long* bs64 = (unsigned long long*)(mem + o_bs64);
    unsigned long long* look = (unsigned long long*)(mem + o_look);
    uint32_t* ticket = (uint32_t*)(mem + o_ticket);
    Bounds* bounds = (Bounds*)(mem + o_bounds);
    RoundState* state = (RoundState*)(mem + o_state);

    // 1-2: centroids, bounds, codes
    init_bounds<<<1, 32, 0, s>>>(bounds);
    centroid_bounds<<<cdiv(n, 256), 256, 0, s>>>(d_tris, n, cent, bounds);
    morton_codes<<<cdiv(n, 256), 256, 0, s>>>(cent, n, bounds, k0, v0);
    // 3: four stable 8-bit passes over the 30-bit codes
    for (int pass = 0; pass < 4; ++pass) {
        const int shift = 8 * pass;
        rs_hist<<<nbs, kThreads, 0, s>>>(k0, n, shift, nbs, hist);
        scan_exclusive_u32(hist, offs, 256 * nbs, bsum, nullptr, s);
        rs_scatter<<<nbs, kThreads, 0, s>>>(k0, v0, n, shift, nbs, offs, k1, v1);
        std::swap(k0, k1);
        std::swap(v0, v1);
    }
    // 4: leaves
    make_leaves<<<cdiv(n, 256), 256, 0, s>>>(d_tris, v0, n, out->box, out->left, out->right, out->tri, cb0, cl0);
    if (n > 1) init_internal<<<cdiv(n - 1, 256), 256, 0, s>>>(n, out->box, out->left, out->right, out->tri);
    // 5: rounds, in batches; the host reads the state once per batch. With a tail threshold
    // the launched rounds stop at it (stop) and every batch ends with the tail kernel, which
    // runs the remaining rounds once the state is at or below the threshold and otherwise
    // leaves at once: the batch that reaches the threshold also finishes the tree.
    const uint32_t tail_max = (uint32_t)ctx().tune.ploc_tail;
    RoundState init{};
    init.m = n;
    init.next = n;
    init.root = -1;
    init.stop = tail_max > 1 ? tail_max : 1u;
    RN_CUDA(cudaMemcpyAsync(state, &init, sizeof init, cudaMemcpyHostToDevice, s), st);
    const bool fused = ctx().tune.ploc_fused != 0;
    if (fused) {
        // the look-back words of an earlier build must not pass for this one's
        RN_CUDA(cudaMemsetAsync(look, 0, (size_t)(nbs + 1) * 8, s), st);
        RN_CUDA(cudaMemsetAsync(ticket, 0, 8, s), st);
    }
    uint32_t merge_launch = 0;
    uint32_t m_known = n;
    RoundState hs = init;
    const int kBatch = 6;
    const int ctas = ctx().tune.ploc_tail_ctas;
    for (int batch = 0; m_known > 1; ++batch) {
        if (batch > 2000) return fail(st, RN_ERR_BUDGET, "PLOC: more than %d rounds", batch * kBatch);
        if (m_known > tail_max) {
            const uint32_t nbn = cdiv(m_known, kThreads), nbc = cdiv(m_known, kTile);
            for (int r = 0; r < kBatch; ++r) {
                if (radius == 16)
                    ploc_nn<16><<<nbn, kThreads, 0, s>>>(state, cb0, cb1, nn);
                else if (radius == 8)
                    ploc_nn<8><<<nbn, kThreads, 0, s>>>(state, cb0, cb1, nn);
                else if (radius == 32)
                    ploc_nn<32><<<nbn, kThreads, 0, s>>>(state, cb0, cb1, nn);
                else
                    ploc_nn_any<<<nbn, kThreads, 0, s>>>(state, cb0, cb1, nn, radius);
                if (fused) {
                    ploc_merge<<<nbc, kThreads, 0, s>>>(state, nn, look, ticket, merge_launch++, cl0, cl1, cb0, cb1,
                                                        out->box, out->left, out->right);
                    continue;
                }
                ploc_count<<<nbc, kThreads, 0, s>>>(state, nn, bs64);
                ploc_top<<<1, kThreads, 0, s>>>(state, bs64);
                ploc_scatter<<<nbc, kThreads, 0, s>>>(state, nn, bs64, cl0, cl1, cl0, cl1, cb0, cb1, cb0, cb1,
                                                      out->box, out->left, out->right);
                ploc_commit<<<1, 1, 0, s>>>(state);
            }
        }
        if (tail_max > 1) {
            // the last rounds in one block or one cluster of blocks (at most one round per
            // cluster: each merges one pair or more)
            const uint32_t rounds_max = tail_max + 1;
            cudaError_t le = cudaSuccess;
            if (ctas == 16)
                le = launch_tail_cluster<16>(s, state, cl0, cl1, cb0, cb1, nn, out->box, out->left, out->right, radius,
                                             rounds_max, tail_max);
            else if (ctas == 8)
                le = launch_tail_cluster<8>(s, state, cl0, cl1, cb0, cb1, nn, out->box, out->left, out->right, radius,
                                            rounds_max, tail_max);
            else if (ctas == 4)
                le = launch_tail_cluster<4>(s, state, cl0, cl1, cb0, cb1, nn, out->box, out->left, out->right, radius,
                                            rounds_max, tail_max);
            else
                ploc_tail<<<1, kTailThreads, 0, s>>>(state, cl0, cl1, cb0, cb1, nn, out->box, out->left, out->right,
                                                     radius, rounds_max, tail_max);
            RN_CUDA(le, st);
        }
        RN_CUDA(cudaGetLastError(), st);
        RN_CUDA(cudaMemcpyAsync(&hs, state, sizeof hs, cudaMemcpyDeviceToHost, s), st);
        RN_CUDA(cudaStreamSynchronize(s), st);
        if (hs.error & DEV_PLOC_NO_MERGE)
            return fail(st, RN_ERR_STATE, "PLOC round %u made no merge (%u clusters)", hs.rounds, hs.m);
        if (hs.error & DEV_GUARD) return fail(st, RN_ERR_BUDGET, "PLOC: rounds left %u clusters", hs.m);
        m_known = hs.m;
    }
    const int32_t tail_root = hs.root;
    if (hs.next != 2 * n - 1)
        return fail(st, RN_ERR_STATE, "PLOC made %u nodes, expected %u", hs.next, 2 * n - 1);
    int32_t root = tail_root;                // the tail kernels leave the root in the state
    if (root < 0 || n == 1) {
        RN_CUDA(cudaMemcpyAsync(&root, hs.parity ? cl1 : cl0, 4, cudaMemcpyDeviceToHost, s), st);
        RN_CUDA(cudaStreamSynchronize(s), st);
    }
    out->root = root;
    out->rounds = hs.rounds;
    return ok(st);
}

void ploc_free(PlocTree* t) { *t = PlocTree{}; }

int ploc_export(const PlocTree& t, int32_t* d_nodes9, cudaStream_t s, rn_status* st) {
    if (t.n == 0) return ok(st);
    const uint32_t N = 2 * t.n - 1;
    export_nodes9<<<cdiv(N, 256), 256, 0, s>>>(N, t.box, t.left, t.right, t.tri, d_nodes9);
    RN_CUDA(cudaGetLastError(), st);
    return ok(st);
}

int collapse_bvh4(const PlocTree& t, const float* d_tris, rn_accel* acc, int leaf_max, cudaStream_t s,
                  rn_status* st) {
    if (leaf_max < 1 || leaf_max > kLeafCap) return fail(st, RN_ERR_INVALID, "leaf size %d outside [1, %d]", leaf_max, kLeafCap);
    const uint32_t n = t.n;
    acc->ntri = n;
    acc->rounds = t.rounds;
    if (n == 0) return ok(st);
    const uint32_t N = 2 * n - 1;
    const uint32_t node_cap = n;              // every 4-wide node has at least 2 children
    // the accelerator's nodes and leaf triangles in one allocation (rn_accel_free frees d_nodes)
    const size_t node_bytes = ((size_t)node_cap * sizeof(Node4) + 255) & ~size_t(255);
    char* block = nullptr;
    RN_CUDA(cudaMallocFromPoolAsync((void**)&block, node_bytes + (size_t)n * sizeof(LeafTri), ctx().accel_pool, s), st);
    acc->d_nodes = (Node4*)block;
    acc->d_tris = (LeafTri*)(block + node_bytes);
    size_t off = 0;
    auto take = [&](size_t bytes) { const size_t o = off; off += (bytes + 255) & ~size_t(255); return o; };
    const size_t o_parent = take((size_t)N * 4), o_visits = take((size_t)N * 4), o_count = take((size_t)N * 4);
    const size_t o_q0 = take((size_t)n * sizeof(Task)), o_q1 = take((size_t)n * sizeof(Task));
    const size_t o_ctr = take(8 * 4);
    char* mem = nullptr;
    RN_TRY(ws_get(WS_COLLAPSE, off, (void**)&mem, st));
    int32_t* parent = (int32_t*)(mem + o_parent);
    uint32_t* visits = (uint32_t*)(mem + o_visits);
    uint32_t* count = (uint32_t*)(mem + o_count);
    Task* q0 = (Task*)(mem + o_q0);
    Task* q1 = (Task*)(mem + o_q1);
    uint32_t* ctr = (uint32_t*)(mem + o_ctr);   // [0] nin [1] nout [2] nodes [3] tris [4] err
    RN_CUDA(cudaMemsetAsync(parent, 0xFF, (size_t)N * 4, s), st);
    RN_CUDA(cudaMemsetAsync(visits, 0, (size_t)N * 4, s), st);
    RN_CUDA(cudaMemsetAsync(ctr, 0, 8 * 4, s), st);
    if (n > 1) set_parents<<<cdiv(n - 1, 256), 256, 0, s>>>(n, t.left, t.right, parent);
    subtree_counts<<<cdiv(n, 256), 256, 0, s>>>(n, t.left, t.right, parent, visits, count, ctr + 4);
    const Task root{t.root, 0};
    const uint32_t init[4] = {1u, 0u, 1u, 0u};
    RN_CUDA(cudaMemcpyAsync(q0, &root, sizeof root, cudaMemcpyHostToDevice, s), st);
    RN_CUDA(cudaMemcpyAsync(ctr, init, sizeof init, cudaMemcpyHostToDevice, s), st);
    // levels in batches of kLevels per host read; a level after the last one finds no task.
    // Small trees run every level in one block and are read once.
    constexpr int kLevels = 8;
    const uint32_t grid = std::max(1u, std::min(cdiv(n, 128), (uint32_t)ctx().sm_count * 16u));
    uint32_t level_tasks = 1, depth = 0;
    uint32_t hc[6] = {0, 0, 0, 0, 0, 0};
    if (n <= (uint32_t)ctx().tune.collapse_block) {
        collapse_block<<<1, kCollapseThreads, 0, s>>>(q0, q1, ctr, n, node_cap, t.box, t.left, t.right, t.tri, count,
                                                      d_tris, acc->d_nodes, acc->d_tris, (uint32_t)leaf_max, 4097u);
        RN_CUDA(cudaGetLastError(), st);
        RN_CUDA(cudaMemcpyAsync(hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, s), st);
        RN_CUDA(cudaStreamSynchronize(s), st);
        level_tasks = hc[0];
        depth = hc[5];
        if (level_tasks > 0) return fail(st, RN_ERR_BUDGET, "collapse: more than 4096 levels");
    }
    while (level_tasks > 0) {
        if (depth > 4096) return fail(st, RN_ERR_BUDGET, "collapse: more than 4096 levels");
        for (int k = 0; k < kLevels; ++k) {
            collapse_level<<<grid, 128, 0, s>>>(q0, ctr + 0, q1, ctr + 1, n, ctr + 2, node_cap, ctr + 3, t.box,
                                                t.left, t.right, t.tri, count, d_tris, acc->d_nodes, acc->d_tris,
                                                (uint32_t)leaf_max, ctr + 4);
            collapse_next<<<1, 1, 0, s>>>(ctr);
            std::swap(q0, q1);
        }
        RN_CUDA(cudaGetLastError(), st);
        RN_CUDA(cudaMemcpyAsync(hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, s), st);
        RN_CUDA(cudaStreamSynchronize(s), st);
        level_tasks = hc[0];
        depth = hc[5];
    }
    RN_CUDA(cudaGetLastError(), st);
    if (hc[4]) return fail(st, RN_ERR_OVERFLOW, "BVH collapse error word 0x%x", hc[4]);
    if (hc[3] != n) return fail(st, RN_ERR_STATE, "collapse placed %u of %u triangles", hc[3], n);
    acc->nodes = hc[2];
    acc->depth = depth;
    return ok(st);
}

}  // namespace rn
