// GPU BVH build and batch ray casting: replaces the Embree scene build behind
// rtcCommitScene (src/scene.cpp:19-34, src/shapes/triangle_mesh.inl:1-22,
// src/shapes/sphere.inl:151-162) and the rtcIntersect1 / rtcOccluded1 calls
// (src/intersection.cpp:32, :83).
//
// Build pipeline (all on the device, one stream):
//   1. primitive boxes + centroids, scene box and centroid box (block reduce
//      + ordered-uint atomics)
//   2. 30-bit Morton codes of centroids over the centroid box
//   3. stable LSD radix sort of (code, primitive) -- 4 passes of 8 bits,
//      warp-match ranking, no library sort
//   4. binary tree by PLOC clustering over the Morton order (Meister and
//      Bittner 2018; below), or -- BvhInput::karras -- the Karras (HPG 2012)
//      radix tree with bottom-up boxes (atomic arrival counters)
//   5. level-synchronous collapse into the compressed 8-wide layout of
//      lj_scene.cuh: the SAH-optimal choice of which binary nodes become wide
//      nodes, leaves or are opened (Ylitie, Karras and Laine, HPG 2017,
//      section 3.1: bottom-up cost tables per PLOC round, then top-down
//      decisions; greedy largest-area child expansion for the Karras tree),
//      octant slot assignment, 8-bit conservative quantization, leaves of
//      <= 3 primitives stored contiguously in leaf order.
#include <cfloat>
#include <cmath>
#include <vector>

#include "lj_internal.h"
#include "lj_trace.cuh"
#include "lj_trace_queue.cuh"

namespace lj {

namespace {

constexpr int kRsThreads = kRadixThreads;
constexpr int kRsItems = kRadixItems;
constexpr int kRsTile = kRadixTile;

__device__ __forceinline__ uint32_t f2o(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}
__host__ __forceinline__ float o2f_host(uint32_t u) {
    uint32_t v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
    memcpy(&f, &v, 4);
    return f;
}

// Block-wide min/max of 6 values (3 mins, 3 maxes) -> ordered-uint atomics.
// blockDim.x must be a multiple of 32 and <= 1024.
__device__ void block_minmax6(float v[6], uint32_t *dst) {
    __shared__ float sh[32][6];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 6; k++) {
        for (int o = 16; o > 0; o >>= 1) {
            float x = __shfl_xor_sync(0xffffffffu, v[k], o);
            v[k] = k < 3 ? fminf(v[k], x) : fmaxf(v[k], x);
        }
    }
    if (lane == 0)
        for (int k = 0; k < 6; k++) sh[warp][k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        int nw = blockDim.x >> 5;
        for (int w = 1; w < nw; w++)
            for (int k = 0; k < 6; k++) v[k] = k < 3 ? fminf(v[k], sh[w][k]) : fmaxf(v[k], sh[w][k]);
        for (int k = 0; k < 3; k++) atomicMin(dst + k, f2o(v[k]));
        for (int k = 3; k < 6; k++) atomicMax(dst + k, f2o(v[k]));
    }
}

__global__ void k_init_bounds(uint32_t *b, int count) {
    int i = threadIdx.x;
    if (i < count) b[i] = (i % 6) < 3 ? f2o(FLT_MAX) : f2o(-FLT_MAX);
}

// bounds: [0..5] centroid min/max, [6..11] primitive box min/max
__global__ void k_prim_bounds(BvhInput in, float4 *plo, float4 *phi, float4 *cent, uint32_t *bounds) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int n = in.num_tris + in.num_spheres;
    float cb[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
    float bb[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
    if (i < n) {
        V3 l, h, c;
        if (i < in.num_tris) {
            int a = in.tri_vidx[i * 3], b = in.tri_vidx[i * 3 + 1], cc = in.tri_vidx[i * 3 + 2];
            V3 p0{in.vpos[a * 3], in.vpos[a * 3 + 1], in.vpos[a * 3 + 2]};
            V3 p1{in.vpos[b * 3], in.vpos[b * 3 + 1], in.vpos[b * 3 + 2]};
            V3 p2{in.vpos[cc * 3], in.vpos[cc * 3 + 1], in.vpos[cc * 3 + 2]};
            l = V3{fminf(p0.x, fminf(p1.x, p2.x)), fminf(p0.y, fminf(p1.y, p2.y)), fminf(p0.z, fminf(p1.z, p2.z))};
            h = V3{fmaxf(p0.x, fmaxf(p1.x, p2.x)), fmaxf(p0.y, fmaxf(p1.y, p2.y)), fmaxf(p0.z, fmaxf(p1.z, p2.z))};
            c = tri_centroid(p0, p1, p2);
        } else {
            const float *s = in.spheres + (size_t)(i - in.num_tris) * 4;
            c = V3{s[0], s[1], s[2]};
            float r = s[3];
            l = V3{__fsub_rn(c.x, r), __fsub_rn(c.y, r), __fsub_rn(c.z, r)};
            h = V3{__fadd_rn(c.x, r), __fadd_rn(c.y, r), __fadd_rn(c.z, r)};
        }
        plo[i] = make_float4(l.x, l.y, l.z, 0.f);
        phi[i] = make_float4(h.x, h.y, h.z, 0.f);
        cent[i] = make_float4(c.x, c.y, c.z, 0.f);
        cb[0] = cb[3] = c.x; cb[1] = cb[4] = c.y; cb[2] = cb[5] = c.z;
        bb[0] = l.x; bb[1] = l.y; bb[2] = l.z; bb[3] = h.x; bb[4] = h.y; bb[5] = h.z;
    }
    block_minmax6(cb, bounds);
    __syncthreads();
    block_minmax6(bb, bounds + 6);
}

__global__ void k_morton(const float4 *cent, int64_t n, const uint32_t *bounds, uint32_t *codes,
                         uint32_t *idx) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V3 lo{o2f(bounds[0]), o2f(bounds[1]), o2f(bounds[2])};
    V3 hi{o2f(bounds[3]), o2f(bounds[4]), o2f(bounds[5])};
    V3 sc{morton_scale(lo.x, hi.x), morton_scale(lo.y, hi.y), morton_scale(lo.z, hi.z)};
    float4 c = cent[i];
    codes[i] = morton3(V3{c.x, c.y, c.z}, lo, sc);
    if (idx) idx[i] = (uint32_t)i;
}

__global__ void k_tri_centroids(const float *v, int64_t n, float4 *cent, uint32_t *bounds) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float cb[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
    if (i < n) {
        const float *t = v + i * 9;
        V3 c = tri_centroid(V3{t[0], t[1], t[2]}, V3{t[3], t[4], t[5]}, V3{t[6], t[7], t[8]});
        cent[i] = make_float4(c.x, c.y, c.z, 0.f);
        cb[0] = cb[3] = c.x; cb[1] = cb[4] = c.y; cb[2] = cb[5] = c.z;
    }
    block_minmax6(cb, bounds);
}

// ---- radix sort ----------------------------------------------------------
__global__ void k_rs_hist(const uint32_t *keys, int64_t n, int shift, uint32_t *hist, int tiles) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    int64_t base = (int64_t)blockIdx.x * kRsTile;
#pragma unroll
    for (int k = 0; k < kRsItems; k++) {
        int64_t idx = base + k * kRsThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// single-block exclusive scan of `total` entries in place
__global__ void k_rs_scan(uint32_t *hist, int64_t total) {
    __shared__ uint32_t sums[1024];
    int t = threadIdx.x;
    int64_t chunk = (total + blockDim.x - 1) / blockDim.x;
    int64_t b = t * chunk, e = b + chunk < total ? b + chunk : total;
    uint32_t s = 0;
    for (int64_t i = b; i < e; i++) s += hist[i];
    sums[t] = s;
    __syncthreads();
    for (int off = 1; off < (int)blockDim.x; off <<= 1) {
        uint32_t v = t >= off ? sums[t - off] : 0u;
        __syncthreads();
        sums[t] += v;
        __syncthreads();
    }
    uint32_t run = sums[t] - s;
    for (int64_t i = b; i < e; i++) {
        uint32_t v = hist[i];
        hist[i] = run;
        run += v;
    }
}

__global__ void k_rs_scatter(const uint32_t *kin, const uint32_t *vin, uint32_t *kout, uint32_t *vout,
                             int64_t n, int shift, const uint32_t *hist, int tiles) {
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_wc[kRsThreads / 32][257];
    int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    s_base[tid] = hist[(size_t)tid * tiles + blockIdx.x];
    int64_t base = (int64_t)blockIdx.x * kRsTile;
    uint32_t lt_mask = (1u << lane) - 1u;
    for (int round = 0; round < kRsItems; round++) {
        for (int j = tid; j < (kRsThreads / 32) * 257; j += kRsThreads) (&s_wc[0][0])[j] = 0;
        __syncthreads();
        int64_t idx = base + round * kRsThreads + tid;
        bool valid = idx < n;
        uint32_t key = valid ? kin[idx] : 0u, val = valid ? vin[idx] : 0u;
        uint32_t d = valid ? (key >> shift) & 255u : 256u;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t rank = __popc(peers & lt_mask);
        if (valid && lane == __ffs(peers) - 1) s_wc[warp][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = s_base[tid];
            for (int w = 0; w < kRsThreads / 32; w++) {
                uint32_t c = s_wc[w][tid];
                s_wc[w][tid] = run;
                run += c;
            }
            s_base[tid] = run;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = s_wc[warp][d] + rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
    }
}

// ---- Karras radix tree ---------------------------------------------------
__device__ __forceinline__ int kdelta(const uint32_t *codes, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint32_t a = codes[i], b = codes[j];
    if (a != b) return __clz(a ^ b);
    return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

__global__ void k_karras(const uint32_t *codes, int n, int2 *child, int2 *range, int *parent_int,
                         int *parent_leaf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (kdelta(codes, n, i, i + 1) - kdelta(codes, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = kdelta(codes, n, i, i - d);
    int lmax = 2;
    while (kdelta(codes, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (kdelta(codes, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = kdelta(codes, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (kdelta(codes, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int gamma = i + s * d + min(d, 0);
    int first = min(i, j), last = max(i, j);
    int left = (first == gamma) ? ~gamma : gamma;
    int right = (last == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    child[i] = make_int2(left, right);
    range[i] = make_int2(first, last);
    if (left < 0) parent_leaf[gamma] = i; else parent_int[gamma] = i;
    if (right < 0) parent_leaf[gamma + 1] = i; else parent_int[gamma + 1] = i;
}

__global__ void k_bottom_up(int n, const int2 *child, const int *parent_int, const int *parent_leaf,
                            const uint32_t *sorted, const float4 *plo, const float4 *phi, float4 *nlo,
                            float4 *nhi, uint32_t *flags) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int p = parent_leaf[j];
    int guard = 0;
    while (p >= 0 && guard++ < 64 * 1024) {
        __threadfence();
        if (atomicAdd(&flags[p], 1u) == 0u) return;
        int2 c = child[p];
        float4 l0, h0, l1, h1;
        if (c.x < 0) { uint32_t g = sorted[~c.x]; l0 = plo[g]; h0 = phi[g]; }
        else { l0 = __ldcg(nlo + c.x); h0 = __ldcg(nhi + c.x); }
        if (c.y < 0) { uint32_t g = sorted[~c.y]; l1 = plo[g]; h1 = phi[g]; }
        else { l1 = __ldcg(nlo + c.y); h1 = __ldcg(nhi + c.y); }
        __stcg(nlo + p, make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), 0.f));
        __stcg(nhi + p, make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.f));
        p = parent_int[p];
    }
}

// ---- PLOC: parallel locally-ordered clustering ------------------------------
// Meister and Bittner, "Parallel Locally-Ordered Clustering for Bounding
// Volume Hierarchy Construction" (IEEE TVCG 2018).  Clusters start as the
// Morton-sorted primitives; each round every cluster finds, among the
// kPlocRadius clusters on either side in the current (Morton-ordered) array,
// the one whose union box has the least surface area (ties: lower index);
// mutual nearest neighbours merge into a new binary node, and the array is
// compacted in order.  The result is a binary tree of near-SAH quality, in
// the same child / range / box arrays the Karras tree fills, so the collapse
// below serves both; range holds (0, primitives - 1) here.
constexpr int kPlocRadius = 16;
constexpr int kPlocBlock = 256;

struct PlocClusters {
    int *id;          // binary node id, or ~sorted position for a primitive
    float4 *lo, *hi;
    int *cnt;         // primitives below
};

__device__ __forceinline__ float union_half_area(float4 l0, float4 h0, float4 l1, float4 h1) {
    float dx = fmaxf(h0.x, h1.x) - fminf(l0.x, l1.x);
    float dy = fmaxf(h0.y, h1.y) - fminf(l0.y, l1.y);
    float dz = fmaxf(h0.z, h1.z) - fminf(l0.z, l1.z);
    return dx * dy + dy * dz + dz * dx;
}

__global__ void k_ploc_init(const uint32_t *sorted, const float4 *plo, const float4 *phi, int n, PlocClusters c) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t g = sorted[i];
    c.id[i] = ~i;
    c.lo[i] = plo[g];
    c.hi[i] = phi[g];
    c.cnt[i] = 1;
}

__global__ void __launch_bounds__(kPlocBlock) k_ploc_nn(PlocClusters c, int count, int *nn) {
    __shared__ float4 slo[kPlocBlock + 2 * kPlocRadius], shi[kPlocBlock + 2 * kPlocRadius];
    const int base = blockIdx.x * kPlocBlock - kPlocRadius;
    for (int k = threadIdx.x; k < kPlocBlock + 2 * kPlocRadius; k += kPlocBlock) {
        int g = base + k;
        if (g >= 0 && g < count) {
            slo[k] = c.lo[g];
            shi[k] = c.hi[g];
        }
    }
    __syncthreads();
    const int i = blockIdx.x * kPlocBlock + threadIdx.x;
    if (i >= count) return;
    const float4 l = slo[i - base], h = shi[i - base];
    float best = __int_as_float(0x7f800000);
    int bj = -1;
    const int j0 = max(0, i - kPlocRadius), j1 = min(count - 1, i + kPlocRadius);
    for (int j = j0; j <= j1; j++) {
        if (j == i) continue;
        float cost = union_half_area(l, h, slo[j - base], shi[j - base]);
        if (cost < best) {   // ascending j: equal costs keep the lower index
            best = cost;
            bj = j;
        }
    }
    if (bj < 0) bj = i > 0 ? i - 1 : min(i + 1, count - 1);   // non-finite boxes: still progress
    nn[i] = bj;
}

// flags[i] = (keep, merge): i merges with its partner j > i; j disappears.
__global__ void k_ploc_flags(const int *nn, int count, int2 *flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    int j = nn[i];
    bool mutual = j != i && nn[j] == i;
    flags[i] = make_int2(mutual && j < i ? 0 : 1, mutual && i < j ? 1 : 0);
}

// Exclusive scan of int2 (two independent sums), 1024 elements per block.
constexpr int kScanBlock = 256, kScanItems = 4, kScanTile = kScanBlock * kScanItems;
__global__ void __launch_bounds__(kScanBlock) k_scan2_tiles(const int2 *in, int2 *out, int n, int2 *tile_sums) {
    __shared__ int2 warp_sums[kScanBlock / 32];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int2 v[kScanItems];
    int2 run = make_int2(0, 0);
    for (int k = 0; k < kScanItems; k++) {
        int2 x = base + k < n ? in[base + k] : make_int2(0, 0);
        v[k] = run;
        run.x += x.x;
        run.y += x.y;
    }
    // warp-inclusive scan of the thread totals
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int2 incl = run;
    for (int o = 1; o < 32; o <<= 1) {
        int ax = __shfl_up_sync(0xffffffffu, incl.x, o), ay = __shfl_up_sync(0xffffffffu, incl.y, o);
        if (lane >= o) {
            incl.x += ax;
            incl.y += ay;
        }
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    int2 woff = make_int2(0, 0);
    for (int w = 0; w < warp; w++) {
        woff.x += warp_sums[w].x;
        woff.y += warp_sums[w].y;
    }
    const int2 toff = make_int2(woff.x + incl.x - run.x, woff.y + incl.y - run.y);
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n) out[base + k] = make_int2(v[k].x + toff.x, v[k].y + toff.y);
    if (threadIdx.x == kScanBlock - 1) tile_sums[blockIdx.x] = make_int2(toff.x + run.x, toff.y + run.y);
}
// one block of 1024 threads: exclusive scan of the tile sums in place,
// total in sums[tiles]
__global__ void __launch_bounds__(1024) k_scan2_sums(int2 *sums, int tiles) {
    __shared__ int2 wsum[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int2 carry = make_int2(0, 0);
    for (int base = 0; base < tiles; base += 1024) {
        const int t = base + threadIdx.x;
        const int2 x = t < tiles ? sums[t] : make_int2(0, 0);
        int2 incl = x;
        for (int o = 1; o < 32; o <<= 1) {
            int ax = __shfl_up_sync(0xffffffffu, incl.x, o), ay = __shfl_up_sync(0xffffffffu, incl.y, o);
            if (lane >= o) {
                incl.x += ax;
                incl.y += ay;
            }
        }
        if (lane == 31) wsum[warp] = incl;
        __syncthreads();
        int2 woff = make_int2(0, 0);
        for (int w = 0; w < warp; w++) {
            woff.x += wsum[w].x;
            woff.y += wsum[w].y;
        }
        int2 total = make_int2(0, 0);
        for (int w = 0; w < 32; w++) {
            total.x += wsum[w].x;
            total.y += wsum[w].y;
        }
        if (t < tiles) sums[t] = make_int2(carry.x + woff.x + incl.x - x.x, carry.y + woff.y + incl.y - x.y);
        carry.x += total.x;
        carry.y += total.y;
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[tiles] = carry;
}
__global__ void k_scan2_add(int2 *out, int n, const int2 *tile_sums) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int2 o = tile_sums[i / kScanTile], v = out[i];
    out[i] = make_int2(v.x + o.x, v.y + o.y);
}

__global__ void k_ploc_compact(PlocClusters in, PlocClusters out, const int *nn, const int2 *flags,
                               const int2 *prefix, int count, int node_base, int2 *child, int2 *range,
                               float4 *nlo, float4 *nhi) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int2 f = flags[i];
    if (!f.x) return;
    const int dst = prefix[i].x;
    if (f.y) {
        const int j = nn[i];
        const int id = node_base - prefix[i].y;
        const float4 l0 = in.lo[i], h0 = in.hi[i], l1 = in.lo[j], h1 = in.hi[j];
        const float4 l = make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), 0.0f);
        const float4 h = make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.0f);
        const int cnt = in.cnt[i] + in.cnt[j];
        child[id] = make_int2(in.id[i], in.id[j]);
        range[id] = make_int2(0, cnt - 1);
        nlo[id] = l;
        nhi[id] = h;
        out.id[dst] = id;
        out.lo[dst] = l;
        out.hi[dst] = h;
        out.cnt[dst] = cnt;
    } else {
        out.id[dst] = in.id[i];
        out.lo[dst] = in.lo[i];
        out.hi[dst] = in.hi[i];
        out.cnt[dst] = in.cnt[i];
    }
}

// ---- collapse to the compressed 8-wide layout ----------------------------
// ---- SAH-optimal collapse: cost tables over the binary tree ---------------
// C(n, i) = the least SAH cost of the subtree of binary node n as at most i
// children of a wide node (i = 1..7):
//   C(n, 1) = min(leaf: A(n) p(n) c_prim if p(n) <= 3 primitives,
//                 internal: A(n) c_node + D(n, 8))
//   C(n, i) = min(C(n, i - 1), D(n, i)),
//   D(n, j) = min over 0 < k < j of C(left, k) + C(right, j - k),
// A = half the box surface, p = primitives below.  A primitive child is a
// one-primitive leaf at every i.  dec[8 n + i] records the choice: i = 1:
// 1 = leaf, 0 = a wide node of its own; i > 1: 0 = as with i - 1 children,
// else the left child's share k; dec[8 n] = the left child's share of the
// 8 children when n is a wide node.
// The costs: a primitive test costs the traversal about what a node visit
// does -- fewer instructions, but a warp runs its lanes' primitive loops
// while most lanes wait (measured: 2.7 loop iterations per step with 13 %
// of the lanes busy) -- so both weigh 1 (0.5 for a primitive built trees
// whose 1 M-triangle soup traced 6 % slower; 2 gained no more).
constexpr float kSahNode = 1.0f, kSahPrim = 1.0f;

__device__ __forceinline__ float box_half_area(float4 l, float4 h) {
    const float dx = h.x - l.x, dy = h.y - l.y, dz = h.z - l.z;
    return dx * dy + dy * dz + dz * dx;
}

// The cost table of binary node id, its children's tables complete.  Reads
// bypass L1 (the bottom-up walk reads what other SMs wrote).
__device__ void sah_table(float *cost, uint8_t *dec, const int2 *child, const int2 *range, const float4 *nlo,
                          const float4 *nhi, const uint32_t *sorted, const float4 *plo, const float4 *phi, int id) {
    const int2 c = __ldcg(child + id);
    float cl[8], cr[8];
    auto load = [&](int enc, float *cc) {
        if (enc < 0) {
            const uint32_t g = sorted[~enc];
            const float a = box_half_area(plo[g], phi[g]) * kSahPrim;
            for (int i = 1; i < 8; i++) cc[i] = a;
        } else {
            for (int i = 1; i < 8; i++) cc[i] = __ldcg(cost + (size_t)enc * 8 + i);
        }
    };
    load(c.x, cl);
    load(c.y, cr);
    float D[9];
    uint8_t K[9];
    for (int j = 2; j <= 8; j++) {
        float best = __int_as_float(0x7f800000);
        int bk = 1;
        for (int k = 1; k < j; k++) {
            const float v = cl[k] + cr[j - k];
            if (v < best) {
                best = v;
                bk = k;
            }
        }
        D[j] = best;
        K[j] = (uint8_t)bk;
    }
    const float A = box_half_area(__ldcg(nlo + id), __ldcg(nhi + id));
    const int2 rg = __ldcg(range + id);
    const int p = rg.y - rg.x + 1;
    const float c_int = A * kSahNode + D[8];
    const float c_leaf = p <= 3 ? A * (float)p * kSahPrim : __int_as_float(0x7f800000);
    float C = fminf(c_leaf, c_int);
    float *co = cost + (size_t)id * 8;
    uint8_t *de = dec + (size_t)id * 8;
    co[1] = C;
    de[1] = c_leaf <= c_int ? 1 : 0;
    for (int i = 2; i < 8; i++) {
        if (C <= D[i]) {
            de[i] = 0;
        } else {
            C = D[i];
            de[i] = K[i];
        }
        co[i] = C;
    }
    de[0] = K[8];
}

// Cost tables bottom-up: one thread per primitive walks towards the root;
// the second thread to reach a node (both subtrees done) fills its table.
__global__ void k_sah_costs_up(float *cost, uint8_t *dec, const int2 *child, const int2 *range, const float4 *nlo,
                               const float4 *nhi, const uint32_t *sorted, const float4 *plo, const float4 *phi,
                               const int *parent_int, const int *parent_leaf, int *visit, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int id = __ldcg(parent_leaf + i);
    while (id >= 0) {
        __threadfence();
        if (atomicAdd(visit + id, 1) == 0) return;
        __threadfence();
        sah_table(cost, dec, child, range, nlo, nhi, sorted, plo, phi, id);
        id = __ldcg(parent_int + id);
    }
}

// ---- treelet restructuring (Karras and Aila, "Fast Parallel Construction
// of High-Quality Bounding Volume Hierarchies", HPG 2013) ------------------
// Bottom-up over the binary tree; at a node with at least min_prims
// primitives below, the treelet of its kTreeletLeaves largest descendants
// (grown by opening the largest-area inner leaf until there are 7) is
// rebuilt with the topology of least SAH cost, found exactly by dynamic
// programming over the 127 subsets of its leaves; the treelet's inner node
// ids are reused.  Costs: binary SAH, kSahNode per node, kSahPrim per
// primitive, areas as half surface areas.
constexpr int kTreeletLeaves = 7;

struct TreeletArgs {
    int2 *child, *range;
    float4 *nlo, *nhi;
    float *sahc;            // binary SAH cost of each inner node's subtree
    int *parent_int, *parent_leaf, *visit;
    const uint32_t *sorted;
    const float4 *plo, *phi;
};

__device__ void treelet_leaf(const TreeletArgs &a, int enc, float4 &lo, float4 &hi, int &cnt, float &cost) {
    if (enc < 0) {
        const uint32_t g = a.sorted[~enc];
        lo = a.plo[g];
        hi = a.phi[g];
        cnt = 1;
        cost = box_half_area(lo, hi) * kSahPrim;
    } else {
        lo = __ldcg(a.nlo + enc);
        hi = __ldcg(a.nhi + enc);
        const int2 r = __ldcg(a.range + enc);
        cnt = r.y - r.x + 1;
        cost = __ldcg(a.sahc + enc);
    }
}

// Per-warp scratch of the subset DP (shared memory).
struct TreeletSmem {
    float area[1 << kTreeletLeaves];
    float cost[1 << kTreeletLeaves];
    uint8_t split[1 << kTreeletLeaves];
};

// The treelet at R, by the whole warp: every lane forms the treelet (same
// loads, uniform control flow), the lanes share the subsets' union areas
// and, size by size, their least costs; the full set's splits are spread
// over the lanes and reduced.  Lane 0 writes the new topology.
__device__ void treelet_at_warp(const TreeletArgs &a, int R, int min_prims, TreeletSmem &sm, int lane) {
    const unsigned kFull = 0xffffffffu;
    int leaf[kTreeletLeaves], inner[kTreeletLeaves - 1];
    float4 llo[kTreeletLeaves], lhi[kTreeletLeaves];
    int lcnt[kTreeletLeaves];
    float lcost[kTreeletLeaves];
    const int2 cR = __ldcg(a.child + R);
    leaf[0] = cR.x;
    leaf[1] = cR.y;
    treelet_leaf(a, leaf[0], llo[0], lhi[0], lcnt[0], lcost[0]);
    treelet_leaf(a, leaf[1], llo[1], lhi[1], lcnt[1], lcost[1]);
    const float AR = box_half_area(__ldcg(a.nlo + R), __ldcg(a.nhi + R));
    const float current = AR * kSahNode + lcost[0] + lcost[1];
    int nl = 2, nin = 1;
    inner[0] = R;
    if (lcnt[0] + lcnt[1] >= min_prims) {
        while (nl < kTreeletLeaves) {
            int best = -1;
            float ba = -1.0f;
            for (int k = 0; k < nl; k++) {
                if (leaf[k] < 0) continue;
                const float ar = box_half_area(llo[k], lhi[k]);
                if (ar > ba) { ba = ar; best = k; }
            }
            if (best < 0) break;
            const int e = leaf[best];
            inner[nin++] = e;
            const int2 c = __ldcg(a.child + e);
            leaf[best] = c.x;
            treelet_leaf(a, c.x, llo[best], lhi[best], lcnt[best], lcost[best]);
            leaf[nl] = c.y;
            treelet_leaf(a, c.y, llo[nl], lhi[nl], lcnt[nl], lcost[nl]);
            nl++;
        }
    }
    if (nl < 4) {   // two or three leaves: every topology is the same up to order
        if (lane == 0) __stcg(a.sahc + R, current);
        __syncwarp();
        return;
    }
    const int full = (1 << nl) - 1;
    // union areas, 4 subsets per lane
    for (int sset = lane + 1; sset <= full; sset += 32) {
        float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int k = 0; k < nl; k++) {
            if (!(sset & (1 << k))) continue;
            lo[0] = fminf(lo[0], llo[k].x); lo[1] = fminf(lo[1], llo[k].y); lo[2] = fminf(lo[2], llo[k].z);
            hi[0] = fmaxf(hi[0], lhi[k].x); hi[1] = fmaxf(hi[1], lhi[k].y); hi[2] = fmaxf(hi[2], lhi[k].z);
        }
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        sm.area[sset] = dx * dy + dy * dz + dz * dx;
        if (__popc(sset) == 1) sm.cost[sset] = lcost[__ffs(sset) - 1];
    }
    __syncwarp();
    // least costs of the proper subsets, size by size (each split {p, s ^ p}
    // once: p holds the lowest leaf of s)
    for (int size = 2; size < nl; size++) {
        for (int sset = lane + 1; sset < full; sset += 32) {
            if (__popc(sset) != size) continue;
            const int low = sset & -sset;
            float best = FLT_MAX;
            int bp = low;
            for (int p = (sset - 1) & sset; p > 0; p = (p - 1) & sset) {
                if (!(p & low)) continue;
                const float c = sm.cost[p] + sm.cost[sset ^ p];
                if (c < best) { best = c; bp = p; }
            }
            sm.cost[sset] = sm.area[sset] * kSahNode + best;
            sm.split[sset] = (uint8_t)bp;
        }
        __syncwarp();
    }
    // the full set: its 2^(nl-1) - 1 splits over the lanes, then the least
    // (ties to the larger split, the one the sequential order meets first)
    float best = FLT_MAX;
    int bp = 0;
    for (int j = lane; j < (1 << (nl - 1)) - 1; j += 32) {
        const int p = (j << 1) | 1;   // the splits holding leaf 0, j over the other leaves (not all of them)
        const float c = sm.cost[p] + sm.cost[full ^ p];
        if (c < best || (c == best && p > bp)) { best = c; bp = p; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(kFull, best, o);
        const int op = __shfl_xor_sync(kFull, bp, o);
        if (ob < best || (ob == best && op > bp)) { best = ob; bp = op; }
    }
    const float cfull = sm.area[full] * kSahNode + best;
    if (lane == 0) {
        sm.cost[full] = cfull;
        sm.split[full] = (uint8_t)bp;
    }
    __syncwarp();
    if (!(cfull < current * (1.0f - 1e-6f))) {
        if (lane == 0) __stcg(a.sahc + R, current);
        __syncwarp();
        return;
    }
    if (lane == 0) {
        // rebuild: each subset of two or more leaves becomes an inner node (the
        // full set keeps R); box, primitive count and cost follow from the subset
        int st[kTreeletLeaves], ids[kTreeletLeaves], sp = 0, next = 1;
        st[sp] = full;
        ids[sp++] = R;
        while (sp > 0) {
            --sp;
            const int sset = st[sp], id = ids[sp];
            int enc[2];
            const int part[2] = {sm.split[sset], sset ^ sm.split[sset]};
            for (int h = 0; h < 2; h++) {
                if (__popc(part[h]) == 1) {
                    enc[h] = leaf[__ffs(part[h]) - 1];
                } else {
                    enc[h] = inner[next++];
                    st[sp] = part[h];
                    ids[sp++] = enc[h];
                }
                if (enc[h] >= 0) __stcg(a.parent_int + enc[h], id);
                else __stcg(a.parent_leaf + ~enc[h], id);
            }
            float4 lo = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.0f),
                   hi = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.0f);
            int cnt = 0;
            for (int k = 0; k < nl; k++) {
                if (!(sset & (1 << k))) continue;
                lo.x = fminf(lo.x, llo[k].x); lo.y = fminf(lo.y, llo[k].y); lo.z = fminf(lo.z, llo[k].z);
                hi.x = fmaxf(hi.x, lhi[k].x); hi.y = fmaxf(hi.y, lhi[k].y); hi.z = fmaxf(hi.z, lhi[k].z);
                cnt += lcnt[k];
            }
            __stcg(a.child + id, make_int2(enc[0], enc[1]));
            __stcg(a.nlo + id, lo);
            __stcg(a.nhi + id, hi);
            __stcg(a.range + id, make_int2(0, cnt - 1));
            __stcg(a.sahc + id, sm.cost[sset]);
        }
    }
    __syncwarp();
}

// Bottom-up with whole warps: each lane walks from its primitive towards the
// root (the second lane to reach a node goes on); in each step the warp
// handles, one after another and all lanes together, the nodes its lanes
// reached.  Lanes that are done stay in the loop for the warp's work.
__global__ void __launch_bounds__(128) k_treelets(TreeletArgs a, int n, int min_prims) {
    __shared__ TreeletSmem smem[4];
    const unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    TreeletSmem &sm = smem[threadIdx.x >> 5];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int node = -1;
    bool alive = false;
    if (i < n) {
        node = __ldcg(a.parent_leaf + i);
        __threadfence();
        alive = node >= 0 && atomicAdd(a.visit + node, 1) != 0;
    }
    for (;;) {   // a step per tree level: alive lanes move up one node each step
        unsigned todo = __ballot_sync(kFull, alive);
        if (!todo) break;
        __threadfence();
        while (todo) {
            const int leader = __ffs(todo) - 1;
            todo &= todo - 1;
            const int R = __shfl_sync(kFull, node, leader);
            treelet_at_warp(a, R, min_prims, sm, lane);
        }
        if (alive) {
            const int p = __ldcg(a.parent_int + node);
            __threadfence();
            alive = p >= 0 && atomicAdd(a.visit + p, 1) != 0;
            node = p;
        }
    }
}

__global__ void k_parents(const int2 *child, int ni, int *parent_int, int *parent_leaf) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= ni) return;
    const int2 c = child[id];
    if (c.x >= 0) parent_int[c.x] = id; else parent_leaf[~c.x] = id;
    if (c.y >= 0) parent_int[c.y] = id; else parent_leaf[~c.y] = id;
}

struct CollapseArgs {
    const int2 *child;      // binary internal nodes
    const int2 *range;
    const float4 *nlo, *nhi;
    const uint32_t *sorted;   // sorted position -> global prim
    const float4 *plo, *phi;  // per global prim
    BvhInput in;
    uint4 *nodes;
    float4 *prims;
    int *node_counter, *prim_counter;
    const uint8_t *dec;     // SAH decisions (sah_table), or null: greedy expansion
    const int2 *qin;        // (binary node encoded, wide node index)
    const int *qin_count;
    int2 *qout;
    int *qout_count;
};

struct ChildInfo {
    int enc;            // >= 0 internal binary node, < 0 leaf (~sorted index)
    int first, count;
    float lo[3], hi[3];
};

__device__ void child_info(const CollapseArgs &a, int enc, ChildInfo &c) {
    c.enc = enc;
    float4 l, h;
    if (enc < 0) {
        int j = ~enc;
        uint32_t g = a.sorted[j];
        l = a.plo[g];
        h = a.phi[g];
        c.first = j;
        c.count = 1;
    } else {
        l = a.nlo[enc];
        h = a.nhi[enc];
        int2 r = a.range[enc];
        c.first = r.x;
        c.count = r.y - r.x + 1;
    }
    c.lo[0] = l.x; c.lo[1] = l.y; c.lo[2] = l.z;
    c.hi[0] = h.x; c.hi[1] = h.y; c.hi[2] = h.z;
}

__device__ float half_area(const ChildInfo &c) {
    float dx = c.hi[0] - c.lo[0], dy = c.hi[1] - c.lo[1], dz = c.hi[2] - c.lo[2];
    return dx * dy + dy * dz + dz * dx;
}

__device__ void write_prim(const CollapseArgs &a, int sorted_pos, int slot) {
    uint32_t g = a.sorted[sorted_pos];
    float4 *dst = a.prims + (size_t)slot * kPrimF4;
    if ((int)g < a.in.num_tris) {
        int i0 = a.in.tri_vidx[g * 3], i1 = a.in.tri_vidx[g * 3 + 1], i2 = a.in.tri_vidx[g * 3 + 2];
        V3 p0{a.in.vpos[i0 * 3], a.in.vpos[i0 * 3 + 1], a.in.vpos[i0 * 3 + 2]};
        V3 p1{a.in.vpos[i1 * 3], a.in.vpos[i1 * 3 + 1], a.in.vpos[i1 * 3 + 2]};
        V3 p2{a.in.vpos[i2 * 3], a.in.vpos[i2 * 3 + 1], a.in.vpos[i2 * 3 + 2]};
        V3 e1 = xsub(p1, p0), e2 = xsub(p2, p0);
        dst[0] = make_float4(p0.x, p0.y, p0.z, __int_as_float((int)g));
        dst[1] = make_float4(e1.x, e1.y, e1.z, 0.0f);
        dst[2] = make_float4(e2.x, e2.y, e2.z, 0.0f);
    } else {
        const float *s = a.in.spheres + (size_t)((int)g - a.in.num_tris) * 4;
        dst[0] = make_float4(s[0], s[1], s[2], __int_as_float((int)g));
        dst[1] = make_float4(s[3], 0.0f, 0.0f, 1.0f);
        dst[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

// Quantisation frame of a wide node over its box [lo, hi]: per axis a
// power-of-two step s (exponent e, stored biased by 127) with lo + 255 s >= hi.
__device__ void quant_frame(const float lo[3], const float hi[3], uint32_t ebits[3], float sc[3]) {
    for (int ax = 0; ax < 3; ax++) {
        float ext = hi[ax] - lo[ax];
        int e = ext > 0.0f ? (int)ceilf(log2f(ext / 255.0f)) : -126;
        e = max(-126, min(127, e));
        float s = ldexpf(1.0f, e);
        while (lo[ax] + 255.0f * s < hi[ax] && e < 127) { e++; s = ldexpf(1.0f, e); }
        ebits[ax] = (uint32_t)(e + 127);
        sc[ax] = s;
    }
}
// Conservative 8-bit planes of a child box [clo, chi] in that frame: the
// dequantised box always contains the child's.
__device__ void quant_child(const float clo[3], const float chi[3], const float lo[3], const float sc[3],
                            uint32_t ql_out[3], uint32_t qh_out[3]) {
    for (int ax = 0; ax < 3; ax++) {
        float fl = floorf((clo[ax] - lo[ax]) / sc[ax]);
        float fh = ceilf((chi[ax] - lo[ax]) / sc[ax]);
        int ql = (int)fmaxf(0.0f, fminf(255.0f, fl));
        int qh = (int)fmaxf(0.0f, fminf(255.0f, fh));
        while (ql > 0 && lo[ax] + (float)ql * sc[ax] > clo[ax]) ql--;
        while (qh < 255 && lo[ax] + (float)qh * sc[ax] < chi[ax]) qh++;
        if (qh <= ql) { if (qh < 255) qh = ql + 1; else ql = qh - 1; }
        ql_out[ax] = (uint32_t)ql;
        qh_out[ax] = (uint32_t)qh;
    }
}
__device__ uint32_t pack4(const uint32_t *b) { return b[0] | (b[1] << 8) | (b[2] << 16) | (b[3] << 24); }

__global__ void k_collapse(CollapseArgs a) {
    int item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= *a.qin_count) return;
    int2 q = a.qin[item];
    ChildInfo ch[8];
    bool inner[8];   // child k becomes a wide node of its own (else a leaf)
    int cnt = 0;
    if (q.x < 0) {
        child_info(a, q.x, ch[0]);
        cnt = 1;
    } else if (a.dec) {
        // the SAH decisions: 8 children shared between the two subtrees,
        // each share opened further or taken as fewer children
        int2 st_enc[16];   // (binary node encoded, children it may fill)
        int sp = 0;
        const int2 c = a.child[q.x];
        const int k8 = a.dec[(size_t)q.x * 8];
        st_enc[sp++] = make_int2(c.y, 8 - k8);
        st_enc[sp++] = make_int2(c.x, k8);
        while (sp > 0 && cnt < 8) {
            const int2 it = st_enc[--sp];
            if (it.x < 0 || it.y == 1) {
                child_info(a, it.x, ch[cnt]);
                inner[cnt] = it.x >= 0 && a.dec[(size_t)it.x * 8 + 1] == 0;
                cnt++;
                continue;
            }
            const int d = a.dec[(size_t)it.x * 8 + it.y];
            if (d == 0) {
                st_enc[sp++] = make_int2(it.x, it.y - 1);
            } else {
                const int2 cc = a.child[it.x];
                st_enc[sp++] = make_int2(cc.y, it.y - d);
                st_enc[sp++] = make_int2(cc.x, d);
            }
        }
    } else {
        int2 c = a.child[q.x];
        child_info(a, c.x, ch[0]);
        child_info(a, c.y, ch[1]);
        cnt = 2;
        // greedy expansion of the largest child that must stay internal
        while (cnt < 8) {
            int best = -1;
            float best_area = -1.0f;
            for (int k = 0; k < cnt; k++) {
                if (ch[k].enc >= 0 && ch[k].count > 3) {
                    float ar = half_area(ch[k]);
                    if (ar > best_area) { best_area = ar; best = k; }
                }
            }
            if (best < 0) break;
            int2 c2 = a.child[ch[best].enc];
            child_info(a, c2.y, ch[cnt]);
            child_info(a, c2.x, ch[best]);
            cnt++;
        }
    }
    if (!a.dec || q.x < 0)
        for (int k = 0; k < cnt; k++) inner[k] = ch[k].count > 3;
    // node box
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int k = 0; k < cnt; k++)
        for (int ax = 0; ax < 3; ax++) {
            lo[ax] = fminf(lo[ax], ch[k].lo[ax]);
            hi[ax] = fmaxf(hi[ax], ch[k].hi[ax]);
        }
    // octant slot assignment: slot s prefers children offset toward
    // (+x if s&4, +y if s&2, +z if s&1); greedy on the 8x8 cost table.
    float pc[3] = {(lo[0] + hi[0]) * 0.5f, (lo[1] + hi[1]) * 0.5f, (lo[2] + hi[2]) * 0.5f};
    int slot_of[8], child_in_slot[8];
    for (int k = 0; k < 8; k++) { slot_of[k] = -1; child_in_slot[k] = -1; }
    for (int round = 0; round < cnt; round++) {
        float best = FLT_MAX;
        int bc = -1, bs = -1;
        for (int k = 0; k < cnt; k++) {
            if (slot_of[k] >= 0) continue;
            float ox = (ch[k].lo[0] + ch[k].hi[0]) * 0.5f - pc[0];
            float oy = (ch[k].lo[1] + ch[k].hi[1]) * 0.5f - pc[1];
            float oz = (ch[k].lo[2] + ch[k].hi[2]) * 0.5f - pc[2];
            for (int s = 0; s < 8; s++) {
                if (child_in_slot[s] >= 0) continue;
                float cost = -((s & 4 ? ox : -ox) + (s & 2 ? oy : -oy) + (s & 1 ? oz : -oz));
                if (cost < best) { best = cost; bc = k; bs = s; }
            }
        }
        slot_of[bc] = bs;
        child_in_slot[bs] = bc;
    }
    int n_int = 0, n_prims = 0;
    for (int k = 0; k < cnt; k++) {
        if (inner[k]) n_int++;
        else n_prims += ch[k].count;
    }
    int child_base = n_int ? atomicAdd(a.node_counter, n_int) : 0;
    int prim_base = n_prims ? atomicAdd(a.prim_counter, n_prims) : 0;
    int qbase = n_int ? atomicAdd(a.qout_count, n_int) : 0;
    // quantization frame: per-axis power-of-two scale with 255 * s >= extent
    uint32_t ebits[3];
    float sc[3];
    quant_frame(lo, hi, ebits, sc);
    uint32_t meta[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint32_t qlo[3][8], qhi[3][8];
    uint32_t imask = 0;
    int int_rank = 0, prim_off = 0;
    for (int s = 0; s < 8; s++) {
        for (int ax = 0; ax < 3; ax++) { qlo[ax][s] = 0; qhi[ax][s] = 0; }
        int k = child_in_slot[s];
        if (k < 0) continue;
        const ChildInfo &c = ch[k];
        {
            uint32_t ql[3], qh[3];
            quant_child(c.lo, c.hi, lo, sc, ql, qh);
            for (int ax = 0; ax < 3; ax++) {
                qlo[ax][s] = ql[ax];
                qhi[ax][s] = qh[ax];
            }
        }
        if (inner[k]) {
            meta[s] = (1u << 5) | (24u + (uint32_t)s);
            imask |= 1u << s;
            int2 e = make_int2(c.enc, child_base + int_rank);
            a.qout[qbase + int_rank] = e;
            int_rank++;
        } else {
            uint32_t unary = c.count == 1 ? 1u : (c.count == 2 ? 3u : 7u);
            meta[s] = (unary << 5) | (uint32_t)prim_off;
            // the subtree's primitives, left to right (a walk of at most 2
            // internal nodes: Karras subtrees are contiguous, PLOC ones need not be)
            int todo[4], nt = 0, m = 0;
            todo[nt++] = c.enc;
            while (nt > 0 && m < c.count) {
                const int e = todo[--nt];
                if (e < 0) {
                    write_prim(a, ~e, prim_base + prim_off + m);
                    m++;
                } else if (nt + 2 <= 4) {
                    const int2 ce = a.child[e];
                    todo[nt++] = ce.y;
                    todo[nt++] = ce.x;
                }
            }
            prim_off += c.count;
        }
    }
    uint4 *dst = a.nodes + (size_t)q.y * kWideNodeU4;
    dst[0] = make_uint4(__float_as_uint(lo[0]), __float_as_uint(lo[1]), __float_as_uint(lo[2]),
                        ebits[0] | (ebits[1] << 8) | (ebits[2] << 16) | (imask << 24));
    dst[1] = make_uint4((uint32_t)child_base, (uint32_t)prim_base, pack4(meta), pack4(meta + 4));
    dst[2] = make_uint4(pack4(qlo[0]), pack4(qlo[0] + 4), pack4(qlo[1]), pack4(qlo[1] + 4));
    dst[3] = make_uint4(pack4(qlo[2]), pack4(qlo[2] + 4), pack4(qhi[0]), pack4(qhi[0] + 4));
    dst[4] = make_uint4(pack4(qhi[1]), pack4(qhi[1] + 4), pack4(qhi[2]), pack4(qhi[2] + 4));
}

// ---- refit: the tree keeps its topology, boxes follow moved vertices ----
// Leaf records of triangles rewritten from the vertex array (as write_prim
// does at build time); sphere records are unchanged.
__global__ void k_refit_prims(BvhInput in, float4 *prims, int n) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    float4 *dst = prims + (size_t)r * kPrimF4;
    const int g = __float_as_int(dst[0].w);
    if (g >= in.num_tris) return;
    const int i0 = in.tri_vidx[g * 3], i1 = in.tri_vidx[g * 3 + 1], i2 = in.tri_vidx[g * 3 + 2];
    V3 p0{in.vpos[i0 * 3], in.vpos[i0 * 3 + 1], in.vpos[i0 * 3 + 2]};
    V3 p1{in.vpos[i1 * 3], in.vpos[i1 * 3 + 1], in.vpos[i1 * 3 + 2]};
    V3 p2{in.vpos[i2 * 3], in.vpos[i2 * 3 + 1], in.vpos[i2 * 3 + 2]};
    V3 e1 = xsub(p1, p0), e2 = xsub(p2, p0);
    dst[0] = make_float4(p0.x, p0.y, p0.z, __int_as_float(g));
    dst[1] = make_float4(e1.x, e1.y, e1.z, 0.0f);
    dst[2] = make_float4(e2.x, e2.y, e2.z, 0.0f);
}

// Box of primitive g from the vertex array (triangles) or its record (spheres).
__device__ void prim_box(const BvhInput &in, const float4 *rec, int g, float lo[3], float hi[3]) {
    if (g < in.num_tris) {
        for (int k = 0; k < 3; k++) {
            const int v = in.tri_vidx[g * 3 + k];
            for (int ax = 0; ax < 3; ax++) {
                const float x = in.vpos[v * 3 + ax];
                lo[ax] = fminf(lo[ax], x);
                hi[ax] = fmaxf(hi[ax], x);
            }
        }
    } else {
        const float c[3] = {rec[0].x, rec[0].y, rec[0].z}, r = rec[1].x;
        for (int ax = 0; ax < 3; ax++) {
            lo[ax] = fminf(lo[ax], c[ax] - r);
            hi[ax] = fmaxf(hi[ax], c[ax] + r);
        }
    }
}

// One level of wide nodes [begin, end), children (deeper levels) done: each
// child's box (leaf primitives from the records, inner children from nbox),
// the node's new frame and planes; topology (child_base, prim_base, meta,
// slots) unchanged.  nbox[2 i], nbox[2 i + 1] = node i's lo, hi.
__global__ void k_refit_nodes(BvhInput in, uint4 *nodes, const float4 *prims, float4 *nbox, int begin, int end) {
    const int i = begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= end) return;
    uint4 *nd = nodes + (size_t)i * kWideNodeU4;
    const uint4 w0 = nd[0], w1 = nd[1];
    const uint32_t imask = w0.w >> 24;
    const uint32_t child_base = w1.x, prim_base = w1.y;
    float clo[8][3], chi[8][3];
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int s = 0; s < 8; s++) {
        const uint32_t meta = ((s < 4 ? w1.z : w1.w) >> (8 * (s & 3))) & 0xffu;
        for (int ax = 0; ax < 3; ax++) { clo[s][ax] = FLT_MAX; chi[s][ax] = -FLT_MAX; }
        if (meta == 0) continue;
        if (imask & (1u << s)) {
            const int c = (int)child_base + __popc(imask & ((1u << s) - 1u));
            const float4 a = nbox[2 * c], b = nbox[2 * c + 1];
            clo[s][0] = a.x; clo[s][1] = a.y; clo[s][2] = a.z;
            chi[s][0] = b.x; chi[s][1] = b.y; chi[s][2] = b.z;
        } else {
            const int count = __popc(meta >> 5), off = (int)(meta & 31u);
            for (int m = 0; m < count; m++) {
                const float4 *rec = prims + (size_t)(prim_base + off + m) * kPrimF4;
                prim_box(in, rec, __float_as_int(rec[0].w), clo[s], chi[s]);
            }
        }
        for (int ax = 0; ax < 3; ax++) {
            lo[ax] = fminf(lo[ax], clo[s][ax]);
            hi[ax] = fmaxf(hi[ax], chi[s][ax]);
        }
    }
    uint32_t ebits[3];
    float sc[3];
    quant_frame(lo, hi, ebits, sc);
    uint32_t qlo[3][8], qhi[3][8];
    for (int s = 0; s < 8; s++) {
        uint32_t ql[3] = {0, 0, 0}, qh[3] = {0, 0, 0};
        if (clo[s][0] <= chi[s][0]) quant_child(clo[s], chi[s], lo, sc, ql, qh);
        for (int ax = 0; ax < 3; ax++) {
            qlo[ax][s] = ql[ax];
            qhi[ax][s] = qh[ax];
        }
    }
    nd[0] = make_uint4(__float_as_uint(lo[0]), __float_as_uint(lo[1]), __float_as_uint(lo[2]),
                       ebits[0] | (ebits[1] << 8) | (ebits[2] << 16) | (imask << 24));
    nd[2] = make_uint4(pack4(qlo[0]), pack4(qlo[0] + 4), pack4(qlo[1]), pack4(qlo[1] + 4));
    nd[3] = make_uint4(pack4(qlo[2]), pack4(qlo[2] + 4), pack4(qhi[0]), pack4(qhi[0] + 4));
    nd[4] = make_uint4(pack4(qhi[1]), pack4(qhi[1] + 4), pack4(qhi[2]), pack4(qhi[2] + 4));
    nbox[2 * i] = make_float4(lo[0], lo[1], lo[2], 0.0f);
    nbox[2 * i + 1] = make_float4(hi[0], hi[1], hi[2], 0.0f);
}

__global__ void k_set_int(int *p, int v) { *p = v; }

// Batch ray casting: lj_ray / lj_hit have the wavefront queues' layout, so
// the persistent dynamic-fetch traversal of lj_trace_queue.cuh serves them.
struct AnyBatchIO {
    DevBvh b;
    const float4 *rays;
    uint8_t *occ;
    LJ_D const DevBvh &bvh(int) const { return b; }
    LJ_D void load(int r, V3 &o, V3 &d, float &tn, float &tf) const { load_ray(rays, r, o, d, tn, tf); }
    LJ_D void store(int r, const Trav &s) const { occ[r] = s.found() ? 1 : 0; }
};

__global__ void __launch_bounds__(128, 8) k_trace_closest(DevBvh bvh, const float4 *rays, float4 *hits, int n,
                                                          int *fetch, int *status) {
    ClosestQueueIO io{bvh, rays, hits};
    trace_queue<false, 128>(io, n, fetch, status);
}

__global__ void __launch_bounds__(128, 8) k_trace_any(DevBvh bvh, const float4 *rays, uint8_t *occ, int n,
                                                      int *fetch, int *status) {
    AnyBatchIO io{bvh, rays, occ};
    trace_queue<true, 128>(io, n, fetch, status);
}

// persistent grid of a traversal kernel on the current device
int batch_grid(const void *kernel) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0);
    return std::max(1, sms * std::max(1, per_sm));
}

template <bool kAny>
__global__ void k_trace_count(DevBvh bvh, const float4 *rays, int64_t n, unsigned long long *counts,
                              int *status) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t nn = 0, np = 0;
    if (i < n) {
        float4 r0 = rays[2 * i], r1 = rays[2 * i + 1];
        TraceHit h{0.0f, -1, 0.0f, 0.0f};
        int ovf = 0;
        trace_bvh<kAny, true>(bvh, V3{r0.x, r0.y, r0.z}, V3{r1.x, r1.y, r1.z}, r0.w, r1.w, h, &ovf, &nn, &np);
        if (ovf) atomicOr(status, kStatusStackOverflow);
    }
    for (int o = 16; o > 0; o >>= 1) {
        nn += __shfl_xor_sync(0xffffffffu, nn, o);
        np += __shfl_xor_sync(0xffffffffu, np, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(counts, (unsigned long long)nn);
        atomicAdd(counts + 1, (unsigned long long)np);
    }
}

template <bool kAny>
__global__ void k_trace_count_queue(DevBvh bvh, const float4 *rays, const int *count, int stride,
                                    unsigned long long *counts, int *status) {
    const int64_t n = *count;
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * stride;
    uint32_t nn = 0, np = 0, nr = 0;
    if (i < n) {
        float4 r0 = rays[2 * i], r1 = rays[2 * i + 1];
        TraceHit h{0.0f, -1, 0.0f, 0.0f};
        int ovf = 0;
        trace_bvh<kAny, true>(bvh, V3{r0.x, r0.y, r0.z}, V3{r1.x, r1.y, r1.z}, r0.w, r1.w, h, &ovf, &nn, &np);
        if (ovf) atomicOr(status, kStatusStackOverflow);
        nr = 1;
    }
    for (int o = 16; o > 0; o >>= 1) {
        nr += __shfl_xor_sync(0xffffffffu, nr, o);
        nn += __shfl_xor_sync(0xffffffffu, nn, o);
        np += __shfl_xor_sync(0xffffffffu, np, o);
    }
    if ((threadIdx.x & 31) == 0 && nr) {
        atomicAdd(counts, (unsigned long long)nr);
        atomicAdd(counts + 1, (unsigned long long)nn);
        atomicAdd(counts + 2, (unsigned long long)np);
    }
}

inline int grid_for(int64_t n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

int refit_bvh(const BvhInput &in, uint4 *nodes, float4 *prims, int num_prims, const std::vector<int> &level_start,
              float lo[3], float hi[3], cudaStream_t s, std::string *err) {
    if (num_prims <= 0 || level_start.size() < 2) return 0;
    const int num_nodes = level_start.back();
    k_refit_prims<<<grid_for(num_prims, 256), 256, 0, s>>>(in, prims, num_prims);
    float4 *nbox = nullptr;
    LJ_CUDA_TRY(cudaMallocAsync(&nbox, sizeof(float4) * 2 * (size_t)num_nodes, s));
    for (int l = (int)level_start.size() - 2; l >= 0; l--) {
        const int b = level_start[l], e = level_start[l + 1];
        k_refit_nodes<<<grid_for(e - b, 128), 128, 0, s>>>(in, nodes, prims, nbox, b, e);
    }
    float4 root[2];
    LJ_CUDA_TRY(cudaMemcpyAsync(root, nbox, sizeof(root), cudaMemcpyDeviceToHost, s));
    LJ_CUDA_TRY(cudaFreeAsync(nbox, s));
    LJ_CUDA_TRY(cudaStreamSynchronize(s));
    LJ_CUDA_TRY(cudaGetLastError());
    lo[0] = root[0].x; lo[1] = root[0].y; lo[2] = root[0].z;
    hi[0] = root[1].x; hi[1] = root[1].y; hi[2] = root[1].z;
    return 0;
}

int launch_trace_counters_queue(const DevBvh &bvh, const void *rays, const int *d_count, int64_t cap, int stride,
                                bool any, unsigned long long *d_counts, int *d_status, cudaStream_t s) {
    if (cap <= 0 || stride <= 0) return 0;
    const int g = grid_for((cap + stride - 1) / stride, 128);
    if (any) k_trace_count_queue<true><<<g, 128, 0, s>>>(bvh, (const float4 *)rays, d_count, stride, d_counts, d_status);
    else k_trace_count_queue<false><<<g, 128, 0, s>>>(bvh, (const float4 *)rays, d_count, stride, d_counts, d_status);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int launch_trace_counters(const DevBvh &bvh, const void *rays, int64_t n, bool any,
                          unsigned long long *d_counts, int *d_status, cudaStream_t s) {
    if (n <= 0) return 0;
    if (any) k_trace_count<true><<<grid_for(n, 128), 128, 0, s>>>(bvh, (const float4 *)rays, n, d_counts, d_status);
    else k_trace_count<false><<<grid_for(n, 128), 128, 0, s>>>(bvh, (const float4 *)rays, n, d_counts, d_status);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *tmp_keys, uint32_t *tmp_vals,
                     uint32_t *hist, int64_t n, cudaStream_t s, std::string *err) {
    if (n <= 1) return 0;
    int tiles = (int)((n + kRsTile - 1) / kRsTile);
    uint32_t *ki = keys, *vi = vals, *ko = tmp_keys, *vo = tmp_vals;
    for (int shift = 0; shift < 32; shift += 8) {
        k_rs_hist<<<tiles, kRsThreads, 0, s>>>(ki, n, shift, hist, tiles);
        k_rs_scan<<<1, 1024, 0, s>>>(hist, (int64_t)256 * tiles);
        k_rs_scatter<<<tiles, kRsThreads, 0, s>>>(ki, vi, ko, vo, n, shift, hist, tiles);
        std::swap(ki, ko);
        std::swap(vi, vo);
    }
    LJ_CUDA_TRY(cudaGetLastError());
    return 0;   // four passes: the result is back in keys / vals
}

int morton_codes_tris(const float *tri_vertices, int64_t n, uint32_t *codes, uint32_t *bounds,
                      cudaStream_t s, std::string *err) {
    float4 *cent = nullptr;
    LJ_CUDA_TRY(cudaMallocAsync(&cent, (size_t)n * sizeof(float4), s));
    k_init_bounds<<<1, 32, 0, s>>>(bounds, 6);
    k_tri_centroids<<<grid_for(n, 256), 256, 0, s>>>(tri_vertices, n, cent, bounds);
    k_morton<<<grid_for(n, 256), 256, 0, s>>>(cent, n, bounds, codes, nullptr);
    LJ_CUDA_TRY(cudaGetLastError());
    LJ_CUDA_TRY(cudaFreeAsync(cent, s));
    return 0;
}

int morton_codes_tris_into(const float *tri_vertices, int64_t n, uint32_t *codes, uint32_t *bounds,
                           float4 *cent, cudaStream_t s) {
    k_init_bounds<<<1, 32, 0, s>>>(bounds, 6);
    k_tri_centroids<<<grid_for(n, 256), 256, 0, s>>>(tri_vertices, n, cent, bounds);
    k_morton<<<grid_for(n, 256), 256, 0, s>>>(cent, n, bounds, codes, nullptr);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int build_bvh(const BvhInput &in, BvhOutput *out, cudaStream_t s, std::string *err) {
    const int n = in.num_tris + in.num_spheres;
    out->num_nodes = 0;
    out->num_binary = 0;
    if (n == 0) return 0;
    cudaEvent_t e0, e1;
    LJ_CUDA_TRY(cudaEventCreate(&e0));
    LJ_CUDA_TRY(cudaEventCreate(&e1));
    LJ_CUDA_TRY(cudaEventRecord(e0, s));

    // scratch (freed at the end of the build)
    float4 *plo, *phi, *cent, *nlo, *nhi;
    uint32_t *bounds, *codes, *idx, *tk, *tv, *hist, *flags;
    int2 *child, *range, *q0, *q1;
    int *parent_int, *parent_leaf, *counters;
    const int ni = n > 1 ? n - 1 : 1;
    size_t hist_n = radix_hist_entries(n);
    LJ_CUDA_TRY(cudaMallocAsync(&plo, sizeof(float4) * n, s));
    LJ_CUDA_TRY(cudaMallocAsync(&phi, sizeof(float4) * n, s));
    LJ_CUDA_TRY(cudaMallocAsync(&cent, sizeof(float4) * n, s));
    LJ_CUDA_TRY(cudaMallocAsync(&nlo, sizeof(float4) * ni, s));
    LJ_CUDA_TRY(cudaMallocAsync(&nhi, sizeof(float4) * ni, s));
    LJ_CUDA_TRY(cudaMallocAsync(&bounds, sizeof(uint32_t) * 16, s));
    LJ_CUDA_TRY(cudaMallocAsync(&codes, sizeof(uint32_t) * n, s));
    LJ_CUDA_TRY(cudaMallocAsync(&idx, sizeof(uint32_t) * n, s));
    LJ_CUDA_TRY(cudaMallocAsync(&tk, sizeof(uint32_t) * n, s));
    LJ_CUDA_TRY(cudaMallocAsync(&tv, sizeof(uint32_t) * n, s));
    LJ_CUDA_TRY(cudaMallocAsync(&hist, sizeof(uint32_t) * hist_n, s));
    LJ_CUDA_TRY(cudaMallocAsync(&flags, sizeof(uint32_t) * ni, s));
    LJ_CUDA_TRY(cudaMallocAsync(&child, sizeof(int2) * ni, s));
    LJ_CUDA_TRY(cudaMallocAsync(&range, sizeof(int2) * ni, s));
    LJ_CUDA_TRY(cudaMallocAsync(&q0, sizeof(int2) * n, s));
    LJ_CUDA_TRY(cudaMallocAsync(&q1, sizeof(int2) * n, s));
    LJ_CUDA_TRY(cudaMallocAsync(&parent_int, sizeof(int) * ni, s));
    LJ_CUDA_TRY(cudaMallocAsync(&parent_leaf, sizeof(int) * n, s));
    LJ_CUDA_TRY(cudaMallocAsync(&counters, sizeof(int) * 4, s));
    // outputs
    LJ_CUDA_TRY(cudaMalloc(&out->nodes, sizeof(uint4) * kWideNodeU4 * (size_t)ni));
    LJ_CUDA_TRY(cudaMalloc(&out->prims, sizeof(float4) * kPrimF4 * (size_t)n));

    float *sah_cost = nullptr;
    uint8_t *sah_dec = nullptr;
    k_init_bounds<<<1, 32, 0, s>>>(bounds, 12);
    k_prim_bounds<<<grid_for(n, 256), 256, 0, s>>>(in, plo, phi, cent, bounds);
    k_morton<<<grid_for(n, 256), 256, 0, s>>>(cent, n, bounds, codes, idx);
    if (radix_sort_pairs(codes, idx, tk, tv, hist, n, s, err)) return -2;
    LJ_CUDA_TRY(cudaMemsetAsync(parent_int, 0xff, sizeof(int) * ni, s));
    LJ_CUDA_TRY(cudaMemsetAsync(parent_leaf, 0xff, sizeof(int) * n, s));
    LJ_CUDA_TRY(cudaMemsetAsync(flags, 0, sizeof(uint32_t) * ni, s));
    if (n > 1 && !in.karras) {
        // PLOC rounds; each round reads its cluster count back (a few dozen rounds)
        PlocClusters cl[2];
        int *nn;
        int2 *pflags, *prefix, *tsums;
        const int tiles_max = (n + kScanTile - 1) / kScanTile;
        for (int k = 0; k < 2; k++) {
            LJ_CUDA_TRY(cudaMallocAsync(&cl[k].id, sizeof(int) * n, s));
            LJ_CUDA_TRY(cudaMallocAsync(&cl[k].lo, sizeof(float4) * n, s));
            LJ_CUDA_TRY(cudaMallocAsync(&cl[k].hi, sizeof(float4) * n, s));
            LJ_CUDA_TRY(cudaMallocAsync(&cl[k].cnt, sizeof(int) * n, s));
        }
        LJ_CUDA_TRY(cudaMallocAsync(&nn, sizeof(int) * n, s));
        LJ_CUDA_TRY(cudaMallocAsync(&pflags, sizeof(int2) * n, s));
        LJ_CUDA_TRY(cudaMallocAsync(&prefix, sizeof(int2) * n, s));
        LJ_CUDA_TRY(cudaMallocAsync(&tsums, sizeof(int2) * (tiles_max + 1), s));
        k_ploc_init<<<grid_for(n, 256), 256, 0, s>>>(idx, plo, phi, n, cl[0]);
        int count = n, merged = 0, c = 0;
        for (int round = 0; round < 1 << 16 && count > 1; round++) {
            const int tiles = (count + kScanTile - 1) / kScanTile;
            k_ploc_nn<<<grid_for(count, kPlocBlock), kPlocBlock, 0, s>>>(cl[c], count, nn);
            k_ploc_flags<<<grid_for(count, 256), 256, 0, s>>>(nn, count, pflags);
            k_scan2_tiles<<<tiles, kScanBlock, 0, s>>>(pflags, prefix, count, tsums);
            k_scan2_sums<<<1, 1024, 0, s>>>(tsums, tiles);
            k_scan2_add<<<grid_for(count, 256), 256, 0, s>>>(prefix, count, tsums);
            k_ploc_compact<<<grid_for(count, 256), 256, 0, s>>>(cl[c], cl[c ^ 1], nn, pflags, prefix, count,
                                                                 n - 2 - merged, child, range, nlo, nhi);
            int2 tot;
            LJ_CUDA_TRY(cudaMemcpyAsync(&tot, tsums + tiles, sizeof(int2), cudaMemcpyDeviceToHost, s));
            LJ_CUDA_TRY(cudaStreamSynchronize(s));
            if (tot.y <= 0) {
                if (err) *err = "BVH build: a clustering round merged nothing";
                return -5;
            }
            merged += tot.y;
            count = tot.x;
            c ^= 1;
        }
        for (int k = 0; k < 2; k++) {
            cudaFreeAsync(cl[k].id, s); cudaFreeAsync(cl[k].lo, s); cudaFreeAsync(cl[k].hi, s);
            cudaFreeAsync(cl[k].cnt, s);
        }
        cudaFreeAsync(nn, s); cudaFreeAsync(pflags, s); cudaFreeAsync(prefix, s); cudaFreeAsync(tsums, s);
        if (merged != n - 1) {
            if (err) *err = "BVH build: clustering left " + std::to_string(n - merged) + " roots";
            return -5;
        }
        // parent links (the root, node 0, keeps -1), then treelet passes
        // with a growing minimum subtree size (7, 14, 28 primitives)
        k_parents<<<grid_for(ni, 256), 256, 0, s>>>(child, ni, parent_int, parent_leaf);
        float *sahc = nullptr;
        int *visit = (int *)flags;
        LJ_CUDA_TRY(cudaMallocAsync(&sahc, sizeof(float) * (size_t)ni, s));
        TreeletArgs ta{child, range, nlo, nhi, sahc, parent_int, parent_leaf, visit, idx, plo, phi};
        for (int pass = 0; pass < in.treelet_passes; pass++) {
            LJ_CUDA_TRY(cudaMemsetAsync(visit, 0, sizeof(int) * ni, s));
            k_treelets<<<grid_for(n, 128), 128, 0, s>>>(ta, n, kTreeletLeaves << pass);
        }
        LJ_CUDA_TRY(cudaFreeAsync(sahc, s));
        // SAH cost tables of the 8-wide collapse, bottom-up
        LJ_CUDA_TRY(cudaMallocAsync(&sah_cost, sizeof(float) * 8 * (size_t)ni, s));
        LJ_CUDA_TRY(cudaMallocAsync(&sah_dec, sizeof(uint8_t) * 8 * (size_t)ni, s));
        LJ_CUDA_TRY(cudaMemsetAsync(visit, 0, sizeof(int) * ni, s));
        k_sah_costs_up<<<grid_for(n, 256), 256, 0, s>>>(sah_cost, sah_dec, child, range, nlo, nhi, idx, plo, phi,
                                                         parent_int, parent_leaf, visit, n);
        LJ_CUDA_TRY(cudaGetLastError());
    } else if (n > 1) {
        k_karras<<<grid_for(n - 1, 256), 256, 0, s>>>(codes, n, child, range, parent_int, parent_leaf);
        k_bottom_up<<<grid_for(n, 256), 256, 0, s>>>(n, child, parent_int, parent_leaf, idx, plo, phi,
                                                      nlo, nhi, flags);
    }
    // collapse, level by level
    int h_root[2] = {n > 1 ? 0 : ~0, 0};
    LJ_CUDA_TRY(cudaMemcpyAsync(q0, h_root, sizeof(int2), cudaMemcpyHostToDevice, s));
    int h_counters[4] = {1, 0, 1, 0};   // node counter, prim counter, qin count, qout count
    LJ_CUDA_TRY(cudaMemcpyAsync(counters, h_counters, sizeof(h_counters), cudaMemcpyHostToDevice, s));
    CollapseArgs a;
    a.child = child; a.range = range; a.nlo = nlo; a.nhi = nhi; a.sorted = idx;
    a.plo = plo; a.phi = phi; a.in = in; a.nodes = out->nodes; a.prims = out->prims;
    a.node_counter = counters; a.prim_counter = counters + 1;
    a.dec = sah_dec;
    int qcount = 1;
    int2 *qin = q0, *qout = q1;
    int *cin = counters + 2, *cout = counters + 3;
    // one launch per level; the launch for level L allocates all of level
    // L + 1's nodes, so every level is one contiguous index range
    out->level_start.assign({0, 1});
    for (int level = 0; level < 4096 && qcount > 0; level++) {
        k_set_int<<<1, 1, 0, s>>>(cout, 0);
        a.qin = qin; a.qin_count = cin; a.qout = qout; a.qout_count = cout;
        k_collapse<<<grid_for(qcount, 128), 128, 0, s>>>(a);
        int nodes_so_far = 0;
        LJ_CUDA_TRY(cudaMemcpyAsync(&qcount, cout, sizeof(int), cudaMemcpyDeviceToHost, s));
        LJ_CUDA_TRY(cudaMemcpyAsync(&nodes_so_far, counters, sizeof(int), cudaMemcpyDeviceToHost, s));
        LJ_CUDA_TRY(cudaStreamSynchronize(s));
        if (nodes_so_far > out->level_start.back()) out->level_start.push_back(nodes_so_far);
        std::swap(qin, qout);
        std::swap(cin, cout);
    }
    int h_final[2];
    LJ_CUDA_TRY(cudaMemcpyAsync(h_final, counters, sizeof(h_final), cudaMemcpyDeviceToHost, s));
    uint32_t hb[12];
    LJ_CUDA_TRY(cudaMemcpyAsync(hb, bounds, sizeof(hb), cudaMemcpyDeviceToHost, s));
    LJ_CUDA_TRY(cudaEventRecord(e1, s));
    LJ_CUDA_TRY(cudaStreamSynchronize(s));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    out->build_ms = ms;
    out->num_nodes = h_final[0];
    out->num_binary = n - 1;
    for (int k = 0; k < 3; k++) {
        out->lo[k] = o2f_host(hb[6 + k]);
        out->hi[k] = o2f_host(hb[9 + k]);
    }
    cudaFreeAsync(plo, s); cudaFreeAsync(phi, s); cudaFreeAsync(cent, s);
    cudaFreeAsync(nlo, s); cudaFreeAsync(nhi, s); cudaFreeAsync(bounds, s);
    cudaFreeAsync(codes, s); cudaFreeAsync(idx, s); cudaFreeAsync(tk, s); cudaFreeAsync(tv, s);
    cudaFreeAsync(hist, s); cudaFreeAsync(flags, s); cudaFreeAsync(child, s);
    cudaFreeAsync(range, s); cudaFreeAsync(q0, s); cudaFreeAsync(q1, s);
    cudaFreeAsync(parent_int, s); cudaFreeAsync(parent_leaf, s); cudaFreeAsync(counters, s);
    if (sah_cost) cudaFreeAsync(sah_cost, s);
    if (sah_dec) cudaFreeAsync(sah_dec, s);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (h_final[1] != n) {
        if (err) *err = "BVH collapse placed " + std::to_string(h_final[1]) + " of " + std::to_string(n) + " primitives";
        return -5;
    }
    LJ_CUDA_TRY(cudaGetLastError());
    return 0;
}

// Chunks of at most 2^30 rays; each launch gets a zeroed fetch counter of
// its own (stream-ordered allocation), so calls on different streams do not
// share one.
template <bool kAny>
int launch_trace_batch(const DevBvh &bvh, const void *rays, void *out, int64_t n, int *d_status, cudaStream_t s) {
    if (n <= 0) return 0;
    int *fetch = nullptr;
    if (cudaMallocAsync(&fetch, sizeof(int), s) != cudaSuccess) return -2;
    const int grid = batch_grid(kAny ? (const void *)k_trace_any : (const void *)k_trace_closest);
    const int64_t chunk = (int64_t)1 << 30;
    int rc = 0;
    for (int64_t off = 0; off < n && rc == 0; off += chunk) {
        const int m = (int)std::min(chunk, n - off);
        const float4 *r = (const float4 *)rays + 2 * off;
        if (cudaMemsetAsync(fetch, 0, sizeof(int), s) != cudaSuccess) rc = -2;
        if (kAny) k_trace_any<<<grid, 128, 0, s>>>(bvh, r, (uint8_t *)out + off, m, fetch, d_status);
        else k_trace_closest<<<grid, 128, 0, s>>>(bvh, r, (float4 *)out + off, m, fetch, d_status);
        if (cudaGetLastError() != cudaSuccess) rc = -2;
    }
    cudaFreeAsync(fetch, s);
    return rc;
}

int launch_trace_closest(const DevBvh &bvh, const void *rays, void *hits, int64_t n, int *d_status,
                         cudaStream_t s) {
    return launch_trace_batch<false>(bvh, rays, hits, n, d_status, s);
}

int launch_trace_any(const DevBvh &bvh, const void *rays, uint8_t *occ, int64_t n, int *d_status,
                     cudaStream_t s) {
    return launch_trace_batch<true>(bvh, rays, occ, n, d_status, s);
}

}  // namespace lj
