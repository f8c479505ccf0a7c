// Traversal of a whole ray queue by persistent warps with dynamic ray fetch
// (the "persistent while-while" scheme of Aila and Laine, "Understanding the
// Efficiency of Ray Traversal on GPUs", HPG 2009): each lane keeps its ray's
// traversal state in registers and steps it one node (plus the primitives
// that node yields) at a time; when fewer than kRefillLanes lanes of a warp
// still have a ray, the idle lanes take new rays from the queue (one atomic
// per warp) and the warp goes on.  Incoherent secondary rays differ widely
// in length, so this keeps far more lanes busy than one ray per lane per
// loop trip.  Per ray the node order, the tests and the tie rule are those
// of trace_bvh (lj_trace.cuh): results are identical.
#pragma once

#include "lj_internal.h"
#include "lj_trace.cuh"

namespace lj {

constexpr int kRefillLanes = 20;
constexpr int kSmemStack = 8;   // stack entries per thread kept in shared memory

// Traversal stack of one lane: the top kSmemStack entries in shared memory
// (entry k of thread t at column t of row k: consecutive lanes, consecutive
// words, no bank conflicts), deeper entries in local memory.
struct TravStack {
    uint2 *col;       // &smem[threadIdx.x]
    int stride;       // threads per block
    uint2 deep[kTraversalStack - kSmemStack];
    LJ_D void put(int k, uint2 v) {
        if (k < kSmemStack) col[k * stride] = v;
        else deep[k - kSmemStack] = v;
    }
    LJ_D uint2 get(int k) const { return k < kSmemStack ? col[k * stride] : deep[k - kSmemStack]; }
};

struct Trav {
    V3 o, d, inv;
    float tnear, tfar;
    uint32_t oct_xor;
    uint2 ngroup;
    // bits 0-7: stack entries in use; bits 8-31: steps taken (one register
    // for both: the traversal's live state is what limits its occupancy)
    int spi;
    const uint4 *nodes;
    const float4 *prims;
    // closest hit so far: its primitive (-1: none), barycentrics; its
    // distance is tfar (the search interval shrinks to it)
    int prim;
    float u, v;
    LJ_D bool found() const { return prim >= 0; }
};

LJ_D void trav_init(Trav &s, const DevBvh &bvh, V3 o, V3 d, float tnear, float tfar) {
    const float tiny = 1e-30f;
    V3 dd = V3{fabsf(d.x) < tiny ? copysignf(tiny, d.x) : d.x, fabsf(d.y) < tiny ? copysignf(tiny, d.y) : d.y,
               fabsf(d.z) < tiny ? copysignf(tiny, d.z) : d.z};
    s.o = o;
    s.d = d;
    s.inv = V3{__frcp_rn(dd.x), __frcp_rn(dd.y), __frcp_rn(dd.z)};   // = 1.0f / x, correctly rounded
    s.tnear = tnear;
    s.tfar = tfar;
    const uint32_t oct = (d.x < 0.0f ? 4u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 1u : 0u);
    s.oct_xor = 7u - oct;
    s.ngroup = bvh.num_nodes > 0 ? make_uint2(0u, (1u << (24u + (0u ^ s.oct_xor))) | 1u) : make_uint2(0u, 0u);
    s.spi = 0;
    s.nodes = bvh.nodes;
    s.prims = bvh.prims;
    s.prim = -1;
    s.u = 0.0f;
    s.v = 0.0f;
}

// One step: visit one node (or take the pending primitive group) and test
// the primitives it yields.  Returns true when the ray is finished.
// kPacked: the child box test's packed form (child_hits).
template <bool kAny, bool kPacked>
LJ_D bool trav_step(Trav &s, TravStack &stack, int *status) {
    s.spi += 256;
    if (s.spi > (1 << 30)) {   // 2^22 steps: a well-formed tree needs far fewer
        atomicOr(status, kStatusStackOverflow);
        return true;
    }
    uint2 tgroup = make_uint2(0u, 0u);
    if (s.ngroup.y > 0x00ffffffu) {
        const uint32_t k = 31u - __clz(s.ngroup.y & 0xff000000u);
        const uint32_t slot = (k - 24u) ^ s.oct_xor;
        const uint32_t imask = s.ngroup.y & 0xffu;
        const uint32_t child = s.ngroup.x + __popc(imask & ((1u << slot) - 1u));
        s.ngroup.y &= ~(1u << k);
        if (s.ngroup.y > 0x00ffffffu) {
            if ((s.spi & 0xff) < kTraversalStack) stack.put((s.spi++) & 0xff, s.ngroup);
            else atomicOr(status, kStatusStackOverflow);
        }
        const uint4 *np = s.nodes + (size_t)child * kWideNodeU4;
        const uint4 c0 = __ldg(np + 0), c1 = __ldg(np + 1), c2 = __ldg(np + 2), c3 = __ldg(np + 3),
                    c4 = __ldg(np + 4);
        const uint32_t hm = child_hits<kPacked>(c0, c1, c2, c3, c4, s.o, s.inv, s.oct_xor * 0x01010101u, s.tnear,
                                       s.tfar * (1.0f + 1.0e-6f));
        s.ngroup = make_uint2(c1.x, (hm & 0xff000000u) | (c0.w >> 24));
        tgroup = make_uint2(c1.y, hm & 0x00ffffffu);
    } else {
        tgroup = s.ngroup;
        s.ngroup = make_uint2(0u, 0u);
    }
    while (tgroup.y != 0u) {
        const int b = __ffs(tgroup.y) - 1;
        tgroup.y &= tgroup.y - 1u;
        const float4 *pp = s.prims + (size_t)(tgroup.x + (uint32_t)b) * kPrimF4;
        const float4 f0 = __ldg(pp + 0), f1 = __ldg(pp + 1);
        const int prim = __float_as_int(f0.w);
        if (f1.w == 0.0f) {
            const float4 f2 = __ldg(pp + 2);
            float t, u, v;
            // equal distances go to the lower primitive index (prim < s.prim
            // is false while there is no hit: s.prim is -1)
            if (tri_intersect(V3{f0.x, f0.y, f0.z}, V3{f1.x, f1.y, f1.z}, V3{f2.x, f2.y, f2.z}, s.o, s.d, s.tnear,
                              s.tfar, t, u, v) &&
                (t < s.tfar || (!kAny && prim < s.prim))) {
                s.prim = prim;
                if (kAny) return true;
                s.tfar = t;
                s.u = u;
                s.v = v;
            }
        } else {
            const float t = sphere_hit(V3{f0.x, f0.y, f0.z}, f1.x, s.o, s.d, s.tnear, s.tfar);
            if (t >= 0.0f) {
                s.prim = prim;
                if (kAny) return true;
                s.tfar = t;
                s.u = 0.0f;   // sphere uv is recomputed from the hit point
                s.v = 0.0f;
            }
        }
    }
    if (s.ngroup.y <= 0x00ffffffu) {
        if ((s.spi & 0xff) == 0) return true;
        s.ngroup = stack.get((--s.spi) & 0xff);
    }
    return false;
}

// Traces rays [0, n) of a queue.  IO supplies, per ray index r:
//   const DevBvh &bvh(int r)                  the BVH to trace against
//   void load(int r, V3 &o, V3 &d, float &tnear, float &tfar)
//   void store(int r, const Trav &s)          s.found(), s.prim / tfar / u / v hold the result
// *fetch must be 0 at launch; every warp of the grid must call this, with
// blockDim.x == kBlock.  kPacked selects the child box test's packed form:
// fastest where the kernel's registers allow it without spilling.
template <bool kAny, int kBlock, bool kPacked = true, class IO>
LJ_D void trace_queue(IO &io, int n, int *fetch, int *status) {
    const unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    __shared__ uint2 stack_top[kSmemStack * kBlock];
    TravStack stack;
    stack.col = stack_top + threadIdx.x;
    stack.stride = kBlock;
    Trav s;
    int ray = -1;
    bool drained = false;   // warp-uniform: the queue has no rays left
    for (;;) {
        if (!drained) {
            const unsigned want = __ballot_sync(kFull, ray < 0);
            if (want) {
                const int leader = __ffs(want) - 1;
                int base = 0;
                if (lane == leader) base = atomicAdd(fetch, __popc(want));
                base = __shfl_sync(kFull, base, leader);
                if (ray < 0) {
                    const int r = base + __popc(want & ((1u << lane) - 1u));
                    if (r < n) {
                        V3 o, d;
                        float tn, tf;
                        io.load(r, o, d, tn, tf);
                        trav_init(s, io.bvh(r), o, d, tn, tf);
                        ray = r;
                    }
                }
                drained = __any_sync(kFull, base + __popc(want) >= n);
            }
        }
        unsigned act = __ballot_sync(kFull, ray >= 0);
        if (act == 0) break;
        do {
            if (ray >= 0 && trav_step<kAny, kPacked>(s, stack, status)) {
                io.store(ray, s);
                ray = -1;
            }
            act = __ballot_sync(kFull, ray >= 0);
        } while (act != 0 && (drained || __popc(act) >= kRefillLanes));
    }
}

// Ray queue layouts of the wavefront: rays as two float4 (org|tnear,
// dir|tfar), hits as float4 (t, prim bits, u, v).
LJ_D void load_ray(const float4 *rays, int r, V3 &o, V3 &d, float &tn, float &tf) {
    const float4 r0 = rays[2 * r], r1 = rays[2 * r + 1];
    o = V3{r0.x, r0.y, r0.z};
    d = V3{r1.x, r1.y, r1.z};
    tn = r0.w;
    tf = r1.w;
}
LJ_D float4 hit_record(const Trav &s) {
    return s.found() ? make_float4(s.tfar, __int_as_float(s.prim), s.u, s.v)
                   : make_float4(0.0f, __int_as_float(-1), 0.0f, 0.0f);
}

// One scene: closest hits into a hit buffer.
struct ClosestQueueIO {
    DevBvh b;
    const float4 *rays;
    float4 *hits;
    LJ_D const DevBvh &bvh(int) const { return b; }
    LJ_D void load(int r, V3 &o, V3 &d, float &tn, float &tf) const { load_ray(rays, r, o, d, tn, tf); }
    LJ_D void store(int r, const Trav &s) const { hits[r] = hit_record(s); }
};

// One scene: shadow rays; an unoccluded ray adds its NEE contribution to its
// path's radiance -- at the path's entry of the next queue (target >= 0) or
// in the sample slot of a path that ended (~target).  One shadow ray per
// path per pass, so no two lanes write the same path.
struct ShadowQueueIO {
    DevBvh b;
    const float4 *rays;
    const int *targets;
    const float4 *contrib;
    float4 *Lnext;
    float4 *Lres;
    LJ_D const DevBvh &bvh(int) const { return b; }
    LJ_D void load(int r, V3 &o, V3 &d, float &tn, float &tf) const { load_ray(rays, r, o, d, tn, tf); }
    LJ_D void store(int r, const Trav &s) const {
        if (s.found()) return;
        const int t = targets[r];
        float4 *L = t >= 0 ? Lnext + t : Lres + ~t;
        const float4 c = contrib[r], l = *L;
        *L = make_float4(l.x + c.x, l.y + c.y, l.z + c.z, l.w);
    }
};

}  // namespace lj
