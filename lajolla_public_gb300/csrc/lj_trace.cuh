// Ray traversal of the compressed 8-wide BVH: the GPU replacement of
// rtcIntersect1 / rtcOccluded1 (src/intersection.cpp:32, :83).
//
// Node groups follow the hit-mask scheme of Ylitie, Karras and Laine,
// "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs"
// (HPG 2017): a group is (base index, 32-bit mask); bits 24-31 mark hit
// internal children, placed at slot ^ (7 - ray octant) so that popping the
// highest bit first visits children roughly front to back; bits 0-23 mark
// hit leaf primitives (prim_base + bit).  Each node is five 128-bit loads.
//
// Primitive hits use the exact-rounding Moller-Trumbore test of
// lj_common.cuh (bit-identical to the CPU oracle) and, for spheres, the
// reference's user-geometry semantics (src/shapes/sphere.inl:40-106: nearest
// root in [tnear, tfar)).
#pragma once

#include "lj_common.cuh"
#include "lj_scene.cuh"

namespace lj {

struct TraceHit {
    float t;
    int prim;
    float u, v;
};

// Sphere, exact form: returns t in [tnear, tfar) of the nearest root, or -1,
// in FP64 exactly like the reference's user-geometry callback
// (src/shapes/sphere.inl:15-106: FP32 ray widened to FP64, the stable
// quadratic of solve_quadratic), with explicit round-to-nearest intrinsics
// so no contraction changes a rounding: t is bit-identical to the CPU
// oracle's.  FP64 is slow on this GPU; sphere_hit below takes this path only
// when its FP32 form cannot certify a decision.
LJ_D double ddot(double ax, double ay, double az, double bx, double by, double bz) {
    return __dadd_rn(__dadd_rn(__dmul_rn(ax, bx), __dmul_rn(ay, by)), __dmul_rn(az, bz));
}
LJ_D float sphere_hit_fp64(V3 c, float r, V3 o, V3 d, float tnear, float tfar) {
    double vx = __dsub_rn((double)o.x, (double)c.x), vy = __dsub_rn((double)o.y, (double)c.y),
           vz = __dsub_rn((double)o.z, (double)c.z);
    double dx = d.x, dy = d.y, dz = d.z, rr = r;
    double A = ddot(dx, dy, dz, dx, dy, dz);
    double B = __dmul_rn(2.0, ddot(dx, dy, dz, vx, vy, vz));
    double C = __dsub_rn(ddot(vx, vy, vz, vx, vy, vz), __dmul_rn(rr, rr));
    double t0, t1;
    if (A == 0.0) {
        if (B == 0.0) return -1.0f;
        t0 = t1 = __ddiv_rn(-C, B);
    } else {
        double disc = __dsub_rn(__dmul_rn(B, B), __dmul_rn(__dmul_rn(4.0, A), C));
        if (disc < 0.0) return -1.0f;
        double rd = __dsqrt_rn(disc);
        if (B >= 0.0) {
            t0 = __ddiv_rn(__dsub_rn(-B, rd), __dmul_rn(2.0, A));
            t1 = __ddiv_rn(__dmul_rn(2.0, C), __dsub_rn(-B, rd));
        } else {
            t0 = __ddiv_rn(__dmul_rn(2.0, C), __dadd_rn(-B, rd));
            t1 = __ddiv_rn(__dadd_rn(-B, rd), __dmul_rn(2.0, A));
        }
    }
    if (t0 > t1) { double tmp = t0; t0 = t1; t1 = tmp; }
    double tn = tnear, tf = tfar, t = -1.0;
    if (t0 >= tn && t0 < tf) t = t0;
    if (t1 >= tn && t1 < tf && t < 0.0) t = t1;
    return (t >= tn && t < tf) ? (float)t : -1.0f;
}

// Double-float (hi + lo pair of FP32) arithmetic for sphere_hit: the
// error-free transformations of Dekker / Knuth (two_sum, two_prod by FMA)
// with round-to-nearest intrinsics, so no contraction changes them.
struct F2 {
    float h, l;
};
LJ_D F2 two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return F2{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
LJ_D F2 fast_two_sum(float a, float b) {   // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return F2{s, __fsub_rn(b, __fsub_rn(s, a))};
}
LJ_D F2 two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return F2{p, __fmaf_rn(a, b, -p)};
}
LJ_D F2 df_add(F2 a, F2 b) {   // accurate sum (also under cancellation)
    F2 s = two_sum(a.h, b.h);
    const F2 t = two_sum(a.l, b.l);
    s = fast_two_sum(s.h, __fadd_rn(s.l, t.h));
    return fast_two_sum(s.h, __fadd_rn(s.l, t.l));
}
LJ_D F2 df_neg(F2 a) { return F2{-a.h, -a.l}; }
LJ_D F2 df_mul(F2 a, F2 b) {
    const F2 p = two_prod(a.h, b.h);
    return fast_two_sum(p.h, __fadd_rn(p.l, __fadd_rn(__fmul_rn(a.h, b.l), __fmul_rn(a.l, b.h))));
}

// Sphere, fast form: the same quadratic (halved: t = (-B' +- sqrt(B'^2 -
// A C)) / A with B' = d.v) with A, B', C and the discriminant in
// double-float (relative error ~2^-44 of the terms' magnitudes, far below
// the FP64 callback's own distance to any decision here) and the roots in
// FP32, each with a forward error bound taken well above the derived one.
// Hit / miss, the order of the roots and each root's comparison with tnear /
// tfar are decided here only when the bounds leave no doubt, and a returned
// t is within 6e-7 relative of the FP64 root; anything closer to a decision
// boundary (grazing rays, roots near tnear / tfar or each other) goes to
// sphere_hit_fp64.  So the hit / miss outcome is the FP64 callback's, and t
// agrees with it to 6e-7 relative (a triangle closer than that to the
// sphere along the ray may win where the FP64 t would lose).
LJ_D float sphere_hit(V3 c, float r, V3 o, V3 d, float tnear, float tfar) {
    constexpr float u = 5.9604645e-8f;         // 2^-24
    constexpr float kDiscRel = 3.6379788e-12f;  // 2^-38, derived bound ~30 u^2
    const F2 vx = two_sum(o.x, -c.x), vy = two_sum(o.y, -c.y), vz = two_sum(o.z, -c.z);   // exact
    const F2 A = df_add(df_add(two_prod(d.x, d.x), two_prod(d.y, d.y)), two_prod(d.z, d.z));
    const F2 Bh = df_add(df_add(df_add(two_prod(d.x, vx.h), two_prod(d.y, vy.h)), two_prod(d.z, vz.h)),
                         two_sum(__fmaf_rn(d.x, vx.l, __fmul_rn(d.y, vy.l)), __fmul_rn(d.z, vz.l)));
    const F2 V = df_add(df_add(df_add(two_prod(vx.h, vx.h), two_prod(vy.h, vy.h)), two_prod(vz.h, vz.h)),
                        two_sum(2.0f * __fmaf_rn(vx.h, vx.l, __fmaf_rn(vy.h, vy.l, __fmul_rn(vz.h, vz.l))), 0.0f));
    const F2 r2 = two_prod(r, r);
    const F2 C = df_add(V, df_neg(r2));
    const F2 disc = df_add(df_mul(Bh, Bh), df_neg(df_mul(A, C)));
    const float P = fabsf(d.x * vx.h) + fabsf(d.y * vy.h) + fabsf(d.z * vz.h);
    const float W = V.h + r2.h;
    const float M = P * P + A.h * W;
    const float e_disc = kDiscRel * M + 1e-30f;
    if (!(A.h > 0.0f) || !(M < 1e30f) || !(fabsf(disc.h) > 4.0f * e_disc) || !(tnear >= 0.0f))
        return sphere_hit_fp64(c, r, o, d, tnear, tfar);
    if (disc.h < 0.0f) return -1.0f;
    const float sq = sqrtf(disc.h);
    const float q = -(Bh.h + copysignf(sq, Bh.h));
    const float aq = fabsf(q);
    // relative error of a root: u (disc to FP32) / 2 + u (sqrt) + u (B' to
    // FP32, the sum) + u (A or C to FP32) + u (division), plus half the
    // double-float error of the discriminant; C's absolute double-float
    // error (~8 u^2 W) adds to the root C / q.  Bounds: 1.25x those.
    const float rel = 0.5f * (e_disc / disc.h) + 4.5f * u;
    const float ra = q / A.h, rc = C.h / q;
    const float ea = 1.25f * fabsf(ra) * rel;
    const float ec = 1.25f * (fabsf(rc) * rel + 16.0f * u * u * W / aq);
    float t0 = ra, e0 = ea, t1 = rc, e1 = ec;
    if (t0 > t1) {
        t0 = rc;
        e0 = ec;
        t1 = ra;
        e1 = ea;
    }
    if (!(t1 - t0 > e0 + e1)) return sphere_hit_fp64(c, r, o, d, tnear, tfar);
    // 1: in [tnear, tfar), 0: outside, -1: too close to tell
    auto in_range = [&](float t, float e) {
        if (t + e < tnear || t - e >= tfar) return 0;
        if (t - e >= tnear && t + e < tfar) return 1;
        return -1;
    };
    const int s0 = in_range(t0, e0);
    if (s0 == 1 && e0 <= 6e-7f * fabsf(t0)) return t0;
    if (s0 != 0) return sphere_hit_fp64(c, r, o, d, tnear, tfar);
    const int s1 = in_range(t1, e1);
    if (s1 == 1 && e1 <= 6e-7f * fabsf(t1)) return t1;
    if (s1 != 0) return sphere_hit_fp64(c, r, o, d, tnear, tfar);
    return -1.0f;
}

// Three-input min / max (one instruction each on this GPU); exact, like the
// nested fminf / fmaxf they replace, including the NaN rule (a NaN operand
// is ignored).
LJ_D float fmax3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
LJ_D float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
// Box slack of the traversal: a child box is entered when
// max(near planes, tnear) * (1 - 1e-6) <= min(far planes, tfar (1 + 1e-6)) *
// (1 + 1e-6), i.e. ~8 ulps either side, so hits on box faces and hits at
// exactly the current closest distance (ties) are never culled; applied as
// one factor, their quotient, on the near side.
constexpr float kBoxSlack = (1.0f - 1.0e-6f) / (1.0f + 1.0e-6f);

// Pairs of FP32 values in one 64-bit register pair, for the packed FP32
// instructions of this GPU (PTX add / fma .f32x2): each half is rounded
// exactly like the scalar instruction, two lanes of work per issue slot.
typedef unsigned long long f32x2;
LJ_D f32x2 pk2(float lo, float hi) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
LJ_D float2 upk2(f32x2 r) {
    float2 f;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(f.x), "=f"(f.y) : "l"(r));
    return f;
}
LJ_D f32x2 add2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
LJ_D f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// Byte i of w placed in the mantissa of 2^23 (bits 0x4B000000): the float
// 2^23 + byte, exactly, in one byte permute.
LJ_D float byte_biased(uint32_t w, int i) { return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + (uint32_t)i)); }
LJ_D uint32_t byte_of(uint32_t w, int i) { return __byte_perm(w, 0u, 0x4440u + (uint32_t)i); }

// Box test of the 8 children of one wide node (node words c0..c4) for one
// ray: returns the node's hit mask -- bits 24-31 the hit internal children
// at slot ^ (7 - octant), bits 0-23 the hit leaf primitives (prim_base +
// bit).  oct_inv4 is (7 - octant) in every byte; inv the reciprocal
// direction; tfar_s = tfar * (1 + 1e-6).
//
// Plane t = q * a + b with a = 2^e / d, b = (p - o) / d per axis (q the
// plane's byte).  kPacked: the x and y planes of one side (near or far)
// form one packed pair with the coefficient pairs (a_x, a_y), (b_x, b_y),
// so one packed add removes the 2^23 bias of both bytes and one packed FMA
// gives both t; z goes alone.  The packed form needs a few more live
// registers: it pays in the any-hit traversal, while the closest-hit one
// (more state per ray) spills with it and runs the scalar form.  Both give
// the same t, bit for bit.
// The mask bits follow Ylitie, Karras and Laine (HPG 2017): a child's meta
// byte is (unary prim count << 5) | offset for a leaf, (1 << 5) | (24 +
// slot) for an internal child; XOR-ing the offset of internal children
// with the octant gives the bit index of every child in one byte op per
// four children.  Empty slots have meta 0 and add no bit.
template <bool kPacked>
LJ_D uint32_t child_hits(uint4 c0, uint4 c1, uint4 c2, uint4 c3, uint4 c4, V3 o, V3 inv, uint32_t oct_inv4,
                         float tnear, float tfar_s) {
    const float px = __uint_as_float(c0.x), py = __uint_as_float(c0.y), pz = __uint_as_float(c0.z);
    const float sx = __uint_as_float((c0.w & 0xffu) << 23);
    const float sy = __uint_as_float(((c0.w >> 8) & 0xffu) << 23);
    const float sz = __uint_as_float(((c0.w >> 16) & 0xffu) << 23);
    const float ax = sx * inv.x, bx = (px - o.x) * inv.x;
    const float ay = sy * inv.y, by = (py - o.y) * inv.y;
    const float az = sz * inv.z, bz = (pz - o.z) * inv.z;
    const f32x2 AXY = pk2(ax, ay), BXY = pk2(bx, by);
    const f32x2 BIAS = pk2(-8388608.0f, -8388608.0f);
    // the words holding the near / far plane bytes of the 8 children, per
    // axis (lo planes are near for a positive direction component)
    const bool negx = inv.x < 0.0f, negy = inv.y < 0.0f, negz = inv.z < 0.0f;
    const uint32_t nx0 = negx ? c3.z : c2.x, nx1 = negx ? c3.w : c2.y;
    const uint32_t fx0 = negx ? c2.x : c3.z, fx1 = negx ? c2.y : c3.w;
    const uint32_t ny0 = negy ? c4.x : c2.z, ny1 = negy ? c4.y : c2.w;
    const uint32_t fy0 = negy ? c2.z : c4.x, fy1 = negy ? c2.w : c4.y;
    const uint32_t nz0 = negz ? c4.z : c3.x, nz1 = negz ? c4.w : c3.y;
    const uint32_t fz0 = negz ? c3.x : c4.z, fz1 = negz ? c3.y : c4.w;
    uint32_t hits = 0;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        // per four children: bit index and prim bits of each child's mask entry
        const uint32_t m = h == 0 ? c1.z : c1.w;
        const uint32_t inner7 = (((m & (m << 1)) >> 4) & 0x01010101u) * 7u;   // 7 in internal children's bytes
        const uint32_t bit4 = (m ^ (oct_inv4 & inner7)) & 0x1f1f1f1fu;
        const uint32_t cnt4 = (m >> 5) & 0x07070707u;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            float2 n, f;
            if (kPacked) {
                n = upk2(fma2(add2(pk2(byte_biased(h ? nx1 : nx0, k), byte_biased(h ? ny1 : ny0, k)), BIAS), AXY, BXY));
                f = upk2(fma2(add2(pk2(byte_biased(h ? fx1 : fx0, k), byte_biased(h ? fy1 : fy0, k)), BIAS), AXY, BXY));
            } else {
                n.x = fmaf(byte_biased(h ? nx1 : nx0, k) - 8388608.0f, ax, bx);
                n.y = fmaf(byte_biased(h ? ny1 : ny0, k) - 8388608.0f, ay, by);
                f.x = fmaf(byte_biased(h ? fx1 : fx0, k) - 8388608.0f, ax, bx);
                f.y = fmaf(byte_biased(h ? fy1 : fy0, k) - 8388608.0f, ay, by);
            }
            const float nz = fmaf(byte_biased(h ? nz1 : nz0, k) - 8388608.0f, az, bz);
            const float fz = fmaf(byte_biased(h ? fz1 : fz0, k) - 8388608.0f, az, bz);
            // slack of ~8 ulps (kBoxSlack): hits on box faces, and hits at
            // exactly the current closest distance (ties), are never culled
            const float tmin = fmaxf(fmax3(n.x, n.y, nz), tnear) * kBoxSlack;
            const float tmax = fmin3(f.x, f.y, fminf(fz, tfar_s));
            if (tmin <= tmax) hits |= byte_of(cnt4, k) << byte_of(bit4, k);
        }
    }
    return hits;
}

// Returns true on hit.  kAny: stop at the first hit (occlusion query).
// `hit` is updated with the closest hit; tfar shrinks as hits are found.
// *overflow is set if the traversal stack was exhausted (bounded loop).
// kCount: also count fetched nodes and tested primitives (instrumented
// variant used only for byte accounting).
template <bool kAny, bool kCount = false>
LJ_D bool trace_bvh(const DevBvh &bvh, V3 o, V3 d, float tnear, float tfar, TraceHit &hit,
                    int *overflow, uint32_t *n_nodes = nullptr, uint32_t *n_prims = nullptr) {
    if (bvh.num_nodes == 0) return false;
    // direction components of exactly zero would give inf * 0 in the slab test
    const float tiny = 1e-30f;
    V3 dd = V3{fabsf(d.x) < tiny ? copysignf(tiny, d.x) : d.x,
               fabsf(d.y) < tiny ? copysignf(tiny, d.y) : d.y,
               fabsf(d.z) < tiny ? copysignf(tiny, d.z) : d.z};
    // __frcp_rn: the correctly rounded reciprocal, the same bits as 1.0f / x
    V3 inv = V3{__frcp_rn(dd.x), __frcp_rn(dd.y), __frcp_rn(dd.z)};
    const uint32_t oct = (d.x < 0.0f ? 4u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 1u : 0u);
    const uint32_t oct_xor = 7u - oct;
    const uint32_t oct_inv4 = oct_xor * 0x01010101u;

    uint2 stack[kTraversalStack];
    int sp = 0;
    bool found = false;
    // virtual parent: one internal child in slot 0 pointing at node 0
    uint2 ngroup = make_uint2(0u, (1u << (24u + (0u ^ oct_xor))) | 1u);
    // every iteration visits one node or one primitive group; a well-formed
    // tree needs far fewer than this, a corrupt one stops here with a flag
    const int kMaxIterations = 1 << 22;
    for (int iter = 0;; iter++) {
        if (iter >= kMaxIterations) {
            *overflow = 1;
            break;
        }
        uint2 tgroup = make_uint2(0u, 0u);
        if (ngroup.y > 0x00ffffffu) {
            uint32_t k = 31u - __clz(ngroup.y & 0xff000000u);
            uint32_t slot = (k - 24u) ^ oct_xor;
            uint32_t imask = ngroup.y & 0xffu;
            uint32_t child = ngroup.x + __popc(imask & ((1u << slot) - 1u));
            ngroup.y &= ~(1u << k);
            if (ngroup.y > 0x00ffffffu) {
                if (sp < kTraversalStack) stack[sp++] = ngroup;
                else *overflow = 1;
            }
            if (kCount) (*n_nodes)++;
            const uint4 *np = bvh.nodes + (size_t)child * kWideNodeU4;
            uint4 c0 = __ldg(np + 0), c1 = __ldg(np + 1), c2 = __ldg(np + 2),
                  c3 = __ldg(np + 3), c4 = __ldg(np + 4);
            const uint32_t hm = child_hits<kAny>(c0, c1, c2, c3, c4, o, inv, oct_inv4, tnear, tfar * (1.0f + 1.0e-6f));
            ngroup = make_uint2(c1.x, (hm & 0xff000000u) | (c0.w >> 24));
            tgroup = make_uint2(c1.y, hm & 0x00ffffffu);
        } else {
            tgroup = ngroup;
            ngroup = make_uint2(0u, 0u);
        }
        while (tgroup.y != 0u) {
            int b = __ffs(tgroup.y) - 1;
            tgroup.y &= tgroup.y - 1u;
            if (kCount) (*n_prims)++;
            const float4 *pp = bvh.prims + (size_t)(tgroup.x + (uint32_t)b) * kPrimF4;
            float4 f0 = __ldg(pp + 0), f1 = __ldg(pp + 1);
            if (f1.w == 0.0f) {
                float4 f2 = __ldg(pp + 2);
                float t, u, v;
                const int prim = __float_as_int(f0.w);
                // equal distances go to the lower primitive index, so the
                // result does not depend on the traversal order
                if (tri_intersect(V3{f0.x, f0.y, f0.z}, V3{f1.x, f1.y, f1.z}, V3{f2.x, f2.y, f2.z}, o,
                                  d, tnear, tfar, t, u, v) &&
                    (t < tfar || (!kAny && found && prim < hit.prim))) {
                    found = true;
                    if (kAny) return true;
                    tfar = t;
                    hit.t = t;
                    hit.u = u;
                    hit.v = v;
                    hit.prim = prim;
                }
            } else {
                float t = sphere_hit(V3{f0.x, f0.y, f0.z}, f1.x, o, d, tnear, tfar);
                if (t >= 0.0f) {
                    found = true;
                    if (kAny) return true;
                    tfar = t;
                    hit.t = t;
                    hit.u = 0.0f;   // sphere uv is recomputed from the hit point
                    hit.v = 0.0f;
                    hit.prim = __float_as_int(f0.w);
                }
            }
        }
        if (ngroup.y <= 0x00ffffffu) {
            if (sp == 0) break;
            ngroup = stack[--sp];
        }
    }
    return found;
}

}  // namespace lj
