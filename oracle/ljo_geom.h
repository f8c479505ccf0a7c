// ORACLE / TEST INFRASTRUCTURE -- not part of the product.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may use anything
// under oracle/.
//
// FP32 ray/primitive tests and a CPU BVH shared by the Embree-API shim
// (embree_shim.cpp, which lets the reference renderer link without the
// missing libembree4.so.4) and the C++ restatement of the path (lj_oracle.cpp).
//
// The triangle test is the exact FP32 operation sequence the GPU kernels use
// (lajolla_public_gb300/csrc/lj_tri.cuh): Moller-Trumbore on precomputed
// edges, every dot/cross written with explicit fmaf so that the CPU and the
// GPU round identically.  Build this file with -ffp-contract=off so the
// compiler adds no contractions of its own.
//
// Hit convention (Embree's RTCHit, embree4/rtcore_ray.h:31-46):
//   p = (1-u-v) p0 + u p1 + v p2,  Ng = (p1-p0) x (p2-p0),
//   accepted iff tnear < t < tfar (strict on both ends).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace ljo {

struct f3 { float x, y, z; };

inline f3 f3_sub(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
// c = a x b, each component as fma(a_i, b_j, -(a_j * b_i)).
inline f3 f3_cross(f3 a, f3 b) {
    return f3{std::fmaf(a.y, b.z, -(a.z * b.y)),
              std::fmaf(a.z, b.x, -(a.x * b.z)),
              std::fmaf(a.x, b.y, -(a.y * b.x))};
}
// dot = fma(a.z, b.z, fma(a.y, b.y, a.x * b.x))
inline float f3_dot(f3 a, f3 b) {
    return std::fmaf(a.z, b.z, std::fmaf(a.y, b.y, a.x * b.x));
}

struct TriPre {  // per-triangle precomputation, identical on CPU and GPU
    f3 v0, e1, e2;
};

inline TriPre tri_pre(f3 p0, f3 p1, f3 p2) {
    return TriPre{p0, f3_sub(p1, p0), f3_sub(p2, p0)};
}

// Returns true and fills t,u,v if the ray hits the triangle in (tnear, tfar].
// Callers reject t == tfar unless it breaks a tie with the current closest
// hit in favour of the lower primitive index (the GPU traversal's rule), so
// equal distances resolve the same way whatever the traversal order.
inline bool tri_intersect(const TriPre &tri, f3 o, f3 d, float tnear, float tfar,
                          float &t_out, float &u_out, float &v_out) {
    f3 pvec = f3_cross(d, tri.e2);
    float det = f3_dot(tri.e1, pvec);
    if (det == 0.0f) return false;
    float inv_det = 1.0f / det;
    f3 tvec = f3_sub(o, tri.v0);
    float u = f3_dot(tvec, pvec) * inv_det;
    if (!(u >= 0.0f && u <= 1.0f)) return false;
    f3 qvec = f3_cross(tvec, tri.e1);
    float v = f3_dot(d, qvec) * inv_det;
    if (!(v >= 0.0f && u + v <= 1.0f)) return false;
    float t = f3_dot(tri.e2, qvec) * inv_det;
    if (!(t > tnear && t <= tfar)) return false;
    t_out = t; u_out = u; v_out = v;
    return true;
}

// 30-bit Morton code of a triangle centroid over the centroid AABB.
//   c = ((p0 + p1) + p2) * (1/3)   (FP32, that exact order)
//   q_i = clamp(floor((c_i - lo_i) * (1024 / (hi_i - lo_i))), 0, 1023)
//   (the scale is 0 on a degenerate axis)
// Bits interleaved x (bit 2), y (bit 1), z (bit 0) of each 3-bit group.
inline uint32_t expand_bits10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
inline f3 tri_centroid(f3 p0, f3 p1, f3 p2) {
    const float third = 1.0f / 3.0f;
    return f3{((p0.x + p1.x) + p2.x) * third, ((p0.y + p1.y) + p2.y) * third,
              ((p0.z + p1.z) + p2.z) * third};
}
inline uint32_t morton_quant(float c, float lo, float scale) {
    float q = (c - lo) * scale;
    q = std::floor(q);
    if (!(q >= 0.0f)) q = 0.0f;   // also maps NaN to 0
    if (q > 1023.0f) q = 1023.0f;
    return (uint32_t)q;
}
inline float morton_scale(float lo, float hi) {
    float ext = hi - lo;
    return ext > 0.0f ? 1024.0f / ext : 0.0f;
}
inline uint32_t morton3(f3 c, f3 lo, f3 scale) {
    uint32_t x = morton_quant(c.x, lo.x, scale.x);
    uint32_t y = morton_quant(c.y, lo.y, scale.y);
    uint32_t z = morton_quant(c.z, lo.z, scale.z);
    return (expand_bits10(x) << 2) | (expand_bits10(y) << 1) | expand_bits10(z);
}

// ---- a plain binary BVH over boxes (median split on the widest axis) ----
struct Box {
    float lo[3], hi[3];
    void reset() {
        for (int i = 0; i < 3; i++) { lo[i] = INFINITY; hi[i] = -INFINITY; }
    }
    void grow(const Box &b) {
        for (int i = 0; i < 3; i++) {
            lo[i] = std::min(lo[i], b.lo[i]);
            hi[i] = std::max(hi[i], b.hi[i]);
        }
    }
};

struct BvhNode {
    Box box;
    int32_t left, right;   // internal: child indices; leaf: left = -1
    int32_t first, count;  // leaf: range into prim_order
};

struct CpuBvh {
    std::vector<BvhNode> nodes;
    std::vector<int32_t> prim_order;

    void build(const std::vector<Box> &boxes) {
        nodes.clear();
        prim_order.resize(boxes.size());
        for (size_t i = 0; i < boxes.size(); i++) prim_order[i] = (int32_t)i;
        if (boxes.empty()) return;
        std::vector<float> cent(boxes.size() * 3);
        for (size_t i = 0; i < boxes.size(); i++)
            for (int a = 0; a < 3; a++)
                cent[i * 3 + a] = 0.5f * (boxes[i].lo[a] + boxes[i].hi[a]);
        nodes.reserve(boxes.size() * 2);
        build_rec(boxes, cent, 0, (int32_t)boxes.size());
    }

    int32_t build_rec(const std::vector<Box> &boxes, const std::vector<float> &cent,
                      int32_t first, int32_t count) {
        int32_t idx = (int32_t)nodes.size();
        nodes.push_back(BvhNode{});
        Box b; b.reset();
        Box cb; cb.reset();
        for (int32_t i = first; i < first + count; i++) {
            b.grow(boxes[prim_order[i]]);
            Box c;
            for (int a = 0; a < 3; a++) c.lo[a] = c.hi[a] = cent[prim_order[i] * 3 + a];
            cb.grow(c);
        }
        nodes[idx].box = b;
        if (count <= 4) {
            nodes[idx].left = -1; nodes[idx].right = -1;
            nodes[idx].first = first; nodes[idx].count = count;
            return idx;
        }
        int axis = 0;
        float ext = cb.hi[0] - cb.lo[0];
        for (int a = 1; a < 3; a++)
            if (cb.hi[a] - cb.lo[a] > ext) { ext = cb.hi[a] - cb.lo[a]; axis = a; }
        int32_t mid = first + count / 2;
        std::nth_element(prim_order.begin() + first, prim_order.begin() + mid,
                         prim_order.begin() + first + count,
                         [&](int32_t x, int32_t y) {
                             float cx = cent[x * 3 + axis], cy = cent[y * 3 + axis];
                             return cx < cy || (cx == cy && x < y);
                         });
        int32_t l = build_rec(boxes, cent, first, mid - first);
        int32_t r = build_rec(boxes, cent, mid, first + count - mid);
        nodes[idx].left = l; nodes[idx].right = r;
        nodes[idx].first = first; nodes[idx].count = count;
        return idx;
    }
};

// Slab test in FP32; returns entry distance or +inf on miss.
inline bool box_hit(const Box &b, f3 o, f3 inv_d, float tnear, float tfar) {
    // slack of ~8 ulps (the GPU traversal's): hits on box faces, and hits at
    // exactly the current closest distance (ties), are never culled
    float t0 = tnear, t1 = tfar * 1.000001f;
    const float oo[3] = {o.x, o.y, o.z};
    const float id[3] = {inv_d.x, inv_d.y, inv_d.z};
    for (int a = 0; a < 3; a++) {
        float ta = (b.lo[a] - oo[a]) * id[a];
        float tb = (b.hi[a] - oo[a]) * id[a];
        if (std::isnan(ta)) ta = -INFINITY;   // 0 * inf on a slab boundary
        if (std::isnan(tb)) tb = INFINITY;
        float tmin = std::min(ta, tb) * 0.999999f, tmax = std::max(ta, tb) * 1.000001f;
        t0 = std::max(t0, tmin);
        t1 = std::min(t1, tmax);
        if (t0 > t1) return false;
    }
    return true;
}

}  // namespace ljo
