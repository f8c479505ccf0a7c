// Device-side math shared by every kernel of the GB300 hot path.
//
// FP32 restatements of the reference's double-precision helpers:
//   normalize() returns 0 for a zero-length input     src/vector.h:250-257
//   Frisvad orthonormal basis                          src/frame.h:11-21
//   luminance weights                                  src/spectrum.h:32-34
//   PCG32 step and init_pcg32                          src/pcg.h:16-41
// plus the two places that must round exactly like the CPU oracle: the ray /
// triangle test and the Morton code (explicit __fmaf_rn / __fmul_rn /
// __fadd_rn so that nvcc's contraction cannot change a rounding).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define LJ_HD __host__ __device__ __forceinline__
#define LJ_D __device__ __forceinline__

namespace lj {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 1.0f / kPi;
constexpr float kTwoPi = 2.0f * kPi;
constexpr float kInvTwoPi = 1.0f / kTwoPi;
constexpr float kInvFourPi = 1.0f / (4.0f * kPi);

struct V3 {
    float x, y, z;
};
LJ_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
LJ_HD V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
LJ_HD V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
LJ_HD V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
LJ_HD V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
LJ_HD V3 operator*(float s, V3 a) { return V3{a.x * s, a.y * s, a.z * s}; }
LJ_HD V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
LJ_HD V3 operator/(V3 a, float s) { float r = 1.0f / s; return V3{a.x * r, a.y * r, a.z * r}; }
LJ_HD V3 &operator+=(V3 &a, V3 b) { a = a + b; return a; }
LJ_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
LJ_HD V3 cross(V3 a, V3 b) {
    return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
LJ_HD float length2(V3 a) { return dot(a, a); }
LJ_HD float length(V3 a) { return sqrtf(dot(a, a)); }
LJ_HD V3 normalize(V3 a) {
    float l = length(a);
    if (!(l > 0.0f)) return V3{0, 0, 0};
    return V3{a.x / l, a.y / l, a.z / l};
}
LJ_HD float max3(V3 a) { return fmaxf(fmaxf(a.x, a.y), a.z); }
LJ_HD float luminance(V3 s) { return s.x * 0.212671f + s.y * 0.715160f + s.z * 0.072169f; }
LJ_HD float avg3(V3 s) { return (s.x + s.y + s.z) * (1.0f / 3.0f); }
LJ_HD float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

struct Frame {
    V3 x, y, n;
};
LJ_HD Frame frame_from_n(V3 n) {
    Frame f;
    f.n = n;
    if (n.z < -1.0f + 1e-6f) {
        f.x = V3{0, -1, 0};
        f.y = V3{-1, 0, 0};
    } else {
        float a = 1.0f / (1.0f + n.z);
        float b = -n.x * n.y * a;
        f.x = V3{1.0f - n.x * n.x * a, b, -n.x};
        f.y = V3{b, 1.0f - n.y * n.y * a, -n.y};
    }
    return f;
}
LJ_HD Frame flip(const Frame &f) { return Frame{-f.x, -f.y, -f.n}; }
LJ_HD V3 to_local(const Frame &f, V3 v) { return V3{dot(v, f.x), dot(v, f.y), dot(v, f.n)}; }
LJ_HD V3 to_world(const Frame &f, V3 v) { return f.x * v.x + f.y * v.y + f.n * v.z; }

// ---- PCG32 (src/pcg.h:16-41) with per-(job, pixel, sample) keying --------
struct Pcg {
    uint64_t state, inc;
};
LJ_HD uint32_t pcg_next(Pcg &r) {
    uint64_t old = r.state;
    r.state = old * 6364136223846793005ULL + (r.inc | 1ULL);
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
}
LJ_HD Pcg pcg_init(uint64_t stream, uint64_t seed) {
    Pcg s;
    s.state = 0;
    s.inc = (stream << 1u) | 1u;
    pcg_next(s);
    s.state += seed;
    pcg_next(s);
    return s;
}
LJ_HD uint64_t splitmix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
// RNG keyed on (job seed, pixel, sample): a job's image does not depend on
// which slot, queue position or batch its paths ran in.
LJ_HD Pcg pcg_keyed(uint64_t job_seed, uint64_t pixel, uint64_t sample) {
    return pcg_init(pixel, splitmix64(job_seed ^ (0x9e3779b97f4a7c15ULL * (sample + 1))));
}
// Uniform in [0, 1): top 24 bits, exact in FP32.
LJ_HD float pcg_uniform(Pcg &r) { return (float)(pcg_next(r) >> 8) * (1.0f / 16777216.0f); }

// ---- exact-rounding triangle test (oracle/ljo_geom.h has the CPU twin) ---
LJ_D V3 xcross(V3 a, V3 b) {
    return V3{__fmaf_rn(a.y, b.z, -__fmul_rn(a.z, b.y)), __fmaf_rn(a.z, b.x, -__fmul_rn(a.x, b.z)),
              __fmaf_rn(a.x, b.y, -__fmul_rn(a.y, b.x))};
}
LJ_D float xdot(V3 a, V3 b) {
    return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x)));
}
LJ_D V3 xsub(V3 a, V3 b) { return V3{__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)}; }

// Moller-Trumbore on precomputed (v0, e1 = v1 - v0, e2 = v2 - v0); accepts
// tnear < t <= tfar (callers reject t == tfar unless it breaks a tie
// with the current closest hit).  Same operation sequence as
// ljo::tri_intersect.
LJ_D bool tri_intersect(V3 v0, V3 e1, V3 e2, V3 o, V3 d, float tnear, float tfar, float &t_out,
                        float &u_out, float &v_out) {
    V3 pvec = xcross(d, e2);
    float det = xdot(e1, pvec);
    if (det == 0.0f) return false;
    float inv_det = __frcp_rn(det);
    V3 tvec = xsub(o, v0);
    float u = __fmul_rn(xdot(tvec, pvec), inv_det);
    if (!(u >= 0.0f && u <= 1.0f)) return false;
    V3 qvec = xcross(tvec, e1);
    float v = __fmul_rn(xdot(d, qvec), inv_det);
    if (!(v >= 0.0f && __fadd_rn(u, v) <= 1.0f)) return false;
    float t = __fmul_rn(xdot(e2, qvec), inv_det);
    if (!(t > tnear && t <= tfar)) return false;
    t_out = t;
    u_out = u;
    v_out = v;
    return true;
}

// ---- 30-bit Morton code over the centroid box (ljo::morton3's twin) ------
LJ_HD uint32_t expand_bits10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
LJ_D V3 tri_centroid(V3 p0, V3 p1, V3 p2) {
    const float third = 1.0f / 3.0f;
    return V3{__fmul_rn(__fadd_rn(__fadd_rn(p0.x, p1.x), p2.x), third),
              __fmul_rn(__fadd_rn(__fadd_rn(p0.y, p1.y), p2.y), third),
              __fmul_rn(__fadd_rn(__fadd_rn(p0.z, p1.z), p2.z), third)};
}
LJ_D uint32_t morton_quant(float c, float lo, float scale) {
    float q = floorf(__fmul_rn(__fsub_rn(c, lo), scale));
    if (!(q >= 0.0f)) q = 0.0f;
    if (q > 1023.0f) q = 1023.0f;
    return (uint32_t)q;
}
LJ_D float morton_scale(float lo, float hi) {
    float ext = __fsub_rn(hi, lo);
    return ext > 0.0f ? __fdiv_rn(1024.0f, ext) : 0.0f;
}
LJ_D uint32_t morton3(V3 c, V3 lo, V3 scale) {
    uint32_t x = morton_quant(c.x, lo.x, scale.x);
    uint32_t y = morton_quant(c.y, lo.y, scale.y);
    uint32_t z = morton_quant(c.z, lo.z, scale.z);
    return (expand_bits10(x) << 2) | (expand_bits10(y) << 1) | expand_bits10(z);
}

}  // namespace lj
