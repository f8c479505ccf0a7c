// ORACLE / TEST INFRASTRUCTURE -- not part of the product.
//
// Double-precision vector math for the CPU restatement of lajolla's path
// (lj_oracle.cpp).  Follows the reference's own conventions:
//   normalize() returns 0 for a zero-length input      src/vector.h:250-257
//   Frisvad orthonormal basis                          src/frame.h:11-21
//   luminance weights                                   src/spectrum.h:32-34
//   PCG32 + init_pcg32 + next_pcg32_real<double>        src/pcg.h:16-68
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <utility>

namespace ljo {

constexpr double kPi = 3.14159265358979323846;
constexpr double kInvPi = 1.0 / kPi;
constexpr double kTwoPi = 2.0 * kPi;
constexpr double kInvTwoPi = 1.0 / kTwoPi;
constexpr double kInvFourPi = 1.0 / (4.0 * kPi);

struct V2 {
    double x = 0, y = 0;
    double operator[](int i) const { return i == 0 ? x : y; }
};
struct V3 {
    double x = 0, y = 0, z = 0;
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    double &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};

inline V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, double s) { return V3{a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(double s, V3 a) { return V3{a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator/(V3 a, double s) { return V3{a.x / s, a.y / s, a.z / s}; }
inline V3 operator/(V3 a, V3 b) { return V3{a.x / b.x, a.y / b.y, a.z / b.z}; }
inline V3 &operator+=(V3 &a, V3 b) { a = a + b; return a; }
inline V3 &operator*=(V3 &a, double s) { a = a * s; return a; }
inline V3 &operator/=(V3 &a, double s) { a = a / s; return a; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double length_squared(V3 a) { return dot(a, a); }
inline double length(V3 a) { return std::sqrt(length_squared(a)); }
inline double distance(V3 a, V3 b) { return length(a - b); }
inline double distance_squared(V3 a, V3 b) { return length_squared(a - b); }
inline V3 normalize(V3 a) {
    double l = length(a);
    if (l <= 0) return V3{0, 0, 0};
    return a / l;
}
inline double max3(V3 a) { return std::max(std::max(a.x, a.y), a.z); }
inline double luminance(V3 s) { return s.x * 0.212671 + s.y * 0.715160 + s.z * 0.072169; }
inline double avg3(V3 s) { return (s.x + s.y + s.z) / 3; }
inline V3 vmax(V3 a, V3 b) {
    return V3{std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)};
}
// src/vector.h:289-292: true if ANY component is finite (an OR, kept as is).
inline bool isfinite_any(V3 v) {
    return std::isfinite(v.x) || std::isfinite(v.y) || std::isfinite(v.z);
}

inline std::pair<V3, V3> coordinate_system(V3 n) {
    if (n.z < -1 + 1e-6) {
        return {V3{0, -1, 0}, V3{-1, 0, 0}};
    }
    double a = 1 / (1 + n.z);
    double b = -n.x * n.y * a;
    return {V3{1 - n.x * n.x * a, b, -n.x}, V3{b, 1 - n.y * n.y * a, -n.y}};
}

struct Frame {
    V3 x, y, n;
    Frame() {}
    Frame(V3 x_, V3 y_, V3 n_) : x(x_), y(y_), n(n_) {}
    explicit Frame(V3 n_) : n(n_) {
        auto p = coordinate_system(n_);
        x = p.first;
        y = p.second;
    }
};
inline Frame flip(const Frame &f) { return Frame(-f.x, -f.y, -f.n); }
inline V3 to_local(const Frame &f, V3 v) { return V3{dot(v, f.x), dot(v, f.y), dot(v, f.n)}; }
inline V3 to_world(const Frame &f, V3 v) { return f.x * v.x + f.y * v.y + f.n * v.z; }

// Row-major 4x4 (src/matrix.h).
struct M4 {
    double m[4][4] = {};
};
inline M4 mul(const M4 &a, const M4 &b) {
    M4 r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double s = 0;
            for (int k = 0; k < 4; k++) s += a.m[i][k] * b.m[k][j];
            r.m[i][j] = s;
        }
    return r;
}
M4 inverse(const M4 &m);  // lj_oracle.cpp
inline V3 xform_point(const M4 &x, V3 p) {
    double t0 = x.m[0][0] * p.x + x.m[0][1] * p.y + x.m[0][2] * p.z + x.m[0][3];
    double t1 = x.m[1][0] * p.x + x.m[1][1] * p.y + x.m[1][2] * p.z + x.m[1][3];
    double t2 = x.m[2][0] * p.x + x.m[2][1] * p.y + x.m[2][2] * p.z + x.m[2][3];
    double t3 = x.m[3][0] * p.x + x.m[3][1] * p.y + x.m[3][2] * p.z + x.m[3][3];
    double iw = 1.0 / t3;
    return V3{t0 * iw, t1 * iw, t2 * iw};
}
inline V3 xform_vector(const M4 &x, V3 v) {
    return V3{x.m[0][0] * v.x + x.m[0][1] * v.y + x.m[0][2] * v.z,
              x.m[1][0] * v.x + x.m[1][1] * v.y + x.m[1][2] * v.z,
              x.m[2][0] * v.x + x.m[2][1] * v.y + x.m[2][2] * v.z};
}

// ---- PCG32 ----
struct Pcg {
    uint64_t state, inc;
};
inline uint32_t pcg_next(Pcg &r) {
    uint64_t old = r.state;
    r.state = old * 6364136223846793005ULL + (r.inc | 1);
    uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((-rot) & 31));
}
inline Pcg pcg_init(uint64_t stream, uint64_t seed = 0x31e241f862a1fb5eULL) {
    Pcg s;
    s.state = 0;
    s.inc = (stream << 1u) | 1u;
    pcg_next(s);
    s.state += seed;
    pcg_next(s);
    return s;
}
// next_pcg32_real<double>: exactly u32 * 2^-32.
inline double pcg_real_double(Pcg &r) {
    union {
        uint64_t u;
        double d;
    } x;
    x.u = ((uint64_t)pcg_next(r) << 20) | 0x3ff0000000000000ULL;
    return x.d - 1.0;
}
// The GPU's uniform: the top 24 bits of the PCG output, (u32 >> 8) * 2^-24,
// exactly representable in FP32 and in [0, 1).
inline double pcg_real_24(Pcg &r) { return (double)(pcg_next(r) >> 8) * (1.0 / 16777216.0); }

// Per-(job, pixel, sample) stream keying used by the GPU wavefront:
//   stream = pixel index (y * width + x), seed = splitmix64(job_seed ^ (golden * (sample + 1)))
inline uint64_t splitmix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
inline Pcg pcg_keyed(uint64_t job_seed, uint64_t pixel, uint64_t sample) {
    return pcg_init(pixel, splitmix64(job_seed ^ (0x9e3779b97f4a7c15ULL * (sample + 1))));
}

}  // namespace ljo
