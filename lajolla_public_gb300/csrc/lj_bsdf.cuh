// BSDFs on the device, FP32: replaces eval / sample_bsdf / pdf_sample_bsdf
// (src/material.cpp:90-119) for
//   Lambertian       src/materials/lambertian.inl:1-50
//   RoughPlastic     src/materials/roughplastic.inl:3-161
//   RoughDielectric  src/materials/roughdielectric.inl:3-177
//   microfacet       src/microfacet.h:24-114
// and the Disney BSDF family, whose reference bodies are homework stubs
// (src/materials/disney_*.inl): restated from handouts/homework1.tex:93-556.
//
// Materials are evaluated from `MatParams`: every texture slot already
// evaluated at the shading point (RGB slots in .x/.y/.z, scalars in .x).
// The shading vertex is given by its geometric normal and shading frame.
//
// FP32 care: GTR2's 1 + (a^2 - 1) cos^2 is written as sin^2 + a^2 cos^2 with
// sin^2 taken from the local half vector, so tiny roughness does not cancel.
#pragma once

#include "lj_common.cuh"

namespace lj {

constexpr int kMatSlots = 12;

struct MatParams {
    int type;
    float eta;
    V3 s[kMatSlots];
};

struct BsdfVertex {
    V3 ng;        // geometric normal (already flipped toward the shading normal)
    Frame frame;  // shading frame
};

struct BsdfSample {
    V3 dir;
    float eta;        // 0 unless refraction
    float roughness;
    bool valid;
};

LJ_HD float sq(float x) { return x * x; }
LJ_HD float pow5(float x) { float x2 = x * x; return x2 * x2 * x; }
LJ_HD float schlick_w(float c) { return pow5(fmaxf(1.0f - c, 0.0f)); }

// ---- microfacet helpers (src/microfacet.h) ----
LJ_HD float fresnel_dielectric(float n_dot_i, float n_dot_t, float eta) {
    float rs = (n_dot_i - eta * n_dot_t) / (n_dot_i + eta * n_dot_t);
    float rp = (eta * n_dot_i - n_dot_t) / (eta * n_dot_i + n_dot_t);
    return (rs * rs + rp * rp) * 0.5f;
}
LJ_HD float fresnel_dielectric(float n_dot_i, float eta) {
    float n_dot_t_sq = 1.0f - (1.0f - n_dot_i * n_dot_i) / (eta * eta);
    if (n_dot_t_sq < 0.0f) return 1.0f;
    return fresnel_dielectric(fabsf(n_dot_i), sqrtf(n_dot_t_sq), eta);
}
// GTR2 / GGX with the local half vector hl (|hl| = 1): a2 / (pi t^2),
// t = 1 + (a2 - 1) cos^2 = sin^2 + a2 cos^2.
LJ_HD float gtr2_local(V3 hl, float roughness) {
    float alpha = roughness * roughness, a2 = alpha * alpha;
    float t = (hl.x * hl.x + hl.y * hl.y) + a2 * hl.z * hl.z;
    return a2 / (kPi * t * t);
}
LJ_HD float smith_gtr2(V3 v, float roughness) {
    float alpha = roughness * roughness, a2 = alpha * alpha;
    float lambda = (-1.0f + sqrtf(1.0f + (v.x * v.x * a2 + v.y * v.y * a2) / (v.z * v.z))) * 0.5f;
    return 1.0f / (1.0f + lambda);
}
// anisotropic GTR2 and Smith (homework1.tex:200-240)
LJ_HD float aniso_D(V3 hl, float ax, float ay) {
    float t = hl.x * hl.x / (ax * ax) + hl.y * hl.y / (ay * ay) + hl.z * hl.z;
    return 1.0f / (kPi * ax * ay * t * t);
}
LJ_HD float aniso_G1(V3 wl, float ax, float ay) {
    float lam = (sqrtf(1.0f + (sq(wl.x * ax) + sq(wl.y * ay)) / (wl.z * wl.z)) - 1.0f) * 0.5f;
    return 1.0f / (1.0f + lam);
}
// Heitz 2018 visible-normal sampling with (ax, ay); ax == ay is
// src/microfacet.h:85-114.
LJ_HD V3 sample_vndf(V3 wi, float ax, float ay, float u0, float u1) {
    float sgn = 1.0f;
    if (wi.z < 0.0f) { wi = -wi; sgn = -1.0f; }
    V3 hemi = normalize(V3{ax * wi.x, ay * wi.y, wi.z});
    float r = sqrtf(u0);
    float phi = kTwoPi * u1;
    float sp, cp;
    sincosf(phi, &sp, &cp);
    float t1 = r * cp, t2 = r * sp;
    float s = (1.0f + hemi.z) * 0.5f;
    t2 = (1.0f - s) * sqrtf(fmaxf(0.0f, 1.0f - t1 * t1)) + s * t2;
    V3 disk{t1, t2, sqrtf(fmaxf(0.0f, 1.0f - t1 * t1 - t2 * t2))};
    Frame hf = frame_from_n(hemi);
    V3 hn = to_world(hf, disk);
    V3 h = normalize(V3{ax * hn.x, ay * hn.y, fmaxf(0.0f, hn.z)});
    return h * sgn;
}
// src/material.cpp:4-11
LJ_HD V3 sample_cos_hemisphere(float u0, float u1) {
    float phi = kTwoPi * u0;
    float tmp = sqrtf(clampf(1.0f - u1, 0.0f, 1.0f));
    float sp, cp;
    sincosf(phi, &sp, &cp);
    return V3{cp * tmp, sp * tmp, sqrtf(clampf(u1, 0.0f, 1.0f))};
}
LJ_HD V3 reflect_about(V3 wi, V3 h) { return normalize(-wi + h * (2.0f * dot(wi, h))); }
LJ_HD Frame upper_frame(const BsdfVertex &v, V3 wi) {
    return dot(v.frame.n, wi) < 0.0f ? flip(v.frame) : v.frame;
}
LJ_HD BsdfSample no_sample() { return BsdfSample{V3{0, 0, 0}, 0.0f, 0.0f, false}; }

// ---- Lambertian ----
LJ_HD V3 lambert_eval(V3 R, const BsdfVertex &v, V3 wi, V3 wo) {
    if (dot(v.ng, wi) < 0.0f || dot(v.ng, wo) < 0.0f) return V3{0, 0, 0};
    Frame f = upper_frame(v, wi);
    return R * (fmaxf(dot(f.n, wo), 0.0f) * kInvPi);
}
LJ_HD float lambert_pdf(const BsdfVertex &v, V3 wi, V3 wo) {
    if (dot(v.ng, wi) < 0.0f || dot(v.ng, wo) < 0.0f) return 0.0f;
    Frame f = upper_frame(v, wi);
    return fmaxf(dot(f.n, wo), 0.0f) * kInvPi;
}
LJ_HD BsdfSample lambert_sample(const BsdfVertex &v, V3 wi, float u0, float u1, float roughness) {
    if (dot(v.ng, wi) < 0.0f) return no_sample();
    Frame f = upper_frame(v, wi);
    return BsdfSample{to_world(f, sample_cos_hemisphere(u0, u1)), 0.0f, roughness, true};
}

// ---- RoughPlastic ----
LJ_HD V3 plastic_eval(const MatParams &m, const BsdfVertex &v, V3 wi, V3 wo) {
    if (dot(v.ng, wi) < 0.0f || dot(v.ng, wo) < 0.0f) return V3{0, 0, 0};
    Frame f = upper_frame(v, wi);
    V3 h = normalize(wi + wo);
    V3 hl = to_local(f, h);
    float n_dot_h = hl.z, n_dot_in = dot(f.n, wi), n_dot_out = dot(f.n, wo);
    if (n_dot_out <= 0.0f || n_dot_h <= 0.0f) return V3{0, 0, 0};
    float r = clampf(m.s[2].x, 0.01f, 1.0f);
    float F_o = fresnel_dielectric(dot(h, wo), m.eta);
    float D = gtr2_local(hl, r);
    float G = smith_gtr2(to_local(f, wi), r) * smith_gtr2(to_local(f, wo), r);
    V3 spec = m.s[1] * ((G * F_o * D) / (4.0f * n_dot_in * n_dot_out));
    float F_i = fresnel_dielectric(dot(h, wi), m.eta);
    V3 diff = m.s[0] * ((1.0f - F_o) * (1.0f - F_i) * kInvPi);
    return (spec + diff) * n_dot_out;
}
LJ_HD float plastic_pdf(const MatParams &m, const BsdfVertex &v, V3 wi, V3 wo) {
    if (dot(v.ng, wi) < 0.0f || dot(v.ng, wo) < 0.0f) return 0.0f;
    Frame f = upper_frame(v, wi);
    V3 h = normalize(wi + wo);
    V3 hl = to_local(f, h);
    float n_dot_in = dot(f.n, wi), n_dot_out = dot(f.n, wo), n_dot_h = hl.z;
    if (n_dot_out <= 0.0f || n_dot_h <= 0.0f) return 0.0f;
    float lS = luminance(m.s[1]), lR = luminance(m.s[0]);
    if (lS + lR <= 0.0f) return 0.0f;
    float r = clampf(m.s[2].x, 0.01f, 1.0f);
    float spec_prob = lS / (lS + lR), diff_prob = 1.0f - spec_prob;
    float G = smith_gtr2(to_local(f, wi), r);
    float D = gtr2_local(hl, r);
    return spec_prob * (G * D) / (4.0f * n_dot_in) + diff_prob * n_dot_out * kInvPi;
}
LJ_HD BsdfSample plastic_sample(const MatParams &m, const BsdfVertex &v, V3 wi, float u0, float u1, float w) {
    if (dot(v.ng, wi) < 0.0f) return no_sample();
    Frame f = upper_frame(v, wi);
    float lS = luminance(m.s[1]), lR = luminance(m.s[0]);
    if (lS + lR <= 0.0f) return no_sample();
    float spec_prob = lS / (lS + lR);
    if (w < spec_prob) {
        float r = clampf(m.s[2].x, 0.01f, 1.0f);
        float a = r * r;
        V3 h = to_world(f, sample_vndf(to_local(f, wi), a, a, u0, u1));
        return BsdfSample{reflect_about(wi, h), 0.0f, r, true};
    }
    return BsdfSample{to_world(f, sample_cos_hemisphere(u0, u1)), 0.0f, 1.0f, true};
}

// ---- RoughDielectric (and Disney glass with anisotropic alphas) ----
// iso: clamped roughness with GTR2 / Smith (roughdielectric.inl);
// otherwise (ax, ay) with the anisotropic D / G of homework1.tex:336-380.
struct DielParams {
    V3 Ks, Kt;
    float eta;
    bool iso;
    float roughness;   // iso
    float ax, ay;      // aniso
};
LJ_HD void diel_DG(const DielParams &p, const Frame &f, V3 hl, V3 wi, V3 wo, float &D, float &G_in,
                   float &G_out) {
    if (p.iso) {
        float r = clampf(p.roughness, 0.01f, 1.0f);
        D = gtr2_local(hl, r);
        G_in = smith_gtr2(to_local(f, wi), r);
        G_out = smith_gtr2(to_local(f, wo), r);
    } else {
        D = aniso_D(hl, p.ax, p.ay);
        G_in = aniso_G1(to_local(f, wi), p.ax, p.ay);
        G_out = aniso_G1(to_local(f, wo), p.ax, p.ay);
    }
}
LJ_HD V3 diel_eval(const DielParams &p, const BsdfVertex &v, V3 wi, V3 wo, bool to_view) {
    float ngi = dot(v.ng, wi);
    bool reflect = ngi * dot(v.ng, wo) > 0.0f;
    Frame f = dot(v.frame.n, wi) * ngi < 0.0f ? flip(v.frame) : v.frame;
    float eta = ngi > 0.0f ? p.eta : 1.0f / p.eta;
    V3 h = reflect ? normalize(wi + wo) : normalize(wi + wo * eta);
    if (dot(h, f.n) < 0.0f) h = -h;
    float h_dot_in = dot(h, wi);
    float F = fresnel_dielectric(h_dot_in, eta);
    float D, Gi, Go;
    diel_DG(p, f, to_local(f, h), wi, wo, D, Gi, Go);
    float G = Gi * Go;
    if (reflect) return p.Ks * ((F * D * G) / (4.0f * fabsf(dot(f.n, wi))));
    float eta_factor = to_view ? 1.0f : 1.0f / (eta * eta);
    float h_dot_out = dot(h, wo);
    float sd = h_dot_in + eta * h_dot_out;
    return p.Kt * ((eta_factor * (1.0f - F) * D * G * eta * eta * fabsf(h_dot_out * h_dot_in)) /
                   (fabsf(dot(f.n, wi)) * sd * sd));
}
LJ_HD float diel_pdf(const DielParams &p, const BsdfVertex &v, V3 wi, V3 wo) {
    float ngi = dot(v.ng, wi);
    bool reflect = ngi * dot(v.ng, wo) > 0.0f;
    Frame f = dot(v.frame.n, wi) * ngi < 0.0f ? flip(v.frame) : v.frame;
    float eta = ngi > 0.0f ? p.eta : 1.0f / p.eta;
    V3 h = reflect ? normalize(wi + wo) : normalize(wi + wo * eta);
    if (dot(h, f.n) < 0.0f) h = -h;
    float h_dot_in = dot(h, wi);
    float F = fresnel_dielectric(h_dot_in, eta);
    float D, Gi, Go;
    diel_DG(p, f, to_local(f, h), wi, wo, D, Gi, Go);
    if (reflect) return (F * D * Gi) / (4.0f * fabsf(dot(f.n, wi)));
    float h_dot_out = dot(h, wo);
    float sd = h_dot_in + eta * h_dot_out;
    float dh_dout = eta * eta * h_dot_out / (sd * sd);
    return (1.0f - F) * D * Gi * fabsf(dh_dout * h_dot_in / dot(f.n, wi));
}
LJ_HD BsdfSample diel_sample(const DielParams &p, const BsdfVertex &v, V3 wi, float u0, float u1, float w,
                             float rec_roughness) {
    float ngi = dot(v.ng, wi);
    float eta = ngi > 0.0f ? p.eta : 1.0f / p.eta;
    Frame f = dot(v.frame.n, wi) * ngi < 0.0f ? flip(v.frame) : v.frame;
    float ax, ay;
    if (p.iso) {
        float r = clampf(p.roughness, 0.01f, 1.0f);
        ax = ay = r * r;
        rec_roughness = r;
    } else {
        ax = p.ax;
        ay = p.ay;
    }
    V3 h = to_world(f, sample_vndf(to_local(f, wi), ax, ay, u0, u1));
    if (dot(h, f.n) < 0.0f) h = -h;
    float h_dot_in = dot(h, wi);
    float F = fresnel_dielectric(h_dot_in, eta);
    if (w <= F) return BsdfSample{reflect_about(wi, h), 0.0f, rec_roughness, true};
    float h_dot_out_sq = 1.0f - (1.0f - h_dot_in * h_dot_in) / (eta * eta);
    if (h_dot_out_sq <= 0.0f) return no_sample();
    if (h_dot_in < 0.0f) h = -h;
    float h_dot_out = sqrtf(h_dot_out_sq);
    V3 refr = -wi / eta + h * (fabsf(h_dot_in) / eta - h_dot_out);
    return BsdfSample{refr, eta, rec_roughness, true};
}

// ---- Disney lobes (homework1.tex) ----
LJ_HD void disney_alphas(float roughness, float anisotropic, float &ax, float &ay) {
    float aspect = sqrtf(1.0f - 0.9f * anisotropic);
    ax = fmaxf(0.0001f, roughness * roughness / aspect);
    ay = fmaxf(0.0001f, roughness * roughness * aspect);
}
LJ_HD V3 tint_of(V3 base) {
    float l = luminance(base);
    return l > 0.0f ? base / l : V3{1, 1, 1};
}
LJ_HD V3 ddiffuse_eval(V3 base, float rough, float subsurface, const BsdfVertex &v, V3 wi, V3 wo) {
    if (dot(v.ng, wi) < 0.0f || dot(v.ng, wo) < 0.0f) return V3{0, 0, 0};
    Frame f = upper_frame(v, wi);
    V3 h = normalize(wi + wo);
    float ndi = fabsf(dot(f.n, wi)), ndo = fabsf(dot(f.n, wo)), hdo = fabsf(dot(h, wo));
    float fd90 = 0.5f + 2.0f * rough * hdo * hdo;
    float fdi = 1.0f + (fd90 - 1.0f) * pow5(1.0f - ndi);
    float fdo = 1.0f + (fd90 - 1.0f) * pow5(1.0f - ndo);
    float fss90 = rough * hdo * hdo;
    float fssi = 1.0f + (fss90 - 1.0f) * pow5(1.0f - ndi);
    float fsso = 1.0f + (fss90 - 1.0f) * pow5(1.0f - ndo);
    float base_d = fdi * fdo * ndo * kInvPi;
    float ss = 1.25f * kInvPi * (fssi * fsso * (1.0f / (ndi + ndo) - 0.5f) + 0.5f) * ndo;
    return base * ((1.0f - subsurface) * base_d + subsurface * ss);
}
LJ_HD V3 dmetal_eval(V3 F0, float ax, float ay, const BsdfVertex &v, V3 wi, V3 wo) {
    if (dot(v.ng, wi) < 0.0f || dot(v.ng, wo) < 0.0f) return V3{0, 0, 0};
    Frame f = upper_frame(v, wi);
    V3 h = normalize(wi + wo);
    V3 hl = to_local(f, h);
    if (dot(f.n, wo) <= 0.0f || hl.z <= 0.0f) return V3{0, 0, 0};
    float fw = schlick_w(fabsf(dot(h, wo)));
    V3 F = F0 + (V3{1, 1, 1} - F0) * fw;
    float D = aniso_D(hl, ax, ay);
    float G = aniso_G1(to_local(f, wi), ax, ay) * aniso_G1(to_local(f, wo), ax, ay);
    return F * (D * G / (4.0f * fabsf(dot(f.n, wi))));
}
LJ_HD float dmetal_pdf(float ax, float ay, const BsdfVertex &v, V3 wi, V3 wo) {
    if (dot(v.ng, wi) < 0.0f || dot(v.ng, wo) < 0.0f) return 0.0f;
    Frame f = upper_frame(v, wi);
    V3 h = normalize(wi + wo);
    V3 hl = to_local(f, h);
    if (dot(f.n, wo) <= 0.0f || hl.z <= 0.0f) return 0.0f;
    return aniso_D(hl, ax, ay) * aniso_G1(to_local(f, wi), ax, ay) / (4.0f * fabsf(dot(f.n, wi)));
}
LJ_HD BsdfSample dmetal_sample(float ax, float ay, float rough, const BsdfVertex &v, V3 wi, float u0, float u1) {
    if (dot(v.ng, wi) < 0.0f) return no_sample();
    Frame f = upper_frame(v, wi);
    V3 h = to_world(f, sample_vndf(to_local(f, wi), ax, ay, u0, u1));
    return BsdfSample{reflect_about(wi, h), 0.0f, rough, true};
}
LJ_HD float cc_alpha(float gloss) { return (1.0f - gloss) * 0.1f + gloss * 0.001f; }
LJ_HD float dclearcoat_D(float hz, float a2) {
    return (a2 - 1.0f) / (kPi * logf(a2) * (1.0f + (a2 - 1.0f) * hz * hz));
}
LJ_HD float dclearcoat_eval(float gloss, const BsdfVertex &v, V3 wi, V3 wo) {
    if (dot(v.ng, wi) < 0.0f || dot(v.ng, wo) < 0.0f) return 0.0f;
    Frame f = upper_frame(v, wi);
    V3 h = normalize(wi + wo);
    V3 hl = to_local(f, h);
    if (dot(f.n, wo) <= 0.0f || hl.z <= 0.0f) return 0.0f;
    float ag = cc_alpha(gloss), a2 = ag * ag;
    const float R0 = 0.04f;   // ((1.5 - 1) / (1.5 + 1))^2
    float Fc = R0 + (1.0f - R0) * schlick_w(fabsf(dot(h, wo)));
    float Gc = aniso_G1(to_local(f, wi), 0.25f, 0.25f) * aniso_G1(to_local(f, wo), 0.25f, 0.25f);
    return Fc * dclearcoat_D(hl.z, a2) * Gc / (4.0f * fabsf(dot(f.n, wi)));
}
LJ_HD float dclearcoat_pdf(float gloss, const BsdfVertex &v, V3 wi, V3 wo) {
    if (dot(v.ng, wi) < 0.0f || dot(v.ng, wo) < 0.0f) return 0.0f;
    Frame f = upper_frame(v, wi);
    V3 h = normalize(wi + wo);
    V3 hl = to_local(f, h);
    if (dot(f.n, wo) <= 0.0f || hl.z <= 0.0f) return 0.0f;
    float ag = cc_alpha(gloss), a2 = ag * ag;
    return dclearcoat_D(hl.z, a2) * fabsf(hl.z) / (4.0f * fabsf(dot(h, wo)));
}
LJ_HD BsdfSample dclearcoat_sample(float gloss, const BsdfVertex &v, V3 wi, float u0, float u1) {
    if (dot(v.ng, wi) < 0.0f) return no_sample();
    Frame f = upper_frame(v, wi);
    float ag = cc_alpha(gloss), a2 = ag * ag;
    // (1 - a2^(1 - u0)) written as -expm1((1 - u0) log a2): no cancellation
    float ce = sqrtf(fmaxf(0.0f, -expm1f((1.0f - u0) * logf(a2)) / (1.0f - a2)));
    float se = sqrtf(fmaxf(0.0f, 1.0f - ce * ce));
    float sp, cp;
    sincosf(kTwoPi * u1, &sp, &cp);
    V3 h = to_world(f, V3{se * cp, se * sp, ce});
    return BsdfSample{reflect_about(wi, h), 0.0f, sqrtf(ag), true};
}
LJ_HD V3 dsheen_eval(V3 base, float tint_w, const BsdfVertex &v, V3 wi, V3 wo) {
    if (dot(v.ng, wi) < 0.0f || dot(v.ng, wo) < 0.0f) return V3{0, 0, 0};
    Frame f = upper_frame(v, wi);
    V3 h = normalize(wi + wo);
    V3 cs = V3{1, 1, 1} * (1.0f - tint_w) + tint_of(base) * tint_w;
    return cs * (schlick_w(fabsf(dot(h, wo))) * fmaxf(dot(f.n, wo), 0.0f));
}
LJ_HD V3 sqrt3(V3 s) { return V3{sqrtf(fmaxf(s.x, 0.f)), sqrtf(fmaxf(s.y, 0.f)), sqrtf(fmaxf(s.z, 0.f))}; }

// Disney BSDF (homework1.tex:460-546); slots per lj_gpu.h.
struct DisneyP {
    V3 base;
    float st, metallic, subsurface, specular, rough, spec_tint, aniso, sheen, sheen_tint, cc, cc_gloss, eta;
};
LJ_HD DisneyP disney_params(const MatParams &m) {
    return DisneyP{m.s[0], m.s[1].x, m.s[2].x, m.s[3].x, m.s[4].x, m.s[5].x, m.s[6].x,
                   m.s[7].x, m.s[8].x, m.s[9].x, m.s[10].x, m.s[11].x, m.eta};
}
LJ_HD V3 disney_F0(const DisneyP &p) {
    V3 Ks = V3{1, 1, 1} * (1.0f - p.spec_tint) + tint_of(p.base) * p.spec_tint;
    float R0 = sq(p.eta - 1.0f) / sq(p.eta + 1.0f);
    return Ks * (p.specular * R0 * (1.0f - p.metallic)) + p.base * p.metallic;
}
LJ_HD void disney_weights(const DisneyP &p, bool inside, float w[4]) {
    if (inside) { w[0] = 0; w[1] = 0; w[2] = 1; w[3] = 0; return; }
    w[0] = (1.0f - p.metallic) * (1.0f - p.st);
    w[1] = 1.0f - p.st * (1.0f - p.metallic);
    w[2] = (1.0f - p.metallic) * p.st;
    w[3] = 0.25f * p.cc;
}
LJ_HD DielParams disney_glass(const DisneyP &p, float ax, float ay) {
    return DielParams{p.base, sqrt3(p.base), p.eta, false, 0.0f, ax, ay};
}
LJ_HD V3 disney_eval(const DisneyP &p, const BsdfVertex &v, V3 wi, V3 wo, bool to_view) {
    float ax, ay;
    disney_alphas(p.rough, p.aniso, ax, ay);
    bool inside = dot(v.ng, wi) <= 0.0f;
    V3 r = diel_eval(disney_glass(p, ax, ay), v, wi, wo, to_view) * ((1.0f - p.metallic) * p.st);
    if (inside) return r;
    r += ddiffuse_eval(p.base, p.rough, p.subsurface, v, wi, wo) * ((1.0f - p.st) * (1.0f - p.metallic));
    r += dsheen_eval(p.base, p.sheen_tint, v, wi, wo) * ((1.0f - p.metallic) * p.sheen);
    r += dmetal_eval(disney_F0(p), ax, ay, v, wi, wo) * (1.0f - p.st * (1.0f - p.metallic));
    r += V3{1, 1, 1} * (0.25f * p.cc * dclearcoat_eval(p.cc_gloss, v, wi, wo));
    return r;
}
LJ_HD float disney_pdf(const DisneyP &p, const BsdfVertex &v, V3 wi, V3 wo) {
    float ax, ay;
    disney_alphas(p.rough, p.aniso, ax, ay);
    float w[4];
    disney_weights(p, dot(v.ng, wi) <= 0.0f, w);
    float tw = w[0] + w[1] + w[2] + w[3];
    if (tw <= 0.0f) return 0.0f;
    float pdf = 0.0f;
    if (w[0] > 0.0f) pdf += w[0] * lambert_pdf(v, wi, wo);
    if (w[1] > 0.0f) pdf += w[1] * dmetal_pdf(ax, ay, v, wi, wo);
    if (w[2] > 0.0f) pdf += w[2] * diel_pdf(disney_glass(p, ax, ay), v, wi, wo);
    if (w[3] > 0.0f) pdf += w[3] * dclearcoat_pdf(p.cc_gloss, v, wi, wo);
    return pdf / tw;
}
LJ_HD BsdfSample disney_sample(const DisneyP &p, const BsdfVertex &v, V3 wi, float u0, float u1, float rw) {
    float ax, ay;
    disney_alphas(p.rough, p.aniso, ax, ay);
    float w[4];
    disney_weights(p, dot(v.ng, wi) <= 0.0f, w);
    float tw = w[0] + w[1] + w[2] + w[3];
    if (tw <= 0.0f) return no_sample();
    float x = rw * tw;
    if (x < w[0]) return lambert_sample(v, wi, u0, u1, p.rough);
    x -= w[0];
    if (x < w[1]) return dmetal_sample(ax, ay, p.rough, v, wi, u0, u1);
    x -= w[1];
    if (x < w[2] || w[3] <= 0.0f) {
        float wr = w[2] > 0.0f ? clampf(x / w[2], 0.0f, 1.0f) : 0.0f;
        return diel_sample(disney_glass(p, ax, ay), v, wi, u0, u1, wr, p.rough);
    }
    return dclearcoat_sample(p.cc_gloss, v, wi, u0, u1);
}

// ---- dispatch (src/material.cpp:90-119) ----
// kMats: bit t set = material type t can occur.  A kernel compiled for the
// material set of its scenes drops the other cases (smaller code, fewer
// registers); the default handles every type.
constexpr uint32_t kAllMats = (1u << 9) - 1u;
constexpr uint32_t kLambertMats = 1u << LJ_MAT_LAMBERTIAN;
constexpr uint32_t kClassicMats =
    (1u << LJ_MAT_LAMBERTIAN) | (1u << LJ_MAT_ROUGHPLASTIC) | (1u << LJ_MAT_ROUGHDIELECTRIC);
constexpr uint32_t kDisneyBsdfMats = 1u << LJ_MAT_DISNEY_BSDF;   // the combined Disney BSDF alone
template <uint32_t kMats>
LJ_HD constexpr bool has_mat(int t) { return (kMats >> t) & 1u; }
// texture slots a material type reads (the slot table in lj_gpu.h)
LJ_HD constexpr int mat_slot_count(int t) { return t == 8 ? 12 : (t == 0 || t == 6) ? 1 : (t == 7 ? 2 : 3); }
template <uint32_t kMats>
LJ_HD constexpr int max_mat_slots() {
    int n = 0;
    for (int t = 0; t < 9; t++)
        if (has_mat<kMats>(t) && mat_slot_count(t) > n) n = mat_slot_count(t);
    return n;
}

template <uint32_t kMats = kAllMats>
LJ_HD V3 bsdf_eval(const MatParams &m, const BsdfVertex &v, V3 wi, V3 wo, bool to_view = false) {
    float ax, ay;
    switch (m.type) {
    case 0:
        if (has_mat<kMats>(0)) return lambert_eval(m.s[0], v, wi, wo);
        break;
    case 1:
        if (has_mat<kMats>(1)) return plastic_eval(m, v, wi, wo);
        break;
    case 2:
        if (has_mat<kMats>(2))
            return diel_eval(DielParams{m.s[0], m.s[1], m.eta, true, m.s[2].x, 0, 0}, v, wi, wo, to_view);
        break;
    case 3:
        if (has_mat<kMats>(3)) return ddiffuse_eval(m.s[0], m.s[1].x, m.s[2].x, v, wi, wo);
        break;
    case 4:
        if (!has_mat<kMats>(4)) break;
        disney_alphas(m.s[1].x, m.s[2].x, ax, ay);
        return dmetal_eval(m.s[0], ax, ay, v, wi, wo);
    case 5:
        if (!has_mat<kMats>(5)) break;
        disney_alphas(m.s[1].x, m.s[2].x, ax, ay);
        return diel_eval(DielParams{m.s[0], sqrt3(m.s[0]), m.eta, false, 0, ax, ay}, v, wi, wo, to_view);
    case 6:
        if (!has_mat<kMats>(6)) break;
        ax = dclearcoat_eval(m.s[0].x, v, wi, wo);
        return V3{ax, ax, ax};
    case 7:
        if (has_mat<kMats>(7)) return dsheen_eval(m.s[0], m.s[1].x, v, wi, wo);
        break;
    case 8:
        if (has_mat<kMats>(8)) return disney_eval(disney_params(m), v, wi, wo, to_view);
        break;
    }
    return V3{0, 0, 0};
}
template <uint32_t kMats = kAllMats>
LJ_HD float bsdf_pdf(const MatParams &m, const BsdfVertex &v, V3 wi, V3 wo) {
    float ax, ay;
    switch (m.type) {
    case 0:
        if (has_mat<kMats>(0)) return lambert_pdf(v, wi, wo);
        break;
    case 1:
        if (has_mat<kMats>(1)) return plastic_pdf(m, v, wi, wo);
        break;
    case 2:
        if (has_mat<kMats>(2)) return diel_pdf(DielParams{m.s[0], m.s[1], m.eta, true, m.s[2].x, 0, 0}, v, wi, wo);
        break;
    case 3:
        if (has_mat<kMats>(3)) return lambert_pdf(v, wi, wo);
        break;
    case 4:
        if (!has_mat<kMats>(4)) break;
        disney_alphas(m.s[1].x, m.s[2].x, ax, ay);
        return dmetal_pdf(ax, ay, v, wi, wo);
    case 5:
        if (!has_mat<kMats>(5)) break;
        disney_alphas(m.s[1].x, m.s[2].x, ax, ay);
        return diel_pdf(DielParams{m.s[0], sqrt3(m.s[0]), m.eta, false, 0, ax, ay}, v, wi, wo);
    case 6:
        if (has_mat<kMats>(6)) return dclearcoat_pdf(m.s[0].x, v, wi, wo);
        break;
    case 7:
        if (has_mat<kMats>(7)) return lambert_pdf(v, wi, wo);
        break;
    case 8:
        if (has_mat<kMats>(8)) return disney_pdf(disney_params(m), v, wi, wo);
        break;
    }
    return 0.0f;
}
// bsdf_eval and bsdf_pdf of the same directions under one dispatch: each
// type's two bodies inline side by side, so the terms they share (half
// vector, microfacet D and G, Fresnel) are computed once.  Same values as
// the two calls.
template <uint32_t kMats = kAllMats>
LJ_HD void bsdf_eval_pdf(const MatParams &m, const BsdfVertex &v, V3 wi, V3 wo, V3 &f, float &pdf) {
    float ax, ay;
    switch (m.type) {
    case 0:
        if (!has_mat<kMats>(0)) break;
        f = lambert_eval(m.s[0], v, wi, wo);
        pdf = lambert_pdf(v, wi, wo);
        return;
    case 1:
        if (!has_mat<kMats>(1)) break;
        f = plastic_eval(m, v, wi, wo);
        pdf = plastic_pdf(m, v, wi, wo);
        return;
    case 2:
        if (!has_mat<kMats>(2)) break;
        f = diel_eval(DielParams{m.s[0], m.s[1], m.eta, true, m.s[2].x, 0, 0}, v, wi, wo, false);
        pdf = diel_pdf(DielParams{m.s[0], m.s[1], m.eta, true, m.s[2].x, 0, 0}, v, wi, wo);
        return;
    case 3:
        if (!has_mat<kMats>(3)) break;
        f = ddiffuse_eval(m.s[0], m.s[1].x, m.s[2].x, v, wi, wo);
        pdf = lambert_pdf(v, wi, wo);
        return;
    case 4:
        if (!has_mat<kMats>(4)) break;
        disney_alphas(m.s[1].x, m.s[2].x, ax, ay);
        f = dmetal_eval(m.s[0], ax, ay, v, wi, wo);
        pdf = dmetal_pdf(ax, ay, v, wi, wo);
        return;
    case 5:
        if (!has_mat<kMats>(5)) break;
        disney_alphas(m.s[1].x, m.s[2].x, ax, ay);
        f = diel_eval(DielParams{m.s[0], sqrt3(m.s[0]), m.eta, false, 0, ax, ay}, v, wi, wo, false);
        pdf = diel_pdf(DielParams{m.s[0], sqrt3(m.s[0]), m.eta, false, 0, ax, ay}, v, wi, wo);
        return;
    case 6:
        if (!has_mat<kMats>(6)) break;
        ax = dclearcoat_eval(m.s[0].x, v, wi, wo);
        f = V3{ax, ax, ax};
        pdf = dclearcoat_pdf(m.s[0].x, v, wi, wo);
        return;
    case 7:
        if (!has_mat<kMats>(7)) break;
        f = dsheen_eval(m.s[0], m.s[1].x, v, wi, wo);
        pdf = lambert_pdf(v, wi, wo);
        return;
    case 8:
        if (!has_mat<kMats>(8)) break;
        f = disney_eval(disney_params(m), v, wi, wo, false);
        pdf = disney_pdf(disney_params(m), v, wi, wo);
        return;
    }
    f = V3{0, 0, 0};
    pdf = 0.0f;
}

template <uint32_t kMats = kAllMats>
LJ_HD BsdfSample bsdf_sample(const MatParams &m, const BsdfVertex &v, V3 wi, float u0, float u1, float w) {
    float ax, ay;
    switch (m.type) {
    case 0:
        if (has_mat<kMats>(0)) return lambert_sample(v, wi, u0, u1, 1.0f);
        break;
    case 1:
        if (has_mat<kMats>(1)) return plastic_sample(m, v, wi, u0, u1, w);
        break;
    case 2:
        if (has_mat<kMats>(2))
            return diel_sample(DielParams{m.s[0], m.s[1], m.eta, true, m.s[2].x, 0, 0}, v, wi, u0, u1, w, 0.0f);
        break;
    case 3:
        if (has_mat<kMats>(3)) return lambert_sample(v, wi, u0, u1, m.s[1].x);
        break;
    case 4:
        if (!has_mat<kMats>(4)) break;
        disney_alphas(m.s[1].x, m.s[2].x, ax, ay);
        return dmetal_sample(ax, ay, m.s[1].x, v, wi, u0, u1);
    case 5:
        if (!has_mat<kMats>(5)) break;
        disney_alphas(m.s[1].x, m.s[2].x, ax, ay);
        return diel_sample(DielParams{m.s[0], sqrt3(m.s[0]), m.eta, false, 0, ax, ay}, v, wi, u0, u1, w, m.s[1].x);
    case 6:
        if (has_mat<kMats>(6)) return dclearcoat_sample(m.s[0].x, v, wi, u0, u1);
        break;
    case 7:
        if (has_mat<kMats>(7)) return lambert_sample(v, wi, u0, u1, 1.0f);
        break;
    case 8:
        if (has_mat<kMats>(8)) return disney_sample(disney_params(m), v, wi, u0, u1, w);
        break;
    }
    return no_sample();
}

// Packed-parameter layout of the BSDF batch API: slot widths per type.
LJ_HD int slot_width(int type, int slot) {
    switch (type) {
    case 0: return slot == 0 ? 3 : 0;
    case 1: case 2: return slot < 2 ? 3 : (slot == 2 ? 1 : 0);
    case 3: case 4: case 5: return slot == 0 ? 3 : (slot < 3 ? 1 : 0);
    case 6: return slot == 0 ? 1 : 0;
    case 7: return slot == 0 ? 3 : (slot == 1 ? 1 : 0);
    case 8: return slot == 0 ? 3 : (slot < 12 ? 1 : 0);
    }
    return 0;
}
LJ_HD int bsdf_param_count(int type) {
    int n = 0;
    for (int s = 0; s < kMatSlots; s++) n += slot_width(type, s);
    return n + 1;
}

}  // namespace lj
