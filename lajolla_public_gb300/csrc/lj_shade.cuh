// Shading-point construction, textures and lights on the device (FP32).
//
//   hit -> PathVertex          src/intersection.cpp:36-65
//   compute_shading_info       src/shapes/triangle_mesh.inl:77-169, sphere.inl:243-268
//   textures                   src/texture.h:117-159, mipmap lookup src/mipmap.h:52-88
//   light selection            src/scene.cpp:61-67 + src/table_dist.cpp:27-33
//   sample/pdf point on light  src/shapes/triangle_mesh.inl:24-58,
//                              src/shapes/sphere.inl:164-238, src/lights/envmap.inl:7-42
//   emission                   src/lights/diffuse_area_light.inl:15-20, envmap.inl:44-73
//   TableDist2D sample / pdf   src/table_dist.cpp:116-151
#pragma once

#include "lj_bsdf.cuh"
#include "lj_scene.cuh"

namespace lj {

struct PN {
    V3 p, n;
};

struct Vertex {
    V3 p, ng;
    Frame frame;
    float u, v;          // texture uv
    float uv_screen_size;
    float mean_curvature;
    int shape, material, light;
    int interior_medium, exterior_medium;
};

LJ_D V3 vload3(const float *a, int i) { return V3{__ldg(a + 3 * i), __ldg(a + 3 * i + 1), __ldg(a + 3 * i + 2)}; }

// first index k in [0, n] with cdf[k] > u, minus one, clamped to [0, n-1]
// (std::upper_bound over n+1 entries, src/table_dist.cpp:27-33)
LJ_D int sample_cdf(const float *cdf, int n, float u) {
    int lo = 0, hi = n + 1;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (__ldg(cdf + mid) > u) hi = mid;
        else lo = mid + 1;
    }
    return min(max(lo - 1, 0), n - 1);
}

LJ_D V3 coordinate_dpdu(V3 n, V3 &dpdv) {
    Frame f = frame_from_n(n);
    dpdv = f.y;
    return f.x;
}

// Build the shading vertex of a hit (prim, t, u, v) on ray (o, d).
// ray_spread: primary rays carry 0.25 / max(w, h) (src/ray.h:35-37), every
// later ray a zero RayDifferential (src/path_tracing.h:237), so uv_screen_size
// is non-zero only at the primary hit.
LJ_D Vertex make_vertex(const DevScene &sc, V3 o, V3 d, float t, int prim, float bu, float bv,
                        float ray_spread) {
    Vertex vx;
    vx.p = o + d * t;
    int shape = __ldg(sc.prim_shape + prim);
    const ShapeRec &sh = sc.shapes[shape];
    vx.shape = shape;
    vx.material = sh.material_id;
    vx.light = sh.area_light_id;
    vx.interior_medium = sh.interior_medium_id;
    vx.exterior_medium = sh.exterior_medium_id;
    float inv_uv_size = 1.0f;
    if (prim < sc.num_tris) {
        int i0 = __ldg(sc.tri_vidx + prim * 3), i1 = __ldg(sc.tri_vidx + prim * 3 + 1),
            i2 = __ldg(sc.tri_vidx + prim * 3 + 2);
        V3 p0 = vload3(sc.vpos, i0), p1 = vload3(sc.vpos, i1), p2 = vload3(sc.vpos, i2);
        vx.ng = normalize(xcross(xsub(p1, p0), xsub(p2, p0)));
        float b0 = 1.0f - bu - bv;
        float uv0x = 0, uv0y = 0, uv1x = 1, uv1y = 0, uv2x = 1, uv2y = 1;
        if (sh.has_uvs) {
            uv0x = __ldg(sc.vuv + 2 * i0); uv0y = __ldg(sc.vuv + 2 * i0 + 1);
            uv1x = __ldg(sc.vuv + 2 * i1); uv1y = __ldg(sc.vuv + 2 * i1 + 1);
            uv2x = __ldg(sc.vuv + 2 * i2); uv2y = __ldg(sc.vuv + 2 * i2 + 1);
        }
        vx.u = b0 * uv0x + bu * uv1x + bv * uv2x;
        vx.v = b0 * uv0y + bu * uv1y + bv * uv2y;
        float dsx = uv2x - uv0x, dsy = uv2y - uv0y;   // duv/ds
        float dtx = uv2x - uv1x, dty = uv2y - uv1y;   // duv/dt
        float det = dsx * dty - dtx * dsy;
        float dsdu = dty / det, dtdu = -dsy / det, dsdv = dtx / det, dtdv = -dsx / det;
        V3 dpdu, dpdv;
        if (fabsf(det) > 1e-8f) {
            V3 dpds = p2 - p0, dpdt = p2 - p1;
            dpdu = dpds * dsdu + dpdt * dtdu;
            dpdv = dpds * dsdv + dpdt * dtdv;
        } else {
            dpdu = coordinate_dpdu(vx.ng, dpdv);
        }
        V3 sn = vx.ng;
        float mc = 0.0f;
        V3 tangent, bitangent;
        if (sh.has_normals) {
            V3 n0 = vload3(sc.vnrm, i0), n1 = vload3(sc.vnrm, i1), n2 = vload3(sc.vnrm, i2);
            sn = normalize(n0 * b0 + n1 * bu + n2 * bv);
            tangent = normalize(dpdu - sn * dot(sn, dpdu));
            V3 dnds = n2 - n0, dndt = n2 - n1;
            V3 dndu = dnds * dsdu + dndt * dtdu;
            V3 dndv = dnds * dsdv + dndt * dtdv;
            bitangent = normalize(cross(sn, tangent));
            mc = (dot(dndu, tangent) + dot(dndv, bitangent)) * 0.5f;
        } else {
            tangent = normalize(dpdu - sn * dot(sn, dpdu));
            bitangent = normalize(cross(sn, tangent));
        }
        vx.frame = Frame{tangent, bitangent, sn};
        vx.mean_curvature = mc;
        inv_uv_size = fmaxf(length(dpdu), length(dpdv));
    } else {
        V3 c{sh.cx, sh.cy, sh.cz};
        float r = sh.radius;
        V3 gn = vx.p - c;
        vx.ng = normalize(gn);
        V3 cart = gn / r;
        float elev = acosf(clampf(cart.y, -1.0f, 1.0f));
        float az = atan2f(cart.z, cart.x);
        float st0 = az * kInvTwoPi, st1 = elev * kInvPi;
        // the reference feeds st (not the angles) into the trig terms
        float s0, c0, s1, c1;
        sincosf(st0, &s0, &c0);
        sincosf(st1, &s1, &c1);
        V3 dpdu{-r * s0 * s1, r * c0 * s1, 0.0f};
        V3 dpdv{r * c0 * c1, r * s0 * c1, -r * s1};
        V3 tangent = normalize(dpdu - vx.ng * dot(vx.ng, dpdu));
        vx.frame = Frame{tangent, normalize(cross(vx.ng, tangent)), vx.ng};
        vx.u = st0;
        vx.v = st1;
        vx.mean_curvature = 1.0f / r;
        inv_uv_size = (length(dpdu) + length(dpdv)) * 0.5f;
    }
    float ray_radius = ray_spread * t * length(d);
    vx.uv_screen_size = ray_radius / inv_uv_size;
    if (dot(vx.ng, vx.frame.n) < 0.0f) vx.ng = -vx.ng;
    return vx;
}

// ---- camera: sample_primary (src/camera.cpp:23-47) with the pixel filter
// importance sampled inside the pixel (src/filters/*.inl) ----
LJ_D void camera_ray(const CamRec &c, float sx, float sy, V3 &o, V3 &d) {
    float px = sx * c.w, py = sy * c.h;
    float dx = px - floorf(px), dy = py - floorf(py);
    float ox, oy;
    if (c.filter_kind == 0) {
        ox = (2.0f * dx - 1.0f) * (c.filter_param * 0.5f);
        oy = (2.0f * dy - 1.0f) * (c.filter_param * 0.5f);
    } else if (c.filter_kind == 1) {
        float h = c.filter_param * 0.5f;
        ox = dx < 0.5f ? h * (sqrtf(2.0f * dx) - 1.0f) : h * (1.0f - sqrtf(1.0f - 2.0f * (dx - 0.5f)));
        oy = dy < 0.5f ? h * (sqrtf(2.0f * dy) - 1.0f) : h * (1.0f - sqrtf(1.0f - 2.0f * (dy - 0.5f)));
    } else {
        float r = c.filter_param * sqrtf(-2.0f * logf(fmaxf(dx, 1e-8f)));
        float sp, cp;
        sincosf(kTwoPi * dy, &sp, &cp);
        ox = r * cp;
        oy = r * sp;
    }
    float rx = (floorf(px) + 0.5f + ox) / c.w, ry = (floorf(py) + 0.5f + oy) / c.h;
    const float *m = c.sample_to_cam;
    float t0 = m[0] * rx + m[1] * ry + m[3];
    float t1 = m[4] * rx + m[5] * ry + m[7];
    float t2 = m[8] * rx + m[9] * ry + m[11];
    float t3 = m[12] * rx + m[13] * ry + m[15];
    V3 pt = normalize(V3{t0 / t3, t1 / t3, t2 / t3});
    const float *w = c.cam_to_world;
    d = normalize(V3{w[0] * pt.x + w[1] * pt.y + w[2] * pt.z, w[4] * pt.x + w[5] * pt.y + w[6] * pt.z,
                     w[8] * pt.x + w[9] * pt.y + w[10] * pt.z});
    o = V3{c.org[0], c.org[1], c.org[2]};
}

// ---- textures ----
LJ_D float modf1(float a) {
    float r = fmodf(a, 1.0f);
    return r < 0.0f ? r + 1.0f : r;
}
LJ_D int modi(int a, int b) {
    int r = a % b;
    return r < 0 ? r + b : r;
}
LJ_D V3 mip_fetch(const MipLevel &lv, int x, int y) {
    const float *p = lv.rgb + ((size_t)y * lv.w + x) * 3;
    return V3{__ldg(p), __ldg(p + 1), __ldg(p + 2)};
}
// bilinear at an integer level, -0.5 shift, truncation + wrap: src/mipmap.h:52-72
LJ_D V3 mip_bilinear(const MipLevel &lv, float u, float v) {
    u = u * lv.w - 0.5f;
    v = v * lv.h - 0.5f;
    int uf = modi((int)u, lv.w), vf = modi((int)v, lv.h);
    int uc = modi(uf + 1, lv.w), vc = modi(vf + 1, lv.h);
    float uo = u - uf, vo = v - vf;
    return mip_fetch(lv, uf, vf) * ((1 - uo) * (1 - vo)) + mip_fetch(lv, uf, vc) * ((1 - uo) * vo) +
           mip_fetch(lv, uc, vf) * (uo * (1 - vo)) + mip_fetch(lv, uc, vc) * (uo * vo);
}
LJ_D V3 eval_texture(const DevScene &sc, const TexRec &t, float u, float v, float footprint) {
    if (t.kind == 0) return V3{t.v0[0], t.v0[1], t.v0[2]};
    float lu = modf1(u * t.us + t.uo), lv = modf1(v * t.vs + t.vo);
    if (t.kind == 2) {
        int x = 2 * modi((int)(lu * 2), 2) - 1, y = 2 * modi((int)(lv * 2), 2) - 1;
        return x * y == 1 ? V3{t.v0[0], t.v0[1], t.v0[2]} : V3{t.v1[0], t.v1[1], t.v1[2]};
    }
    const MipLevel *lvls = sc.image_levels + t.image_id * 8;
    int n = sc.image_num_levels[t.image_id];
    float sf = (float)max(lvls[0].w, lvls[0].h) * fmaxf(t.us, t.vs) * footprint;
    float level = log2f(sf > 1e-8f ? sf : 1e-8f);
    if (level <= 0.0f) return mip_bilinear(lvls[0], lu, lv);
    if (level < (float)(n - 1)) {
        int fl = (int)floorf(level);
        float lo = level - fl;
        return mip_bilinear(lvls[fl], lu, lv) * (1 - lo) + mip_bilinear(lvls[fl + 1], lu, lv) * lo;
    }
    return mip_bilinear(lvls[n - 1], lu, lv);
}
// Texture values of the slots the material's type reads (other slots: 0;
// slots no type of kMats reads are left unset).
template <uint32_t kMats = kAllMats>
LJ_D MatParams resolve_material(const DevScene &sc, int mid, float u, float v, float footprint) {
    const MatRec &m = sc.mats[mid];
    MatParams p;
    p.type = m.type;
    p.eta = m.eta;
    const int textured = m.textured;
    const int n = mat_slot_count(p.type);
#pragma unroll
    for (int k = 0; k < max_mat_slots<kMats>(); k++) {
        if (k >= n) p.s[k] = V3{0.0f, 0.0f, 0.0f};
        else if (textured & (1 << k)) p.s[k] = eval_texture(sc, m.tex[k], u, v, footprint);
        else p.s[k] = V3{m.tex[k].v0[0], m.tex[k].v0[1], m.tex[k].v0[2]};
    }
    return p;
}

// ---- envmap (src/lights/envmap.inl) ----
LJ_D V3 mat3_mul(const float *m, V3 v) {
    return V3{m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
              m[6] * v.x + m[7] * v.y + m[8] * v.z};
}
LJ_D void env_uv(const LightRec &l, V3 world_dir, V3 &local, float &u, float &v) {
    local = mat3_mul(l.to_local, world_dir);
    u = atan2f(local.x, -local.z) * kInvTwoPi;
    v = acosf(clampf(local.y, -1.0f, 1.0f)) * kInvPi;
    if (u < 0.0f) u += 1.0f;
}
// The reference's envmap footprint (envmap.inl:66-72) is always negative or
// NaN and is clamped to 1e-8 by lajolla's max(): every lookup is a bilinear
// fetch at mip level 0.
LJ_D V3 env_emission(const DevScene &sc, V3 view_dir) {
    const LightRec &l = sc.lights[sc.env.light_id];
    V3 local;
    float u, v;
    env_uv(l, -view_dir, local, u, v);
    return mip_bilinear(sc.env.levels[0], u, v) * l.scale;
}
LJ_D float env_pdf(const DevScene &sc, V3 world_dir_from_point) {
    const LightRec &l = sc.lights[sc.env.light_id];
    V3 local;
    float u, v;
    env_uv(l, world_dir_from_point, local, u, v);
    float se = sqrtf(clampf(1.0f - local.y * local.y, 0.0f, 1.0f));
    if (se <= 0.0f) return 0.0f;
    int w = sc.env.tw, h = sc.env.th;
    int x = (int)clampf(u * w, 0.0f, (float)(w - 1));
    int y = (int)clampf(v * h, 0.0f, (float)(h - 1));
    float pdf = __ldg(sc.env.pdf_marg + y) * __ldg(sc.env.pdf_rows + (size_t)y * w + x) * (float)w * (float)h;
    return pdf / (2.0f * kPi * kPi * se);
}
LJ_D V3 env_sample_dir(const DevScene &sc, float u0, float u1) {
    int w = sc.env.tw, h = sc.env.th;
    int yo = sample_cdf(sc.env.cdf_marg, h, u1);
    float c0 = __ldg(sc.env.cdf_marg + yo), c1 = __ldg(sc.env.cdf_marg + yo + 1);
    float dy = u1 - c0;
    if (c1 - c0 > 0.0f) dy /= (c1 - c0);
    const float *cdf = sc.env.cdf_rows + (size_t)yo * (w + 1);
    int xo = sample_cdf(cdf, w, u0);
    float r0 = __ldg(cdf + xo), r1 = __ldg(cdf + xo + 1);
    float dx = u0 - r0;
    if (r1 - r0 > 0.0f) dx /= (r1 - r0);
    float su = (xo + dx) / w, sv = (yo + dy) / h;
    float saz, caz, sel, cel;
    sincosf(su * kTwoPi, &saz, &caz);
    sincosf(sv * kPi, &sel, &cel);
    V3 ld{saz * sel, cel, -caz * sel};
    const LightRec &l = sc.lights[sc.env.light_id];
    return mat3_mul(l.to_world, ld);
}

// ---- area lights ----
LJ_D PN sample_point_on_shape(const DevScene &sc, const ShapeRec &sh, V3 ref, float u0, float u1, float w) {
    if (sh.kind == 0) {
        int t = sh.tri_begin + sample_cdf(sc.tri_cdf + sh.sampler_offset, sh.num_tris, w);
        int i0 = __ldg(sc.tri_vidx + t * 3), i1 = __ldg(sc.tri_vidx + t * 3 + 1), i2 = __ldg(sc.tri_vidx + t * 3 + 2);
        V3 v0 = vload3(sc.vpos, i0), v1 = vload3(sc.vpos, i1), v2 = vload3(sc.vpos, i2);
        V3 e1 = v1 - v0, e2 = v2 - v0;
        float a = sqrtf(clampf(u0, 0.0f, 1.0f));
        float b1 = 1.0f - a, b2 = a * u1;
        V3 gn = normalize(cross(e1, e2));
        if (sh.has_normals) {
            V3 sn = normalize(vload3(sc.vnrm, i0) * (1.0f - b1 - b2) + vload3(sc.vnrm, i1) * b1 +
                              vload3(sc.vnrm, i2) * b2);
            if (dot(gn, sn) < 0.0f) gn = -gn;
        }
        return PN{v0 + e1 * b1 + e2 * b2, gn};
    }
    V3 c{sh.cx, sh.cy, sh.cz};
    float r = sh.radius;
    V3 rc = ref - c;
    float dc2 = dot(rc, rc);
    if (dc2 < r * r) {
        float z = 1.0f - 2.0f * u0;
        float r_ = sqrtf(fmaxf(0.0f, 1.0f - z * z));
        float sp, cp;
        sincosf(kTwoPi * u1, &sp, &cp);
        V3 off{r_ * cp, r_ * sp, z};
        return PN{c + off * r, off};
    }
    // Same cone sampling as sphere.inl:164-212, written without cancellation
    // for FP32: om = 1 - cos_max, 1 - ce^2 = u om (2 - u om), and the point is
    // ref + w * ds with ds the near root along the sampled direction w.
    float dc = sqrtf(dc2);
    Frame fr = frame_from_n((c - ref) / dc);
    float sin_max_sq = r * r / dc2;
    float cos_max = sqrtf(fmaxf(0.0f, 1.0f - sin_max_sq));
    float om = sin_max_sq / (1.0f + cos_max);
    float ce = 1.0f - u0 * om;
    float se = sqrtf(fmaxf(0.0f, u0 * om * (2.0f - u0 * om)));
    // r^2 - dc^2 se^2 = dc^2 om (1 - u0) (2 - om (1 + u0))
    float disc = om * (1.0f - u0) * (2.0f - om * (1.0f + u0));
    float ds = dc * (ce - sqrtf(fmaxf(0.0f, disc)));
    float sp, cp;
    sincosf(u1 * kTwoPi, &sp, &cp);
    // the reference's normal -(sa cos, sa sin, ca) puts the point at azimuth
    // phi + pi as seen from ref
    V3 wdir = to_world(fr, V3{-se * cp, -se * sp, ce});
    V3 p = ref + wdir * ds;
    V3 n = (p - c) / r;
    return PN{p, n};
}
LJ_D float pdf_point_on_shape(const ShapeRec &sh, const PN &pn, V3 ref) {
    if (sh.kind == 0) return 1.0f / sh.total_area;
    V3 c{sh.cx, sh.cy, sh.cz};
    float r = sh.radius;
    V3 rc = ref - c;
    float dc2 = dot(rc, rc);
    if (dc2 < r * r) return 1.0f / sh.total_area;
    float cos_max = sqrtf(fmaxf(0.0f, 1.0f - r * r / dc2));
    // 1 - cos_max without cancellation for distant spheres
    float one_minus = (r * r / dc2) / (1.0f + cos_max);
    float pdf_sa = 1.0f / (kTwoPi * one_minus);
    V3 dv = pn.p - ref;
    float dist2 = dot(dv, dv);
    return pdf_sa * fabsf(dot(pn.n, dv)) * rsqrtf(dist2) / dist2;
}

LJ_D int sample_light(const DevScene &sc, float u) { return sample_cdf(sc.light_cdf, sc.num_lights, u); }

// Point (or envmap direction, stored in n as "from light") on light `lid`.
LJ_D PN sample_point_on_light(const DevScene &sc, int lid, V3 ref, float u0, float u1, float w) {
    const LightRec &l = sc.lights[lid];
    if (l.kind == 0) return sample_point_on_shape(sc, sc.shapes[l.shape_id], ref, u0, u1, w);
    V3 wd = env_sample_dir(sc, u0, u1);
    return PN{V3{0, 0, 0}, -wd};
}
LJ_D float pdf_point_on_light(const DevScene &sc, int lid, const PN &pn, V3 ref) {
    const LightRec &l = sc.lights[lid];
    if (l.kind == 0) return pdf_point_on_shape(sc.shapes[l.shape_id], pn, ref);
    return env_pdf(sc, -pn.n);
}
LJ_D V3 light_emission(const DevScene &sc, int lid, V3 view_dir, const PN &pn) {
    const LightRec &l = sc.lights[lid];
    if (l.kind == 0) {
        if (dot(pn.n, view_dir) <= 0.0f) return V3{0, 0, 0};
        return V3{l.intensity[0], l.intensity[1], l.intensity[2]};
    }
    return env_emission(sc, view_dir);
}

}  // namespace lj
