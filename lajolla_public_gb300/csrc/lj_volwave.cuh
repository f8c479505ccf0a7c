// The shade steps of the volumetric path tracer (v6), shared by the
// single-scene renderer (lj_volpath.cu) and the server (lj_server.cu): the
// GPU form of vol_path_tracing (src/vol_path_tracing.h:59-64, a stub in the
// reference; the algorithm is the one handouts/homework2.tex:303-816
// specifies, restated in oracle/lj_oracle.cpp with the same random-number
// order).  Per queue entry, after its closest hit:
//   a  free-flight delta tracking over [0, t_hit) with the chromatic
//      majorant (one channel sampled per segment), emission with MIS, the
//      depth limits; index-matching surfaces are passed; at a real
//      scattering point or a surface with a material, the light sample of
//      NEE and a request in the NEE queue
//   b  per request, the shadow ray's walk through index-matching surfaces,
//      then ratio tracking through media for an unblocked ray
//   c  per request, the MIS-weighted contribution, phase / BSDF sampling,
//      Russian roulette, the next ray.
// A store decides where the state lives (fixed slots or queue order), as
// for the path tracer.
#pragma once

#include "../../include/lj_gpu.h"
#include "lj_internal.h"
#include "lj_phase.cuh"
#include "lj_shade.cuh"
#include "lj_trace.cuh"
#include "lj_wavefront.cuh"

namespace lj {

constexpr int kMaxShadowSegments = 1024;

// State of one volumetric path between two events.
struct VolState {
    int slot, job, pixel;
    uint64_t rng;
    float4 beta;   // xyz throughput, w eta_scale
    float4 L;      // xyz radiance, w dir_pdf (solid angle) of the last scattering
    float4 neep;   // xyz position of the last vertex that could issue NEE
    float4 mdir;   // xyz product of free-flight pdfs since that vertex
    float4 mnee;   // xyz product of ratio-tracking pdfs since that vertex
    int4 st;       // x medium, y bounces, z never_scatter, w first ray
};

LJ_D float chan(V3 v, int c) { return c == 0 ? v.x : (c == 1 ? v.y : v.z); }
LJ_D V3 vexp(V3 v) { return V3{expf(v.x), expf(v.y), expf(v.z)}; }

// GridVolume lookup (src/volume.h:44-81): trilinear over the voxel corners,
// zero outside the box.  The grid coordinate is (p - pmin) * gscale, one
// multiply per axis (the reference divides by the extent, then scales).
LJ_D V3 vol_lookup(const VolRec &v, V3 p) {
    if (v.kind == 0) return V3{v.value[0], v.value[1], v.value[2]};
    const float nx = (p.x - v.pmin[0]) * v.gscale[0];
    const float ny = (p.y - v.pmin[1]) * v.gscale[1];
    const float nz = (p.z - v.pmin[2]) * v.gscale[2];
    if (!(nx >= 0.f && nx <= (float)(v.res[0] - 1) && ny >= 0.f && ny <= (float)(v.res[1] - 1) && nz >= 0.f &&
          nz <= (float)(v.res[2] - 1)))
        return V3{0, 0, 0};
    int x0 = min(max((int)nx, 0), v.res[0] - 1), y0 = min(max((int)ny, 0), v.res[1] - 1),
        z0 = min(max((int)nz, 0), v.res[2] - 1);
    int x1 = min(x0 + 1, v.res[0] - 1), y1 = min(y0 + 1, v.res[1] - 1), z1 = min(z0 + 1, v.res[2] - 1);
    float dx = nx - x0, dy = ny - y0, dz = nz - z0;
    const float w000 = (1 - dx) * (1 - dy) * (1 - dz), w100 = dx * (1 - dy) * (1 - dz);
    const float w010 = (1 - dx) * dy * (1 - dz), w110 = dx * dy * (1 - dz);
    const float w001 = (1 - dx) * (1 - dy) * dz, w101 = dx * (1 - dy) * dz;
    const float w011 = (1 - dx) * dy * dz, w111 = dx * dy * dz;
    const V3 cs{v.cscale[0], v.cscale[1], v.cscale[2]};
    if (v.channels == 1) {   // scalar grid times the channel scale: one 4-byte load per corner
        auto at = [&](int x, int y, int z) { return __ldg(v.data1 + ((size_t)z * v.res[1] + y) * v.res[0] + x); };
        const float r = at(x0, y0, z0) * w000 + at(x1, y0, z0) * w100 + at(x0, y1, z0) * w010 +
                        at(x1, y1, z0) * w110 + at(x0, y0, z1) * w001 + at(x1, y0, z1) * w101 +
                        at(x0, y1, z1) * w011 + at(x1, y1, z1) * w111;
        return cs * (r * v.scale);
    }
    auto at = [&](int x, int y, int z) {
        const float4 q = __ldg(v.data + ((size_t)z * v.res[1] + y) * v.res[0] + x);
        return V3{q.x, q.y, q.z};
    };
    V3 r = at(x0, y0, z0) * w000 + at(x1, y0, z0) * w100 + at(x0, y1, z0) * w010 + at(x1, y1, z0) * w110 +
           at(x0, y0, z1) * w001 + at(x1, y0, z1) * w101 + at(x0, y1, z1) * w011 + at(x1, y1, z1) * w111;
    return (r * v.scale) * cs;
}
// slab test against the density grid box (src/volume.h:124-144); tfar = inf
LJ_D bool vol_box_hit(const VolRec &v, V3 o, V3 d) {
    if (v.kind == 0) return true;
    float t0 = 0.f, t1 = __int_as_float(0x7f800000);
    // __frcp_rn: the correctly rounded reciprocal, the same bits as 1.0f / x
    // without the division sequence (this test runs in the ratio-tracking loop)
    const float oo[3] = {o.x, o.y, o.z}, inv[3] = {__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z)};
    for (int i = 0; i < 3; i++) {
        float tn = (v.pmin[i] - oo[i]) * inv[i];
        float tf = (v.pmax[i] - oo[i]) * inv[i];
        if (tn > tf) { float x = tn; tn = tf; tf = x; }
        t0 = tn > t0 ? tn : t0;
        t1 = tf < t1 ? tf : t1;
        if (t0 > t1) return false;
    }
    return true;
}
LJ_D V3 majorant(const MediumRec &m, V3 o, V3 d) {
    if (m.kind == 0) return V3{m.sigma_a[0] + m.sigma_s[0], m.sigma_a[1] + m.sigma_s[1], m.sigma_a[2] + m.sigma_s[2]};
    if (vol_box_hit(m.density, o, d)) return V3{m.density.max_value[0], m.density.max_value[1], m.density.max_value[2]};
    return V3{0, 0, 0};
}
// sigma_t = sigma_s + sigma_a at p: the density itself for a
// heterogeneous medium (sigma_s = density * albedo, sigma_a = density *
// (1 - albedo)), so the albedo is looked up only where sigma_s is needed.
LJ_D V3 sigma_t_at(const MediumRec &m, V3 p) {
    if (m.kind == 0) return V3{m.sigma_a[0] + m.sigma_s[0], m.sigma_a[1] + m.sigma_s[1], m.sigma_a[2] + m.sigma_s[2]};
    return vol_lookup(m.density, p);
}
// sigma_s at p, given sigma_t there
LJ_D V3 sigma_s_at(const MediumRec &m, V3 p, V3 st) {
    if (m.kind == 0) return V3{m.sigma_s[0], m.sigma_s[1], m.sigma_s[2]};
    return st * vol_lookup(m.albedo, p);
}
LJ_D int update_medium(const Vertex &v, V3 dir, int medium) {
    if (v.interior_medium != v.exterior_medium) return dot(dir, v.ng) > 0.f ? v.exterior_medium : v.interior_medium;
    return medium;
}

// ---- NEE (next event estimation) in three steps ----
// A path that reaches a real scattering point or a surface with a material
// issues one NEE request: vol_segment_a draws the light sample (4 random
// numbers, as the reference's NEE starts) and appends the request;
// vol_nee_b walks the shadow ray through index-matching surfaces and, when
// no opaque surface or depth limit blocks it, ratio-tracks it through the
// media, drawing from the path's stream (a blocked ray draws nothing);
// vol_segment_c turns its transmittance into the MIS-weighted contribution and
// continues the path with the stream where the shadow loop left it (phase or
// BSDF sampling, Russian roulette).  The random-number order per path is that
// of one sequential NEE call of the oracle; the shadow loop, which does most
// of the grid lookups, runs in a small kernel of its own.
// Requests from scattering points fill the queue from its front, requests
// from surfaces from its back, so that each instance of the c step reads a
// contiguous range (and the warps of the b step see one kind mostly).
constexpr int kNeeSurface = 1, kNeeEnv = 2, kNeeLight = 4, kNeeFirst = 8;

struct NeeQueue {
    int cap;          // capacity (entries of the path queue)
    int *count;       // [0] requests from scattering points (front), [1] from surfaces (back)
    int *entry;       // queue entry of the path
    float4 *org;      // xyz: NEE origin (scattering point or surface vertex)
    float4 *dir;      // xyz: direction to the light sample
    float4 *lp;       // xyz: light sample point, w: light id (int bits)
    float4 *ln;       // xyz: light sample normal, w: kNee* flags (int bits)
    float4 *ss;       // xyz: sigma_s at the scattering point
    int4 *med;        // x: medium the shadow ray starts in, y: path bounces, z: pixel
    uint64_t *rng;    // PCG state after the light sample (a), after the shadow loop (b)
    float4 *T;        // b: xyz transmittance, w: 1 = blocked (no contribution)
    float4 *pn;       // b: xyz product of ratio-tracking pdfs
    float4 *pd;       // b: xyz product of free-flight pdfs
    // request r of the b step's range [0, count[0] + count[1])
    LJ_D int req(int r, int n_front) const { return r < n_front ? r : cap - 1 - (r - n_front); }
};

// The b step's result of request k for the c step: written to the request.
struct NeeToQueue {
    const NeeQueue &nq;
    LJ_D void operator()(int k, uint64_t rng, V3 T, bool blocked, V3 p_nee, V3 p_dir, float4, float4, float4,
                         float4) const {
        nq.rng[k] = rng;
        nq.T[k] = make_float4(T.x, T.y, T.z, blocked ? 1.0f : 0.0f);
        nq.pn[k] = make_float4(p_nee.x, p_nee.y, p_nee.z, 0.0f);
        nq.pd[k] = make_float4(p_dir.x, p_dir.y, p_dir.z, 0.0f);
    }
};

// Shadow loop of request k (b step).  max_depth: the job's.  finish(k, PCG
// state, transmittance, blocked, ratio-tracking pdf product, free-flight pdf
// product, and the request's org / dir / lp / ln as read here) receives the
// result: NeeToQueue hands it to a c step through the request, a caller may
// instead continue the path at once.
template <class Finish = NeeToQueue>
LJ_D void vol_nee_b(const DevScene &sc, const NeeQueue &nq, int k, int max_depth, int *status,
                    unsigned long long *seg_stat, const Finish &finish) {
    const float4 o4 = nq.org[k], d4 = nq.dir[k], lp4 = nq.lp[k], ln4 = nq.ln[k];
    const int4 md = nq.med[k];
    const int flags = __float_as_int(ln4.w);
    V3 T{1, 1, 1}, p_nee{1, 1, 1}, p_dir{1, 1, 1};
    bool blocked = (flags & kNeeLight) == 0;
    Pcg rng;
    rng.state = nq.rng[k];
    rng.inc = ((uint64_t)md.z << 1u) | 1u;
    const bool env = (flags & kNeeEnv) != 0;
    const V3 dir{d4.x, d4.y, d4.z}, lp{lp4.x, lp4.y, lp4.z}, org{o4.x, o4.y, o4.z};
    const float inf = __int_as_float(0x7f800000);
    const int bounces = md.y;
    // pass 1: the shadow ray's path through index-matching surfaces, without
    // random numbers; an opaque surface or the depth limit blocks it, and
    // then no ratio tracking runs (the contribution is zero either way)
    TraceHit h0{0.0f, -1, 0.0f, 0.0f};
    bool hit0 = false;
    if (!blocked) {
        V3 p0 = org;
        float oeps = (flags & kNeeSurface) ? sc.eps : 0.0f;
        for (int seg = 0; seg < kMaxShadowSegments; seg++) {
            const float dist = env ? inf : length(lp - p0);
            const float tmax = env ? inf : (1.0f - sc.eps) * dist;
            TraceHit h{0.0f, -1, 0.0f, 0.0f};
            int ovf = 0;
            const bool hit = trace_bvh<false>(sc.bvh, p0, dir, oeps, tmax, h, &ovf);
            if (ovf) atomicOr(status, kStatusStackOverflow);
            if (seg == 0) {
                h0 = h;
                hit0 = hit;
            }
            if (!hit) break;
            if (sc.shapes[__ldg(sc.prim_shape + h.prim)].material_id >= 0 ||
                (max_depth != -1 && bounces + seg + 2 >= max_depth)) {
                blocked = true;
                break;
            }
            p0 = p0 + dir * h.t;
            oeps = sc.eps;
        }
    }
    // pass 2: the same segments again, with ratio tracking through media
    if (!blocked) {
        int smed = md.x;
        int sbounces = 0;
        V3 p0 = org;
        float oeps = (flags & kNeeSurface) ? sc.eps : 0.0f;
        int segs = 0;
        for (int seg = 0; seg < kMaxShadowSegments; seg++) {
            segs++;
            float dist = env ? inf : length(lp - p0);
            float tmax = env ? inf : (1.0f - sc.eps) * dist;
            TraceHit h = h0;
            bool hit = hit0;
            if (seg > 0) {
                int ovf = 0;
                hit = trace_bvh<false>(sc.bvh, p0, dir, oeps, tmax, h, &ovf);
                if (ovf) atomicOr(status, kStatusStackOverflow);
            }
            float next_t = hit ? h.t : dist;
            if (smed >= 0) {
                // ratio tracking over [0, next_t).  The sample positions
                // depend on the random numbers only, so two steps are drawn
                // ahead and their density lookups issued together; a step
                // that was drawn but not reached (transmittance zero) gives
                // its random number back.
                const MediumRec &m = sc.media[smed];
                const V3 maj = majorant(m, p0, dir);
                const float inv_mmax = 1.0f / max3(maj);
                const V3 maj_n = maj * inv_mmax;
                const int c = min(max((int)(pcg_uniform(rng) * 3.0f), 0), 2);
                const float majc = chan(maj, c), inv_majc = 1.0f / majc;
                const int nmax = sc.max_null_collisions;
                float acc = 0.0f;
                int it = 0;
                while (majc > 0.0f && it < nmax) {
                    const float tA = -logf(1.0f - pcg_uniform(rng)) * inv_majc;
                    const float dtA = next_t - acc;
                    const float accA = fminf(acc + tA, next_t);
                    if (!(tA < dtA)) {   // past next_t
                        const V3 e = vexp(maj * -dtA);
                        T = T * e;
                        p_nee = p_nee * e;
                        p_dir = p_dir * e;
                        break;
                    }
                    const uint64_t after_a = rng.state;
                    const bool have_b = it + 1 < nmax;
                    float tB = 0.0f, dtB = 0.0f, accB = accA;
                    if (have_b) {
                        tB = -logf(1.0f - pcg_uniform(rng)) * inv_majc;
                        dtB = next_t - accA;
                        accB = fminf(accA + tB, next_t);
                    }
                    const bool inside_b = have_b && tB < dtB;
                    const V3 stA = sigma_t_at(m, p0 + dir * accA);
                    const V3 stB = sigma_t_at(m, p0 + dir * (inside_b ? accB : accA));
                    const V3 eA = vexp(maj * -tA);
                    const V3 fA = eA * (maj - stA) * inv_mmax;
                    T = T * fA;
                    p_dir = p_dir * fA;
                    p_nee = p_nee * eA * maj_n;
                    it++;
                    if (max3(T) <= 0.0f) {
                        rng.state = after_a;
                        break;
                    }
                    if (!have_b) break;
                    acc = accB;
                    if (!inside_b) {
                        const V3 e = vexp(maj * -dtB);
                        T = T * e;
                        p_nee = p_nee * e;
                        p_dir = p_dir * e;
                        break;
                    }
                    const V3 eB = vexp(maj * -tB);
                    const V3 fB = eB * (maj - stB) * inv_mmax;
                    T = T * fB;
                    p_dir = p_dir * fB;
                    p_nee = p_nee * eB * maj_n;
                    it++;
                    if (max3(T) <= 0.0f) break;
                }
            }
            if (!hit) break;
            int shape = __ldg(sc.prim_shape + h.prim);
            if (sc.shapes[shape].material_id >= 0) {   // an opaque surface blocks the light
                blocked = true;
                break;
            }
            sbounces++;
            if (max_depth != -1 && bounces + sbounces + 1 >= max_depth) {
                blocked = true;
                break;
            }
            Vertex sv = make_vertex(sc, p0, dir, h.t, h.prim, h.u, h.v, 0.0f);
            smed = update_medium(sv, dir, smed);
            p0 = p0 + dir * next_t;
            oeps = sc.eps;
            if (seg == kMaxShadowSegments - 1) atomicOr(status, kStatusBounceCap);
        }
        if (seg_stat) counter_add(seg_stat, blocked ? 0u : (unsigned)segs);
    }
    finish(k, rng.state, T, blocked, p_nee, p_dir, o4, d4, lp4, ln4);
}

// a step: one queue entry up to its NEE request.  Free-flight delta
// tracking over [0, t_hit) with the chromatic majorant (one channel sampled
// per segment); emission with MIS at a light; depth limits; index-matching
// surfaces are passed here.  Paths that end or pass a surface are emitted;
// the others are saved in place and get a request in nq.
// stats: [3] null collisions, [4] real collisions.
template <class Store>
LJ_D void vol_segment_a(const DevScene &sc, const Store &store, int i, const ShadeCfg &cfg, const NeeQueue &nq,
                        int *status, unsigned long long *stats) {
    const float inf = __int_as_float(0x7f800000);
    VolState vs;
    float4 r0, r1, hit;
    store.load(i, vs, r0, r1, hit);
    V3 ro{r0.x, r0.y, r0.z}, rd{r1.x, r1.y, r1.z};
    int prim = __float_as_int(hit.y);
    V3 beta{vs.beta.x, vs.beta.y, vs.beta.z}, L{vs.L.x, vs.L.y, vs.L.z}, neep{vs.neep.x, vs.neep.y, vs.neep.z};
    V3 mdir{vs.mdir.x, vs.mdir.y, vs.mdir.z}, mnee{vs.mnee.x, vs.mnee.y, vs.mnee.z};
    float dir_pdf = vs.L.w;
    int medium = vs.st.x, bounces = vs.st.y;
    bool never_scatter = vs.st.z != 0, first = vs.st.w != 0;
    Pcg rng;
    rng.state = vs.rng;
    rng.inc = ((uint64_t)vs.pixel << 1u) | 1u;
    bool alive = true;

    float t_hit = prim >= 0 ? hit.x : inf;
    bool scatter = false;
    V3 p_scatter{0, 0, 0}, ss_scatter{0, 0, 0};
    if (medium >= 0) {
        // delta tracking with the chromatic majorant: a sampled collision
        // is real with probability sigma_t / majorant in channel c
        const MediumRec &m = sc.media[medium];
        const V3 maj = majorant(m, ro, rd);
        const float inv_mmax = 1.0f / max3(maj);
        const V3 maj_n = maj * inv_mmax;
        const int c = min(max((int)(pcg_uniform(rng) * 3.0f), 0), 2);
        const float majc = chan(maj, c), inv_majc = 1.0f / majc;
        float acc = 0.0f;
        V3 T{1, 1, 1}, pd{1, 1, 1}, pn{1, 1, 1};
        unsigned nulls = 0;
        for (int it = 0; it < sc.max_null_collisions; it++) {
            if (majc <= 0.0f) break;
            float t = -logf(1.0f - pcg_uniform(rng)) * inv_majc;
            float dt = t_hit - acc;
            acc = fminf(acc + t, t_hit);
            if (t < dt) {
                const V3 pp = ro + rd * acc;
                const V3 stt = sigma_t_at(m, pp);
                const V3 e = vexp(maj * -t);
                if (pcg_uniform(rng) * majc < chan(stt, c)) {
                    scatter = true;
                    T = T * e * inv_mmax;
                    pd = pd * e * stt * inv_mmax;
                    p_scatter = pp;
                    ss_scatter = sigma_s_at(m, pp, stt);
                    break;
                }
                nulls++;
                const V3 f = e * (maj - stt) * inv_mmax;
                T = T * f;
                pd = pd * f;
                pn = pn * e * maj_n;
            } else {
                V3 e = vexp(maj * -dt);
                T = T * e;
                pd = pd * e;
                pn = pn * e;
                break;
            }
        }
        counter_add(stats + 3, nulls);
        counter_add(stats + 4, scatter ? 1u : 0u);
        beta = beta * T / avg3(pd);
        mdir = mdir * pd;
        mnee = mnee * pn;
    }
    Vertex vx;
    if (!scatter) {
        if (prim < 0) {
            if (sc.env.light_id >= 0) {
                V3 Le = env_emission(sc, -rd);
                if (never_scatter) {
                    L += beta * Le;
                } else {
                    float pn = __ldg(sc.light_pmf + sc.env.light_id) * env_pdf(sc, rd) * avg3(mnee);
                    float pd = dir_pdf * avg3(mdir);
                    L += beta * Le * ((pd * pd) / (pd * pd + pn * pn));
                }
            }
            alive = false;
        } else {
            vx = make_vertex(sc, ro, rd, hit.x, prim, hit.z, hit.w, first ? cfg.spread0 : 0.0f);
            if (vx.light >= 0) {
                V3 Le = light_emission(sc, vx.light, -rd, PN{vx.p, vx.ng});
                if (never_scatter) {
                    L += beta * Le;
                } else {
                    V3 dv = vx.p - neep;
                    float G = fabsf(dot(rd, vx.ng)) / dot(dv, dv);
                    float pn = __ldg(sc.light_pmf + vx.light) *
                               pdf_point_on_light(sc, vx.light, PN{vx.p, vx.ng}, neep) * avg3(mnee);
                    float pd = dir_pdf * G * avg3(mdir);
                    L += beta * Le * ((pd * pd) / (pd * pd + pn * pn));
                }
            }
        }
    }
    if (alive && cfg.max_depth != -1 && bounces == cfg.max_depth - 1) alive = false;
    if (alive && bounces > LJ_MAX_BOUNCES) {
        atomicOr(status, kStatusBounceCap);
        alive = false;
    }
    vs.beta = make_float4(beta.x, beta.y, beta.z, vs.beta.w);
    vs.L = make_float4(L.x, L.y, L.z, dir_pdf);
    vs.mdir = make_float4(mdir.x, mdir.y, mdir.z, 0.0f);
    vs.mnee = make_float4(mnee.x, mnee.y, mnee.z, 0.0f);
    if (alive && !scatter && vx.material < 0) {
        // index-matching surface: pass through
        vs.st = make_int4(update_medium(vx, rd, medium), bounces + 1, never_scatter ? 1 : 0, 0);
        vs.rng = rng.state;
        store.emit(vs, true, make_float4(vx.p.x, vx.p.y, vx.p.z, sc.eps), make_float4(rd.x, rd.y, rd.z, inf));
        return;
    }
    if (!alive) {
        vs.st = make_int4(medium, bounces, never_scatter ? 1 : 0, 0);
        vs.rng = rng.state;
        store.emit(vs, false, make_float4(0, 0, 0, 0), make_float4(0, 0, 0, inf));
        return;
    }
    // NEE request from the scattering point or the surface vertex; the light
    // sample's random numbers are drawn here, as the reference's NEE starts
    const bool surface = !scatter;
    const V3 p = surface ? vx.p : p_scatter;
    float lu0 = pcg_uniform(rng), lu1 = pcg_uniform(rng), lw = pcg_uniform(rng), sw = pcg_uniform(rng);
    int flags = (surface ? kNeeSurface : 0) | (first ? kNeeFirst : 0);
    int lid = -1, smed = medium;
    PN pl{V3{0, 0, 0}, V3{0, 0, 0}};
    V3 dir{0, 0, 1};
    if (sc.num_lights > 0) {
        lid = sample_light(sc, lw);
        pl = sample_point_on_light(sc, lid, p, lu0, lu1, sw);
        const bool env = sc.lights[lid].kind != 0;
        dir = env ? -pl.n : normalize(pl.p - p);
        if (surface) smed = update_medium(vx, dir, medium);
        flags |= kNeeLight | (env ? kNeeEnv : 0);
    }
    vs.st = make_int4(medium, bounces, never_scatter ? 1 : 0, first ? 1 : 0);
    store.save(i, vs);
    const int k = surface ? nq.cap - 1 - queue_slot(nq.count + 1) : queue_slot(nq.count);
    nq.entry[k] = i;
    nq.org[k] = make_float4(p.x, p.y, p.z, 0.0f);
    nq.dir[k] = make_float4(dir.x, dir.y, dir.z, 0.0f);
    nq.lp[k] = make_float4(pl.p.x, pl.p.y, pl.p.z, __int_as_float(lid));
    nq.ln[k] = make_float4(pl.n.x, pl.n.y, pl.n.z, __int_as_float(flags));
    nq.ss[k] = make_float4(ss_scatter.x, ss_scatter.y, ss_scatter.z, 0.0f);
    nq.med[k] = make_int4(smed, bounces, vs.pixel, 0);
    nq.rng[k] = rng.state;
}

// c step: request k's contribution (the end of the reference's NEE), then
// phase (kSurface = false: a request from a scattering point) or BSDF
// sampling, Russian roulette and the next ray.
// kMats: the material types the scenes can hold (kAllMats: any).
// The request fields the c step uses: where the light sample points, what
// the b step found (T.w = 1: blocked), sigma_s at a scattering point, the
// PCG state after the shadow loop.
struct NeeReq {
    float4 org, dir, lp, ln, T;
    V3 pn, pd;
    float4 ss;
    uint64_t rng;
};
LJ_D NeeReq load_req(const NeeQueue &nq, int k, bool surface) {
    NeeReq q;
    q.org = nq.org[k];
    q.dir = nq.dir[k];
    q.lp = nq.lp[k];
    q.ln = nq.ln[k];
    q.T = nq.T[k];
    const float4 pn4 = nq.pn[k], pd4 = nq.pd[k];
    q.pn = V3{pn4.x, pn4.y, pn4.z};
    q.pd = V3{pd4.x, pd4.y, pd4.z};
    q.ss = surface ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : nq.ss[k];
    q.rng = nq.rng[k];
    return q;
}

template <uint32_t kMats, bool kSurface, class Store>
LJ_D void vol_c_core(const DevScene &sc, const Store &store, int i, const NeeReq &rq, const ShadeCfg &cfg);

template <uint32_t kMats, bool kSurface, class Store>
LJ_D void vol_segment_c(const DevScene &sc, const Store &store, int k, const ShadeCfg &cfg, const NeeQueue &nq) {
    vol_c_core<kMats, kSurface>(sc, store, nq.entry[k], load_req(nq, k, kSurface), cfg);
}

// The c step of one request of path entry i, from its fields rq.
template <uint32_t kMats, bool kSurface, class Store>
LJ_D void vol_c_core(const DevScene &sc, const Store &store, int i, const NeeReq &rq, const ShadeCfg &cfg) {
    const float inf = __int_as_float(0x7f800000);
    VolState vs;
    float4 r0, r1, hit;
    store.load_c(i, vs, r0, r1, hit);
    const float4 o4 = rq.org, d4 = rq.dir, lp4 = rq.lp, ln4 = rq.ln, T4 = rq.T;
    const int flags = __float_as_int(ln4.w), lid = __float_as_int(lp4.w);
    constexpr bool surface = kSurface;
    const V3 ro{r0.x, r0.y, r0.z}, rd{r1.x, r1.y, r1.z};
    const V3 p{o4.x, o4.y, o4.z}, dir{d4.x, d4.y, d4.z};
    V3 beta{vs.beta.x, vs.beta.y, vs.beta.z}, L{vs.L.x, vs.L.y, vs.L.z};
    float eta_scale = vs.beta.w, dir_pdf = vs.L.w;
    int medium = vs.st.x, bounces = vs.st.y;
    bool never_scatter = vs.st.z != 0;
    Pcg rng;
    rng.state = rq.rng;
    rng.inc = ((uint64_t)vs.pixel << 1u) | 1u;
    const V3 wv = -rd;
    Vertex vx;
    MatParams mat;
    mat.type = 0;
    BsdfVertex bv{V3{0, 0, 1}, frame_from_n(V3{0, 0, 1})};
    if constexpr (surface) {
        vx = make_vertex(sc, ro, rd, hit.x, __float_as_int(hit.y), hit.z, hit.w,
                         (flags & kNeeFirst) ? cfg.spread0 : 0.0f);
        mat = resolve_material<kMats>(sc, vx.material, vx.u, vx.v, vx.uv_screen_size);
        bv = BsdfVertex{vx.ng, vx.frame};
    }
    // the NEE contribution
    V3 nee{0, 0, 0};
    const V3 T{T4.x, T4.y, T4.z};
    if (T4.w == 0.0f && max3(T) > 0.0f) {
        const bool env = (flags & kNeeEnv) != 0;
        const PN pl{V3{lp4.x, lp4.y, lp4.z}, V3{ln4.x, ln4.y, ln4.z}};
        V3 dp = pl.p - p;
        float G = env ? 1.0f : fmaxf(-dot(dir, pl.n), 0.0f) / dot(dp, dp);
        float pdf_nee = __ldg(sc.light_pmf + lid) * pdf_point_on_light(sc, lid, pl, p);
        if (G > 0.0f && pdf_nee > 0.0f) {
            V3 f;
            float pdf_dir;
            if constexpr (surface) {
                bsdf_eval_pdf<kMats>(mat, bv, wv, dir, f, pdf_dir);
            } else {
                const MediumRec &m = sc.media[medium];
                float ph = phase_eval(m.phase_kind, m.g, wv, dir);
                f = V3{ph, ph, ph};
                pdf_dir = ph;
            }
            V3 Le = light_emission(sc, lid, -dir, pl);
            float pn = pdf_nee * avg3(rq.pn);
            float pd = pdf_dir * G * avg3(rq.pd);
            float w = (pn * pn) / (pn * pn + pd * pd);
            nee = T * f * Le * (G * w / pn);
        }
    }
    bool alive = true;
    // the NEE vertex and the pdf products restart at this vertex (a path
    // that ends here needs neither)
    V3 next_o{0, 0, 0}, next_d{0, 0, 0}, neep{0, 0, 0};
    V3 mdir{1, 1, 1}, mnee{1, 1, 1};
    float next_tnear = 0.0f;
    if constexpr (!surface) {
        // phase sampling at the scattering point
        const V3 ss{rq.ss.x, rq.ss.y, rq.ss.z};
        const MediumRec &m = sc.media[medium];
        L += beta * ss * nee;
        float u0 = pcg_uniform(rng), u1 = pcg_uniform(rng);
        V3 nd = phase_sample(m.phase_kind, m.g, wv, u0, u1);
        beta = beta * ss;
        dir_pdf = phase_eval(m.phase_kind, m.g, wv, nd);
        neep = p;
        mdir = V3{1, 1, 1};
        mnee = V3{1, 1, 1};
        never_scatter = false;
        next_o = p;
        next_d = nd;
        next_tnear = 0.0f;
    } else {
        L += beta * nee;
        float b0 = pcg_uniform(rng), b1 = pcg_uniform(rng), b2 = pcg_uniform(rng);
        BsdfSample bs = bsdf_sample<kMats>(mat, bv, wv, b0, b1, b2);
        if (!bs.valid) {
            alive = false;
        } else {
            V3 f;
            float pdf;
            bsdf_eval_pdf<kMats>(mat, bv, wv, bs.dir, f, pdf);
            if (!(pdf > 0.0f)) {
                alive = false;
            } else {
                if (bs.eta != 0.0f) eta_scale /= (bs.eta * bs.eta);
                beta = beta * f / pdf;
                dir_pdf = pdf;
                neep = vx.p;
                mdir = V3{1, 1, 1};
                mnee = V3{1, 1, 1};
                never_scatter = false;
                medium = update_medium(vx, bs.dir, medium);
                next_o = vx.p;
                next_d = bs.dir;
                next_tnear = sc.eps;
            }
        }
    }
    if (alive) {
        if (bounces >= cfg.rr_depth) {
            float rr = fminf(max3(beta) / eta_scale, 0.95f);
            if (pcg_uniform(rng) > rr) alive = false;
            else beta = beta / rr;
        }
        bounces++;
    }
    vs.beta = make_float4(beta.x, beta.y, beta.z, eta_scale);
    vs.L = make_float4(L.x, L.y, L.z, dir_pdf);
    vs.neep = make_float4(neep.x, neep.y, neep.z, 0.0f);
    vs.mdir = make_float4(mdir.x, mdir.y, mdir.z, 0.0f);
    vs.mnee = make_float4(mnee.x, mnee.y, mnee.z, 0.0f);
    vs.st = make_int4(medium, bounces, never_scatter ? 1 : 0, 0);
    vs.rng = rng.state;
    store.emit(vs, alive, make_float4(next_o.x, next_o.y, next_o.z, next_tnear),
               make_float4(next_d.x, next_d.y, next_d.z, inf));
}

// A value the compiler must take as it is: no multiply that produced it is
// fused into an add that uses it, as when it went through memory.
LJ_D float opaque(float x) {
    asm volatile("" : "+f"(x));
    return x;
}

// The b step of a request from a scattering point goes on with its c step at
// once (phase sampling needs no material code): the transmittance and the
// pdf products stay in registers instead of a round trip through the
// request, and the request is not read again.  The pdf products pass
// through opaque() so that the c step rounds them exactly as when they were
// stored, and the path's image does not change.
template <class Store>
struct NeeToPhase {
    const DevScene &sc;
    const Store &store;
    const NeeQueue &nq;
    ShadeCfg cfg;
    LJ_D void operator()(int k, uint64_t rng, V3 T, bool blocked, V3 p_nee, V3 p_dir, float4 o4, float4 d4,
                         float4 lp4, float4 ln4) const {
        NeeReq rq;
        rq.org = o4;
        rq.dir = d4;
        rq.lp = lp4;
        rq.ln = ln4;
        rq.T = make_float4(T.x, T.y, T.z, blocked ? 1.0f : 0.0f);
        rq.pn = V3{opaque(p_nee.x), opaque(p_nee.y), opaque(p_nee.z)};
        rq.pd = V3{opaque(p_dir.x), opaque(p_dir.y), opaque(p_dir.z)};
        rq.ss = nq.ss[k];
        rq.rng = rng;
        vol_c_core<kAllMats, false>(sc, store, nq.entry[k], rq, cfg);
    }
};

}  // namespace lj
