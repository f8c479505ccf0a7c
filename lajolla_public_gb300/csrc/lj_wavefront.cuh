// Wavefront state and the shade step of the unidirectional path tracer
// (src/path_tracing.h:7-325), shared by the single-scene renderer
// (lj_path.cu) and the multi-job server (lj_server.cu).
//
// The shade step reads one path's state and hit, and hands the outcome (the
// next ray, if any, and the NEE shadow ray with its contribution) to a path
// store, which decides where state lives:
//   OrderedPaths (single-scene renderer) state in queue order: an entry of
//                the next queue is written with the path's whole state, so
//                every kernel reads its queue contiguously; a finished
//                path's radiance goes to its sample slot.
//   the server's store does the same across jobs (lj_server.cu).
// The random-number order per path is the reference's: 2 for the screen
// position, then per bounce 4 for light sampling (uv, light, shape), 3 for
// BSDF sampling (uv, w), 1 for Russian roulette when applicable.
#pragma once

#include "../../include/lj_gpu.h"
#include "lj_internal.h"
#include "lj_shade.cuh"

namespace lj {

// State of one path between two bounces.
struct PathState {
    int slot;        // OrderedPaths: the path's sample slot (pixel + sample * pixels)
    int job;         // server: job table slot
    int pixel;
    uint64_t rng;
    float4 beta;     // xyz: throughput after the pending BSDF sample (beta f / p), w: rr_prob
    float4 L;        // xyz: radiance, w: eta_scale
    float4 prev;     // xyz: vertex that sampled the pending ray, w: its BSDF pdf (solid angle)
    int nv;          // num_vertices of the next loop iteration (2 = primary ray pending)
};

// Outcome of one shade step besides the updated state.
struct ShadeOut {
    bool cont;               // a next ray was sampled
    float4 ray0, ray1;       // next ray: org | tnear, dir | tfar
    int shadow;              // the store's handle of this step's shadow ray, -1 if none
};

// Path state of the entries of one queue (queue order, SoA).
struct PathSoA {
    int *slot;       // sample slot: pixel + sample * pixels
    int *pixel;
    uint64_t *rng;
    float4 *beta;
    float4 *L;
    float4 *prev;
    int *nv;
};

struct Queues {
    PathSoA st[2];                // state of the entries of ray queue 0 / 1
    float4 *ray[2];
    float4 *hit;
    float4 *sray;
    int *starget;                 // the path's entry of the next queue, or ~slot when it ended
    float4 *scontrib;
    float4 *Lres;                 // radiance per sample slot of the ended paths
    int *counts;                  // [0], [1]: ray queues, [2]: shadow queue
    unsigned long long *stats;    // [0] closest rays, [1] shadow rays, [2] shade segments
    // select with a branch, not an index: indexing a kernel parameter's
    // array with a run-time value would copy the whole struct to local memory
    LJ_HD float4 *rays(int k) const { return k ? ray[1] : ray[0]; }
    LJ_HD const PathSoA &state(int k) const { return k ? st[1] : st[0]; }
};

// Per-job path options: max_depth / rr_depth as in RenderOptions
// (src/render.h), spread0 = the primary ray differential's spread.
struct ShadeCfg {
    int max_depth, rr_depth;
    float spread0;
};

LJ_D uint32_t lane_id() { return threadIdx.x & 31u; }

// Append one entry per calling thread; one atomicAdd per group of
// converged threads.
LJ_D int queue_slot(int *counter) {
    unsigned active = __activemask();
    int leader = __ffs(active) - 1;
    int base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(counter, __popc(active));
    base = __shfl_sync(active, base, leader);
    return base + __popc(active & ((1u << lane_id()) - 1u));
}

// Add v to a counter that many threads update: one atomic per group of
// converged threads (same-address atomics serialize in L2).
LJ_D void counter_add(unsigned long long *counter, unsigned v) {
    const unsigned active = __activemask();
    const unsigned sum = __reduce_add_sync(active, v);
    if ((int)lane_id() == __ffs(active) - 1 && sum) atomicAdd(counter, (unsigned long long)sum);
}

// The single-scene renderer's store: queue cur holds (ray, state) entries.
struct OrderedPaths {
    Queues q;
    int cur;
    LJ_D void load(int i, PathState &st, float4 &r0, float4 &r1, float4 &hit) const {
        const PathSoA &s = q.state(cur);
        st.slot = s.slot[i];
        st.job = 0;
        st.pixel = s.pixel[i];
        st.rng = s.rng[i];
        st.beta = s.beta[i];
        st.L = s.L[i];
        st.prev = s.prev[i];
        st.nv = s.nv[i];
        const float4 *rays = q.rays(cur);
        r0 = rays[2 * i];
        r1 = rays[2 * i + 1];
        hit = q.hit[i];
    }
    // NEE shadow ray: an unoccluded one adds contrib to the path's radiance,
    // wherever emit puts the path (the returned handle)
    LJ_D int shadow(const PathState &, float4 r0, float4 r1, float4 contrib) const {
        const int s = queue_slot(q.counts + 2);
        q.sray[2 * s] = r0;
        q.sray[2 * s + 1] = r1;
        q.scontrib[s] = contrib;
        return s;
    }
    LJ_D void emit(const PathState &st, const ShadeOut &o) const {
        int target;
        if (o.cont) {
            const int nxt = cur ^ 1;
            const int e = queue_slot(q.counts + nxt);
            const PathSoA &s = q.state(nxt);
            s.slot[e] = st.slot;
            s.pixel[e] = st.pixel;
            s.rng[e] = st.rng;
            s.beta[e] = st.beta;
            s.L[e] = st.L;
            s.prev[e] = st.prev;
            s.nv[e] = st.nv;
            float4 *rays = q.rays(nxt);
            rays[2 * e] = o.ray0;
            rays[2 * e + 1] = o.ray1;
            target = e;
        } else {
            q.Lres[st.slot] = st.L;
            target = ~st.slot;
        }
        if (o.shadow >= 0) q.starget[o.shadow] = target;
    }
};

// One queue entry: the hit of a path -> emission (with MIS for BSDF-sampled
// hits), Russian roulette, NEE (a shadow ray with its contribution), BSDF
// sample -> the next ray.
// kMats: the material types the scenes can hold (kAllMats: any).
template <uint32_t kMats, class Paths>
LJ_D void shade_segment(const DevScene &sc, const Paths &paths, int i, const ShadeCfg &cfg, int *status) {
    PathState st;
    float4 r0, r1, hit;
    paths.load(i, st, r0, r1, hit);
    ShadeOut out;
    out.cont = false;
    out.shadow = -1;
    const V3 ro{r0.x, r0.y, r0.z}, rd{r1.x, r1.y, r1.z};
    const int prim = __float_as_int(hit.y);
    int nv = st.nv;
    V3 L{st.L.x, st.L.y, st.L.z};
    float eta_scale = st.L.w;
    V3 beta{st.beta.x, st.beta.y, st.beta.z};
    const bool primary = nv == 2;
    Pcg rng;
    rng.state = st.rng;
    rng.inc = ((uint64_t)st.pixel << 1u) | 1u;
    bool alive = true;

    if (prim < 0) {
        // miss: environment map (path_tracing.h:17-28, :284-302)
        if (sc.env.light_id >= 0) {
            V3 Le = env_emission(sc, -rd);
            if (primary) {
                L += Le;
            } else {
                float p2 = st.prev.w;   // G = 1 for directions at infinity
                float p1 = __ldg(sc.light_pmf + sc.env.light_id) * env_pdf(sc, rd);
                float w2 = (p2 * p2) / (p1 * p1 + p2 * p2);
                L += beta * Le * w2;
            }
        }
        alive = false;
    } else {
        Vertex vx = make_vertex(sc, ro, rd, hit.x, prim, hit.z, hit.w, primary ? cfg.spread0 : 0.0f);
        if (primary) {
            if (vx.light >= 0) L += light_emission(sc, vx.light, -rd, PN{vx.p, vx.ng});
            beta = V3{1.0f, 1.0f, 1.0f};
            nv = 3;
        } else {
            V3 prev_p{st.prev.x, st.prev.y, st.prev.z};
            if (vx.light >= 0) {
                // BSDF-sampled hit on an area light (path_tracing.h:268-283)
                V3 Le = light_emission(sc, vx.light, -rd, PN{vx.p, vx.ng});
                V3 dv = vx.p - prev_p;
                float G = fabsf(dot(rd, vx.ng)) / dot(dv, dv);
                float p2 = st.prev.w * G;
                float p1 = __ldg(sc.light_pmf + vx.light) *
                           pdf_point_on_light(sc, vx.light, PN{vx.p, vx.ng}, prev_p);
                float w2 = (p2 * p2) / (p1 * p1 + p2 * p2);
                L += beta * Le * w2;
            }
            // Russian roulette of the iteration that sampled this ray
            // (path_tracing.h:311-318): that iteration's num_vertices is nv - 1
            float rr = 1.0f;
            if (nv - 2 >= cfg.rr_depth) {
                rr = st.beta.w;
                if (pcg_uniform(rng) > rr) alive = false;
            }
            beta = beta * (1.0f / rr);
        }
        if (alive && cfg.max_depth != -1 && nv > cfg.max_depth + 1) alive = false;
        if (alive && nv > LJ_MAX_BOUNCES + 2) {
            atomicOr(status, kStatusBounceCap);
            alive = false;
        }
        if (alive) {
            MatParams mat = resolve_material<kMats>(sc, vx.material, vx.u, vx.v, vx.uv_screen_size);
            BsdfVertex bv{vx.ng, vx.frame};
            V3 wv = -rd;
            // ---- next event estimation (path_tracing.h:98-207) ----
            float lu0 = pcg_uniform(rng), lu1 = pcg_uniform(rng);
            float lw = pcg_uniform(rng), sw = pcg_uniform(rng);
            // (a scene without lights has no NEE; the reference asserts there)
            int lid = sc.num_lights > 0 ? sample_light(sc, lw) : -1;
            PN pl{V3{0, 0, 0}, V3{0, 0, 0}};
            if (lid >= 0) pl = sample_point_on_light(sc, lid, vx.p, lu0, lu1, sw);
            V3 dl{0, 0, 1};
            float G = 0.0f, tmax = 0.0f, p1 = 0.0f;
            if (lid < 0) {
                // no light: G stays 0
            } else if (sc.lights[lid].kind == 0) {
                V3 dd = pl.p - vx.p;
                float dist2 = dot(dd, dd);
                float dist = sqrtf(dist2);
                dl = dd / dist;
                G = fmaxf(-dot(dl, pl.n), 0.0f) / dist2;
                tmax = (1.0f - sc.eps) * dist;
            } else {
                dl = -pl.n;
                G = 1.0f;
                tmax = __int_as_float(0x7f800000);
            }
            if (lid >= 0) p1 = __ldg(sc.light_pmf + lid) * pdf_point_on_light(sc, lid, pl, vx.p);
            if (G > 0.0f && p1 > 0.0f) {
                V3 f;
                float pdf_l;
                bsdf_eval_pdf<kMats>(mat, bv, wv, dl, f, pdf_l);
                V3 Le = light_emission(sc, lid, -dl, pl);
                float p2 = pdf_l * G;
                float w1 = (p1 * p1) / (p1 * p1 + p2 * p2);
                V3 c = beta * f * Le * (G * w1 / p1);
                if (c.x > 0.0f || c.y > 0.0f || c.z > 0.0f)
                    out.shadow = paths.shadow(st, make_float4(vx.p.x, vx.p.y, vx.p.z, sc.eps),
                                              make_float4(dl.x, dl.y, dl.z, tmax), make_float4(c.x, c.y, c.z, 0.0f));
            }
            // ---- BSDF sampling (path_tracing.h:210-256) ----
            float bu0 = pcg_uniform(rng), bu1 = pcg_uniform(rng), bwr = pcg_uniform(rng);
            BsdfSample bs = bsdf_sample<kMats>(mat, bv, wv, bu0, bu1, bwr);
            if (bs.valid) {
                V3 f;
                float pdf;
                bsdf_eval_pdf<kMats>(mat, bv, wv, bs.dir, f, pdf);
                if (pdf > 0.0f) {
                    if (bs.eta != 0.0f) eta_scale /= (bs.eta * bs.eta);
                    float rr_prob = fminf(max3(beta) / eta_scale, 0.95f);
                    V3 bn = beta * f / pdf;
                    st.beta = make_float4(bn.x, bn.y, bn.z, rr_prob);
                    st.prev = make_float4(vx.p.x, vx.p.y, vx.p.z, pdf);
                    st.nv = nv + 1;
                    out.cont = true;
                    out.ray0 = make_float4(vx.p.x, vx.p.y, vx.p.z, sc.eps);
                    out.ray1 = make_float4(bs.dir.x, bs.dir.y, bs.dir.z, __int_as_float(0x7f800000));
                }
            }
        }
    }
    st.L = make_float4(L.x, L.y, L.z, eta_scale);
    st.rng = rng.state;
    paths.emit(st, out);
}

}  // namespace lj
