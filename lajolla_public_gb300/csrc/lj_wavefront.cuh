// Wavefront state and the shade step of the unidirectional path tracer
// (src/path_tracing.h:7-325), shared by the single-scene renderer
// (lj_path.cu) and the multi-job server (lj_server.cu).
//
// Path state is SoA indexed by path slot; queues hold (ray, path slot)
// pairs.  The random-number order per path is the reference's: 2 for the
// screen position, then per bounce 4 for light sampling (uv, light, shape),
// 3 for BSDF sampling (uv, w), 1 for Russian roulette when applicable.
#pragma once

#include "lj_shade.cuh"

namespace lj {

struct PathSoA {
    int *job;        // server: job table slot of the path (unused by the plain renderer)
    int *pixel;
    uint64_t *rng;
    float4 *beta;    // xyz: throughput after the pending BSDF sample (beta f / p), w: rr_prob
    float4 *L;       // xyz: radiance, w: eta_scale
    float4 *prev;    // xyz: vertex that sampled the pending ray, w: its BSDF pdf (solid angle)
    int *nv;         // num_vertices of the next loop iteration (2 = primary ray pending)
};

struct Queues {
    float4 *ray[2];
    int *path[2];
    float4 *hit;
    float4 *sray;
    int *spath;
    float4 *scontrib;
    int *retire;                  // server: paths that ended this pass (nullptr: not collected)
    int *counts;                  // [0], [1]: ray queues, [2]: shadow queue, [3]: retire queue
    unsigned long long *stats;    // [0] closest rays, [1] shadow rays, [2] shade segments
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

LJ_D Pcg load_rng(const PathSoA &ps, int p) {
    Pcg r;
    r.state = ps.rng[p];
    r.inc = ((uint64_t)ps.pixel[p] << 1u) | 1u;
    return r;
}



// One queue entry: the hit of path q.path[cur][i] -> emission (with MIS for
// BSDF-sampled hits), Russian roulette, NEE (shadow ray queued with its
// contribution), BSDF sample -> next ray in queue cur ^ 1.
LJ_D void shade_segment(const DevScene &sc, const PathSoA &ps, const Queues &q, int cur, int i,
                        const ShadeCfg &cfg, int *status) {
    const int nxt = cur ^ 1;
    const int p = q.path[cur][i];
    float4 r0 = q.ray[cur][2 * i], r1 = q.ray[cur][2 * i + 1];
    V3 ro{r0.x, r0.y, r0.z}, rd{r1.x, r1.y, r1.z};
    float4 hit = q.hit[i];
    int prim = __float_as_int(hit.y);
    int nv = ps.nv[p];
    float4 Lw = ps.L[p];
    V3 L{Lw.x, Lw.y, Lw.z};
    float eta_scale = Lw.w;
    float4 bw = ps.beta[p];
    V3 beta{bw.x, bw.y, bw.z};
    const bool primary = nv == 2;
    Pcg rng = load_rng(ps, p);
    bool alive = true;
    bool continued = false;

    if (prim < 0) {
        // miss: environment map (path_tracing.h:17-28, :284-302)
        if (sc.env.light_id >= 0) {
            V3 Le = env_emission(sc, -rd);
            if (primary) {
                L += Le;
            } else {
                float4 pv = ps.prev[p];
                float p2 = pv.w;   // G = 1 for directions at infinity
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
            float4 pv = ps.prev[p];
            V3 prev_p{pv.x, pv.y, pv.z};
            if (vx.light >= 0) {
                // BSDF-sampled hit on an area light (path_tracing.h:268-283)
                V3 Le = light_emission(sc, vx.light, -rd, PN{vx.p, vx.ng});
                V3 dv = vx.p - prev_p;
                float G = fabsf(dot(rd, vx.ng)) / dot(dv, dv);
                float p2 = pv.w * G;
                float p1 = __ldg(sc.light_pmf + vx.light) *
                           pdf_point_on_light(sc, vx.light, PN{vx.p, vx.ng}, prev_p);
                float w2 = (p2 * p2) / (p1 * p1 + p2 * p2);
                L += beta * Le * w2;
            }
            // Russian roulette of the iteration that sampled this ray
            // (path_tracing.h:311-318): that iteration's num_vertices is nv - 1
            float rr = 1.0f;
            if (nv - 2 >= cfg.rr_depth) {
                rr = bw.w;
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
            MatParams mat = resolve_material(sc, vx.material, vx.u, vx.v, vx.uv_screen_size);
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
                V3 f = bsdf_eval(mat, bv, wv, dl);
                V3 Le = light_emission(sc, lid, -dl, pl);
                float p2 = bsdf_pdf(mat, bv, wv, dl) * G;
                float w1 = (p1 * p1) / (p1 * p1 + p2 * p2);
                V3 c = beta * f * Le * (G * w1 / p1);
                if (c.x > 0.0f || c.y > 0.0f || c.z > 0.0f) {
                    int s = queue_slot(q.counts + 2);
                    q.sray[2 * s] = make_float4(vx.p.x, vx.p.y, vx.p.z, sc.eps);
                    q.sray[2 * s + 1] = make_float4(dl.x, dl.y, dl.z, tmax);
                    q.spath[s] = p;
                    q.scontrib[s] = make_float4(c.x, c.y, c.z, 0.0f);
                }
            }
            // ---- BSDF sampling (path_tracing.h:210-256) ----
            float bu0 = pcg_uniform(rng), bu1 = pcg_uniform(rng), bwr = pcg_uniform(rng);
            BsdfSample bs = bsdf_sample(mat, bv, wv, bu0, bu1, bwr);
            if (!bs.valid) {
                alive = false;
            } else {
                V3 f = bsdf_eval(mat, bv, wv, bs.dir);
                float pdf = bsdf_pdf(mat, bv, wv, bs.dir);
                if (!(pdf > 0.0f)) {
                    alive = false;
                } else {
                    if (bs.eta != 0.0f) eta_scale /= (bs.eta * bs.eta);
                    float rr_prob = fminf(max3(beta) / eta_scale, 0.95f);
                    V3 bn = beta * f / pdf;
                    ps.beta[p] = make_float4(bn.x, bn.y, bn.z, rr_prob);
                    ps.prev[p] = make_float4(vx.p.x, vx.p.y, vx.p.z, pdf);
                    ps.nv[p] = nv + 1;
                    int s = queue_slot(q.counts + nxt);
                    q.ray[nxt][2 * s] = make_float4(vx.p.x, vx.p.y, vx.p.z, sc.eps);
                    q.ray[nxt][2 * s + 1] = make_float4(bs.dir.x, bs.dir.y, bs.dir.z, __int_as_float(0x7f800000));
                    q.path[nxt][s] = p;
                    continued = true;
                }
            }
        }
    }
    ps.L[p] = make_float4(L.x, L.y, L.z, eta_scale);
    ps.rng[p] = rng.state;
    // a finished path: the server's retire step accumulates it once its
    // pending shadow ray (if any) has been traced
    if (!continued && q.retire) q.retire[queue_slot(q.counts + 3)] = p;
}

}  // namespace lj
