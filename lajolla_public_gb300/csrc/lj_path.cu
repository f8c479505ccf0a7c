// Wavefront unidirectional path tracer: the GPU form of path_render /
// path_tracing (src/render.cpp:71-101, src/path_tracing.h:7-325).
//
// One path per (pixel, sample); its PCG stream is keyed on (job seed, pixel,
// sample), so results do not depend on batching.  Per bounce:
//
//   trace_closest  queue of rays          -> hits (compressed 8-wide BVH)
//   shade          hit -> emission (+MIS for BSDF-sampled hits), Russian
//                  roulette, NEE (light sample + shadow ray, MIS weight),
//                  BSDF sample -> next ray; queues are appended with warp-
//                  aggregated atomics (one atomicAdd per warp)
//   trace_shadow   shadow rays -> add the NEE contribution if unoccluded
//
// The order of random numbers per path is the reference's: 2 for the screen
// position (x then y), then per bounce 4 for light sampling (uv, light, shape),
// 3 for BSDF sampling (uv, w), 1 for Russian roulette when applicable.
// A sample's radiance is accumulated in its own slot and reduced per pixel in
// sample order, so the image is deterministic.
#include <algorithm>
#include <cstring>
#include <vector>

#include "lj_host.h"
#include "lj_shade.cuh"
#include "lj_trace.cuh"

namespace lj {

namespace {

struct PathSoA {
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
    int *counts;                  // [0], [1]: ray queues, [2]: shadow queue, [3]: pad
    unsigned long long *stats;    // [0] closest rays, [1] shadow rays, [2] shade segments
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

// sample_primary, src/camera.cpp:23-47
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

__global__ void k_camera(DevScene sc, PathSoA ps, Queues q, int P, int num_pixels, int sample_base,
                         uint64_t seed) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    int pixel = p % num_pixels;
    int sample = sample_base + p / num_pixels;
    Pcg rng = pcg_keyed(seed, (uint64_t)pixel, (uint64_t)sample);
    int x = pixel % sc.cam.w, y = pixel / sc.cam.w;
    float r1 = pcg_uniform(rng), r2 = pcg_uniform(rng);
    V3 o, d;
    camera_ray(sc.cam, (x + r1) / sc.cam.w, (y + r2) / sc.cam.h, o, d);
    q.ray[0][2 * p] = make_float4(o.x, o.y, o.z, 0.0f);
    q.ray[0][2 * p + 1] = make_float4(d.x, d.y, d.z, __int_as_float(0x7f800000));
    q.path[0][p] = p;
    ps.pixel[p] = pixel;
    ps.rng[p] = rng.state;
    ps.beta[p] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    ps.L[p] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    ps.prev[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    ps.nv[p] = 2;
}

__global__ void __launch_bounds__(128) k_trace_queue(DevBvh bvh, const float4 *rays, float4 *hits,
                                                     const int *count, unsigned long long *stat,
                                                     int *status) {
    int n = *count;
    if (blockIdx.x == 0 && threadIdx.x == 0 && stat) atomicAdd(stat, (unsigned long long)n);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 r0 = rays[2 * i], r1 = rays[2 * i + 1];
        TraceHit h{0.0f, -1, 0.0f, 0.0f};
        int ovf = 0;
        bool f = trace_bvh<false>(bvh, V3{r0.x, r0.y, r0.z}, V3{r1.x, r1.y, r1.z}, r0.w, r1.w, h, &ovf);
        hits[i] = f ? make_float4(h.t, __int_as_float(h.prim), h.u, h.v)
                    : make_float4(0.0f, __int_as_float(-1), 0.0f, 0.0f);
        if (ovf) atomicOr(status, kStatusStackOverflow);
    }
}

__global__ void __launch_bounds__(128) k_trace_shadow(DevBvh bvh, const float4 *rays, const int *paths,
                                                      const float4 *contrib, const int *count, float4 *L,
                                                      unsigned long long *stat, int *status) {
    int n = *count;
    if (blockIdx.x == 0 && threadIdx.x == 0 && stat) atomicAdd(stat, (unsigned long long)n);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 r0 = rays[2 * i], r1 = rays[2 * i + 1];
        TraceHit h{0.0f, -1, 0.0f, 0.0f};
        int ovf = 0;
        bool occ = trace_bvh<true>(bvh, V3{r0.x, r0.y, r0.z}, V3{r1.x, r1.y, r1.z}, r0.w, r1.w, h, &ovf);
        if (ovf) atomicOr(status, kStatusStackOverflow);
        if (!occ) {
            int p = paths[i];
            float4 c = contrib[i];
            float4 l = L[p];
            L[p] = make_float4(l.x + c.x, l.y + c.y, l.z + c.z, l.w);
        }
    }
}

__global__ void __launch_bounds__(128) k_shade(DevScene sc, PathSoA ps, Queues q, int cur,
                                               float spread0, int *status) {
    const int n = q.counts[cur];
    const int nxt = cur ^ 1;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(q.stats + 2, (unsigned long long)n);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
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
            Vertex vx = make_vertex(sc, ro, rd, hit.x, prim, hit.z, hit.w, primary ? spread0 : 0.0f);
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
                if (nv - 2 >= sc.rr_depth) {
                    rr = bw.w;
                    if (pcg_uniform(rng) > rr) alive = false;
                }
                beta = beta * (1.0f / rr);
            }
            if (alive && sc.max_depth != -1 && nv > sc.max_depth + 1) alive = false;
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
                    }
                }
            }
        }
        ps.L[p] = make_float4(L.x, L.y, L.z, eta_scale);
        ps.rng[p] = rng.state;
    }
}

// Per pixel: sum the batch's samples in sample order (deterministic).
__global__ void k_resolve(const float4 *L, int num_pixels, int nsamp, float *accum) {
    int px = blockIdx.x * blockDim.x + threadIdx.x;
    if (px >= num_pixels) return;
    float sx = 0, sy = 0, sz = 0;
    for (int s = 0; s < nsamp; s++) {
        float4 l = L[(size_t)s * num_pixels + px];
        sx += l.x;
        sy += l.y;
        sz += l.z;
    }
    accum[3 * px] += sx;
    accum[3 * px + 1] += sy;
    accum[3 * px + 2] += sz;
}

__global__ void k_scale(float *img, int64_t n, float s) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) img[i] *= s;
}

__global__ void k_set_counts(int *counts, int c0) {
    counts[0] = c0;
    counts[1] = 0;
    counts[2] = 0;
}
__global__ void k_zero2(int *counts, int a, int b) {
    counts[a] = 0;
    counts[b] = 0;
}

template <typename T>
T *carve(char *&p, size_t n) {
    T *r = (T *)p;
    p += ((n * sizeof(T) + 255) / 256) * 256;
    return r;
}

size_t path_bytes(size_t P) {
    size_t per = 0;
    auto add = [&](size_t b) { per += ((b + 255) / 256) * 256; };
    add(P * sizeof(int)); add(P * 8); add(P * 16); add(P * 16); add(P * 16); add(P * sizeof(int));
    add(P * 32); add(P * 32); add(P * 4); add(P * 4); add(P * 16);
    add(P * 32); add(P * 4); add(P * 16);
    add(64); add(64);
    return per;
}

int grid_persistent(const void *kernel, int threads) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
    return std::max(1, sms * std::max(1, per_sm));
}

}  // namespace

int render_path(lj_scene *scene, const lj_render_params *params, float *d_out, cudaStream_t s,
                lj_stats *stats, bool sync_stats) {
    lj_ctx *ctx = scene->ctx;
    const DevScene &sc = scene->dev;
    std::string e;
    std::string *err = &e;
    const int W = scene->width, H = scene->height;
    const int num_pixels = W * H;
    const int spp = params->spp > 0 ? params->spp : scene->options.samples_per_pixel;
    if (spp <= 0) return set_error(ctx, LJ_ERR_INVALID_ARG, "render: samples per pixel must be positive");
    int64_t cap = params->max_paths_in_flight > 0 ? params->max_paths_in_flight : (int64_t)1 << 22;
    int nsamp = (int)std::max<int64_t>(1, std::min<int64_t>(spp, cap / std::max(1, num_pixels)));
    size_t P = (size_t)num_pixels * nsamp;
    size_t need = path_bytes(P);
    if (scene->path.bytes < need) {
        if (scene->path.block) cudaFree(scene->path.block);
        scene->path.block = nullptr;
        scene->path.bytes = 0;
        if (cudaMalloc(&scene->path.block, need) != cudaSuccess) {
            cudaGetLastError();
            return set_error(ctx, LJ_ERR_OUT_OF_MEMORY, "render: cannot allocate wavefront buffers");
        }
        scene->path.bytes = need;
    }
    char *cur = (char *)scene->path.block;
    PathSoA ps;
    ps.pixel = carve<int>(cur, P);
    ps.rng = carve<uint64_t>(cur, P);
    ps.beta = carve<float4>(cur, P);
    ps.L = carve<float4>(cur, P);
    ps.prev = carve<float4>(cur, P);
    ps.nv = carve<int>(cur, P);
    Queues q;
    q.ray[0] = carve<float4>(cur, 2 * P);
    q.ray[1] = carve<float4>(cur, 2 * P);
    q.path[0] = carve<int>(cur, P);
    q.path[1] = carve<int>(cur, P);
    q.hit = carve<float4>(cur, P);
    q.sray = carve<float4>(cur, 2 * P);
    q.spath = carve<int>(cur, P);
    q.scontrib = carve<float4>(cur, P);
    q.counts = carve<int>(cur, 16);
    q.stats = carve<unsigned long long>(cur, 8);

    LJ_CUDA_TRY(cudaMemsetAsync(q.stats, 0, 8 * sizeof(unsigned long long), s));
    LJ_CUDA_TRY(cudaMemsetAsync(d_out, 0, sizeof(float) * 3 * (size_t)num_pixels, s));
    const int g_trace = grid_persistent((const void *)k_trace_queue, 128);
    const int g_shadow = grid_persistent((const void *)k_trace_shadow, 128);
    const int g_shade = grid_persistent((const void *)k_shade, 128);
    const int passes = scene->options.max_depth == -1 ? LJ_MAX_BOUNCES + 1
                                                      : std::max(1, scene->options.max_depth);
    const float spread0 = 0.25f / (float)std::max(W, H);
    cudaEvent_t e0, e1;
    bool timed = stats != nullptr;
    if (timed) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, s);
    }
    int64_t launches = 0;
    // LJ_RENDER_PROFILE: an event pair around every kernel, grouped by class
    const bool profile = timed && (params->flags & LJ_RENDER_PROFILE);
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
    auto mark_begin = [&](int cls) {
        if (!profile) return;
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, s);
        marks.push_back({cls, {a, b}});
    };
    auto mark_end = [&]() {
        if (profile) cudaEventRecord(marks.back().second.second, s);
    };
    int64_t class_launches[LJ_KERNEL_CLASSES] = {0, 0, 0, 0, 0};
    for (int sb = 0; sb < spp; sb += nsamp) {
        int ns = std::min(nsamp, spp - sb);
        int Pb = num_pixels * ns;
        k_set_counts<<<1, 1, 0, s>>>(q.counts, Pb);
        mark_begin(LJ_KERNEL_CAMERA);
        k_camera<<<(Pb + 255) / 256, 256, 0, s>>>(sc, ps, q, Pb, num_pixels, params->sample_offset + sb,
                                                  params->seed);
        mark_end();
        launches += 2;
        class_launches[LJ_KERNEL_OTHER]++;
        class_launches[LJ_KERNEL_CAMERA]++;
        int curq = 0;
        for (int pass = 0; pass < passes; pass++) {
            k_zero2<<<1, 1, 0, s>>>(q.counts, curq ^ 1, 2);
            mark_begin(LJ_KERNEL_TRACE);
            k_trace_queue<<<g_trace, 128, 0, s>>>(sc.bvh, q.ray[curq], q.hit, q.counts + curq, q.stats + 0,
                                                  ctx->d_status);
            mark_end();
            mark_begin(LJ_KERNEL_SHADE);
            k_shade<<<g_shade, 128, 0, s>>>(sc, ps, q, curq, spread0, ctx->d_status);
            mark_end();
            mark_begin(LJ_KERNEL_SHADOW);
            k_trace_shadow<<<g_shadow, 128, 0, s>>>(sc.bvh, q.sray, q.spath, q.scontrib, q.counts + 2, ps.L,
                                                    q.stats + 1, ctx->d_status);
            mark_end();
            launches += 4;
            class_launches[LJ_KERNEL_OTHER]++;
            class_launches[LJ_KERNEL_TRACE]++;
            class_launches[LJ_KERNEL_SHADE]++;
            class_launches[LJ_KERNEL_SHADOW]++;
            curq ^= 1;
            if (scene->options.max_depth == -1 && (pass & 7) == 7) {
                int c = 0;
                LJ_CUDA_TRY(cudaMemcpyAsync(&c, q.counts + curq, sizeof(int), cudaMemcpyDeviceToHost, s));
                LJ_CUDA_TRY(cudaStreamSynchronize(s));
                if (c == 0) break;
            }
        }
        k_resolve<<<(num_pixels + 255) / 256, 256, 0, s>>>(ps.L, num_pixels, ns, d_out);
        launches++;
        class_launches[LJ_KERNEL_OTHER]++;
    }
    int64_t nfl = 3 * (int64_t)num_pixels;
    k_scale<<<(int)((nfl + 255) / 256), 256, 0, s>>>(d_out, nfl, 1.0f / spp);
    launches++;
    class_launches[LJ_KERNEL_OTHER]++;
    LJ_CUDA_TRY(cudaGetLastError());
    if (timed) {
        cudaEventRecord(e1, s);
        unsigned long long st[8];
        LJ_CUDA_TRY(cudaMemcpyAsync(st, q.stats, sizeof(st), cudaMemcpyDeviceToHost, s));
        LJ_CUDA_TRY(cudaStreamSynchronize(s));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        stats->device_ms = ms;
        stats->samples = (int64_t)num_pixels * spp;
        stats->rays_closest = (int64_t)st[0];
        stats->rays_shadow = (int64_t)st[1];
        stats->path_segments = (int64_t)st[2];
        stats->kernel_launches = launches;
        for (int c = 0; c < LJ_KERNEL_CLASSES; c++) {
            stats->class_launches[c] = class_launches[c];
            stats->class_ms[c] = 0.0;
        }
        for (auto &m : marks) {
            float kms = 0;
            cudaEventElapsedTime(&kms, m.second.first, m.second.second);
            stats->class_ms[m.first] += kms;
            cudaEventDestroy(m.second.first);
            cudaEventDestroy(m.second.second);
        }
        if (profile) {
            double other = ms;
            for (int c = 0; c < LJ_KERNEL_OTHER; c++) other -= stats->class_ms[c];
            stats->class_ms[LJ_KERNEL_OTHER] = other > 0 ? other : 0;
        }
        int status = 0;
        LJ_CUDA_TRY(cudaMemcpy(&status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost));
        if (status) {
            cudaMemset(ctx->d_status, 0, sizeof(int));
            return set_error(ctx, LJ_ERR_DEVICE_LIMIT, "render: device loop bound reached (status " +
                                                           std::to_string(status) + ")");
        }
    }
    (void)sync_stats;
    return LJ_OK;
}

}  // namespace lj

using namespace lj;

extern "C" {

int lj_gpu_render_device(lj_scene *scene, const lj_render_params *params, float *d_out_rgb, void *stream,
                         lj_stats *stats) {
    if (!scene || !params || !d_out_rgb) return LJ_ERR_INVALID_ARG;
    cudaSetDevice(scene->ctx->device);
    if (scene->options.integrator != LJ_INTEGRATOR_PATH)
        return set_error(scene->ctx, LJ_ERR_UNSUPPORTED, "render: integrator not available in this build");
    cudaStream_t s = (cudaStream_t)stream;   // NULL: the legacy default stream
    if (stats) memset(stats, 0, sizeof(*stats));
    return render_path(scene, params, d_out_rgb, s, stats, stats != nullptr);
}

int lj_gpu_render(lj_scene *scene, const lj_render_params *params, float *out_rgb, lj_stats *stats) {
    if (!scene || !params || !out_rgb) return LJ_ERR_INVALID_ARG;
    cudaSetDevice(scene->ctx->device);
    size_t bytes = sizeof(float) * 3 * (size_t)scene->width * scene->height;
    float *d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) {
        cudaGetLastError();
        return set_error(scene->ctx, LJ_ERR_OUT_OF_MEMORY, "render: cannot allocate the image");
    }
    lj_stats local;
    int rc = lj_gpu_render_device(scene, params, d, scene->ctx->stream, stats ? stats : &local);
    if (rc == LJ_OK) {
        if (cudaMemcpyAsync(out_rgb, d, bytes, cudaMemcpyDeviceToHost, scene->ctx->stream) != cudaSuccess ||
            cudaStreamSynchronize(scene->ctx->stream) != cudaSuccess)
            rc = set_error(scene->ctx, LJ_ERR_CUDA, "render: copy-back failed");
    }
    cudaFree(d);
    return rc;
}

}  // extern "C"
