// Wavefront volumetric path tracer (v6): the GPU form of vol_path_tracing
// (src/vol_path_tracing.h:59-64, a stub in the reference; the algorithm is the
// one handouts/homework2.tex:303-816 specifies, restated in
// oracle/lj_oracle.cpp with the same random-number order).
//
// Per pass:
//   vol_trace   the path queue's rays -> closest hits (persistent traversal)
//   vol_a       free-flight delta tracking over [0, t_hit) with the
//               chromatic majorant (one channel sampled per segment);
//               emission with MIS; index-matching surfaces passed; at a
//               real scattering point or a surface with a material, the
//               light sample of NEE and a request in the NEE queue
//   vol_b       per NEE request: the shadow ray's walk through
//               index-matching surfaces (closest hits), then ratio
//               tracking through media unless an opaque surface blocks it
//   vol_c       per NEE request: the MIS-weighted contribution, phase /
//               BSDF sampling, Russian roulette, next ray appended to the
//               other queue.
// Null-collision loops are capped by max_null_collisions; shadow-segment and
// bounce loops by the depth limit and LJ_MAX_BOUNCES.
#include <algorithm>
#include <cstring>
#include <vector>

#include "lj_host.h"
#include "lj_trace_queue.cuh"
#include "lj_volwave.cuh"

namespace lj {

namespace {

struct VolSoA {
    int *pixel;
    uint64_t *rng;
    float4 *beta;   // xyz throughput, w eta_scale
    float4 *L;      // xyz radiance, w dir_pdf (solid angle) of the last scattering
    float4 *neep;   // xyz position of the last vertex that could issue NEE
    float4 *mdir;   // xyz product of free-flight pdfs since that vertex
    float4 *mnee;   // xyz product of ratio-tracking pdfs since that vertex
    int4 *st;       // x medium, y bounces, z never_scatter, w first ray
};

struct VolQueues {
    float4 *ray[2];
    int *path[2];
    float4 *hit;
    int *counts;                  // [0], [1] ray queues, [2], [3] NEE requests (front, back), [8] ray fetch
                                  // counter
    unsigned long long *stats;    // [0] closest rays, [1] shadow segments, [2] segments, [3] null, [4] real
    NeeQueue nee;
};


__global__ void k_vol_camera(DevScene sc, VolSoA ps, VolQueues q, int P, int num_pixels, int sample_base,
                             uint64_t seed);

}  // namespace


namespace {

__global__ void k_vol_camera(DevScene sc, VolSoA ps, VolQueues q, int P, int num_pixels, int sample_base,
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
    ps.L[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    ps.neep[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    ps.mdir[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    ps.mnee[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    ps.st[p] = make_int4(sc.camera_medium, 0, 1, 1);
}

// Closest hits of the queue's rays by persistent warps (*fetch = 0 at launch).
__global__ void __launch_bounds__(128, 8) k_vol_trace(DevBvh bvh, const float4 *rays, float4 *hits,
                                                      const int *count, int *fetch, unsigned long long *stat,
                                                      int *status) {
    const int n = *count;
    if (blockIdx.x == 0 && threadIdx.x == 0 && stat) atomicAdd(stat, (unsigned long long)n);
    ClosestQueueIO io{bvh, rays, hits};
    trace_queue<false, 128>(io, n, fetch, status);
}

// The single-scene renderer's store: state in fixed slots, queues carry
// slot ids.
struct VolSlotStore {
    VolSoA ps;
    VolQueues q;
    int cur;
    LJ_D void load(int i, VolState &vs, float4 &r0, float4 &r1, float4 &hit) const {
        const int p = (cur ? q.path[1] : q.path[0])[i];
        const float4 *rays = cur ? q.ray[1] : q.ray[0];
        r0 = rays[2 * i];
        r1 = rays[2 * i + 1];
        hit = q.hit[i];
        vs.slot = p;
        vs.job = 0;
        vs.pixel = ps.pixel[p];
        vs.rng = ps.rng[p];
        vs.beta = ps.beta[p];
        vs.L = ps.L[p];
        vs.neep = ps.neep[p];
        vs.mdir = ps.mdir[p];
        vs.mnee = ps.mnee[p];
        vs.st = ps.st[p];
    }
    // state of a path that waits for its NEE request (the c step resets the
    // NEE vertex and the pdf products, and takes the PCG state from the
    // request, so those stay behind)
    LJ_D void save(int, const VolState &vs) const {
        const int p = vs.slot;
        ps.beta[p] = vs.beta;
        ps.L[p] = vs.L;
        ps.st[p] = vs.st;
    }
    LJ_D void load_c(int i, VolState &vs, float4 &r0, float4 &r1, float4 &hit) const {
        const int p = (cur ? q.path[1] : q.path[0])[i];
        const float4 *rays = cur ? q.ray[1] : q.ray[0];
        r0 = rays[2 * i];
        r1 = rays[2 * i + 1];
        hit = q.hit[i];
        vs.slot = p;
        vs.job = 0;
        vs.pixel = ps.pixel[p];
        vs.beta = ps.beta[p];
        vs.L = ps.L[p];
        vs.st = ps.st[p];
    }
    LJ_D void emit(const VolState &vs, bool alive, float4 ray0, float4 ray1) const {
        const int p = vs.slot, nxt = cur ^ 1;
        if (alive) {
            const int s = queue_slot(q.counts + nxt);
            float4 *nrays = nxt ? q.ray[1] : q.ray[0];
            nrays[2 * s] = ray0;
            nrays[2 * s + 1] = ray1;
            (nxt ? q.path[1] : q.path[0])[s] = p;
        }
        ps.beta[p] = vs.beta;
        ps.L[p] = vs.L;
        ps.neep[p] = vs.neep;
        ps.mdir[p] = vs.mdir;
        ps.mnee[p] = vs.mnee;
        ps.st[p] = vs.st;
        ps.rng[p] = vs.rng;
    }
};

__global__ void __launch_bounds__(128, 4) k_vol_a(DevScene sc, VolSoA ps, VolQueues q, int cur, float spread0,
                                                  int *status) {
    const int n = q.counts[cur];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(q.stats + 2, (unsigned long long)n);
    const ShadeCfg cfg{sc.max_depth, sc.rr_depth, spread0};
    const VolSlotStore store{ps, q, cur};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        vol_segment_a(sc, store, i, cfg, q.nee, status, q.stats);
}
// The requests from scattering points finish their c step here too
// (NeeToPhase); those from surfaces go on to k_vol_c<..., true>.
__global__ void __launch_bounds__(128, 4) k_vol_b(DevScene sc, VolSoA ps, VolQueues q, int cur, float spread0,
                                                  int *status) {
    const int nf = q.counts[2], n = nf + q.counts[3];
    const ShadeCfg cfg{sc.max_depth, sc.rr_depth, spread0};
    const VolSlotStore store{ps, q, cur};
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const int k = q.nee.req(r, nf);
        if (r < nf) vol_nee_b(sc, q.nee, k, sc.max_depth, status, q.stats + 1, NeeToPhase<VolSlotStore>{sc, store, q.nee, cfg});
        else vol_nee_b(sc, q.nee, k, sc.max_depth, status, q.stats + 1, NeeToQueue{q.nee});
    }
}
// kSurface = false: requests from scattering points (front); true: from
// surfaces (back).  64 registers, full occupancy (as the server's c step).
template <uint32_t kMats, bool kSurface>
__global__ void __launch_bounds__(128, 8) k_vol_c(DevScene sc, VolSoA ps, VolQueues q, int cur, float spread0) {
    const int n = q.counts[kSurface ? 3 : 2];
    const ShadeCfg cfg{sc.max_depth, sc.rr_depth, spread0};
    const VolSlotStore store{ps, q, cur};
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
        vol_segment_c<kMats, kSurface>(sc, store, kSurface ? q.nee.cap - 1 - r : r, cfg, q.nee);
}
using VolCKernel = void (*)(DevScene, VolSoA, VolQueues, int, float);

// Per pixel: sum the batch's samples in sample order, skipping samples with
// no finite channel (src/render.cpp:138-143, an OR over channels).
__global__ void k_vol_resolve(const float4 *L, int num_pixels, int nsamp, float *accum) {
    int px = blockIdx.x * blockDim.x + threadIdx.x;
    if (px >= num_pixels) return;
    float sx = 0, sy = 0, sz = 0;
    for (int s = 0; s < nsamp; s++) {
        float4 l = L[(size_t)s * num_pixels + px];
        if (isfinite(l.x) || isfinite(l.y) || isfinite(l.z)) {
            sx += l.x;
            sy += l.y;
            sz += l.z;
        }
    }
    accum[3 * px] += sx;
    accum[3 * px + 1] += sy;
    accum[3 * px + 2] += sz;
}
__global__ void k_vol_scale(float *img, int64_t n, float s) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) img[i] *= s;
}
__global__ void k_vol_set_counts(int *counts, int c0) {
    counts[0] = c0;
    counts[1] = 0;
    counts[2] = 0;
    counts[3] = 0;
    counts[8] = 0;
}
__global__ void k_vol_zero(int *counts, int a) {
    counts[a] = 0;
    counts[2] = 0;
    counts[3] = 0;
    counts[8] = 0;
}

template <typename T>
T *carve(char *&p, size_t n) {
    T *r = (T *)p;
    p += ((n * sizeof(T) + 255) / 256) * 256;
    return r;
}
size_t vol_bytes(size_t P) {
    size_t per = 0;
    auto add = [&](size_t b) { per += ((b + 255) / 256) * 256; };
    add(P * 4); add(P * 8); add(P * 16); add(P * 16); add(P * 16); add(P * 16); add(P * 16); add(P * 16);
    add(P * 32); add(P * 32); add(P * 4); add(P * 4); add(P * 16); add(64); add(64);
    // NEE queue: entry; org, dir, lp, ln, ss, T, pn, pd, med (16 B each); rng
    add(P * 4); for (int k = 0; k < 9; k++) add(P * 16); add(P * 8);
    return per;
}
int grid_for_kernel(const void *kernel, int threads) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
    return std::max(1, sms * std::max(1, per_sm));
}

}  // namespace

int render_volpath(lj_scene *scene, const lj_render_params *params, float *d_out, cudaStream_t s,
                   lj_stats *stats, const lj_job_desc *job) {
    lj_ctx *ctx = scene->ctx;
    DevScene sc = scene->dev;   // job overrides: resolution (camera) and depth options
    int W = scene->width, H = scene->height;
    if (job && job->width > 0 && job->height > 0) {
        W = job->width;
        H = job->height;
        make_cam_rec(scene->camera, W, H, sc.cam);
    }
    if (job && job->override_depth) {
        if (job->max_depth < -1) return set_error(ctx, LJ_ERR_INVALID_ARG, "render: max_depth must be >= -1");
        sc.max_depth = job->max_depth;
        sc.rr_depth = job->rr_depth;
    }
    std::string e;
    std::string *err = &e;
    const int num_pixels = W * H;
    const int spp = params->spp > 0 ? params->spp : scene->options.samples_per_pixel;
    if (spp <= 0) return set_error(ctx, LJ_ERR_INVALID_ARG, "render: samples per pixel must be positive");
    int64_t cap = params->max_paths_in_flight > 0 ? params->max_paths_in_flight : kDefaultPathsInFlight;
    int nsamp = (int)std::max<int64_t>(1, std::min<int64_t>(spp, cap / std::max(1, num_pixels)));
    size_t P = (size_t)num_pixels * nsamp;
    size_t need = vol_bytes(P);
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
    VolSoA ps;
    ps.pixel = carve<int>(cur, P);
    ps.rng = carve<uint64_t>(cur, P);
    ps.beta = carve<float4>(cur, P);
    ps.L = carve<float4>(cur, P);
    ps.neep = carve<float4>(cur, P);
    ps.mdir = carve<float4>(cur, P);
    ps.mnee = carve<float4>(cur, P);
    ps.st = carve<int4>(cur, P);
    VolQueues q;
    q.ray[0] = carve<float4>(cur, 2 * P);
    q.ray[1] = carve<float4>(cur, 2 * P);
    q.path[0] = carve<int>(cur, P);
    q.path[1] = carve<int>(cur, P);
    q.hit = carve<float4>(cur, P);
    q.counts = carve<int>(cur, 16);
    q.stats = carve<unsigned long long>(cur, 8);
    q.nee.cap = (int)P;
    q.nee.count = q.counts + 2;
    q.nee.entry = carve<int>(cur, P);
    q.nee.org = carve<float4>(cur, P);
    q.nee.dir = carve<float4>(cur, P);
    q.nee.lp = carve<float4>(cur, P);
    q.nee.ln = carve<float4>(cur, P);
    q.nee.ss = carve<float4>(cur, P);
    q.nee.T = carve<float4>(cur, P);
    q.nee.pn = carve<float4>(cur, P);
    q.nee.pd = carve<float4>(cur, P);
    q.nee.med = carve<int4>(cur, P);
    q.nee.rng = carve<uint64_t>(cur, P);
    LJ_CUDA_TRY(cudaMemsetAsync(q.stats, 0, 8 * sizeof(unsigned long long), s));
    LJ_CUDA_TRY(cudaMemsetAsync(d_out, 0, sizeof(float) * 3 * (size_t)num_pixels, s));
    const int g_trace = grid_for_kernel((const void *)k_vol_trace, 128);
    const VolCKernel k_cs =
        (scene->mat_mask & ~kClassicMats) == 0 ? k_vol_c<kClassicMats, true> : k_vol_c<kAllMats, true>;
    const int g_a = grid_for_kernel((const void *)k_vol_a, 128);
    const int g_b = grid_for_kernel((const void *)k_vol_b, 128);
    const int g_cs = grid_for_kernel((const void *)k_cs, 128);
    const bool unbounded = sc.max_depth == -1;
    const int passes = unbounded ? LJ_MAX_BOUNCES + 2 : std::max(1, sc.max_depth);
    const float spread0 = 0.25f / (float)std::max(W, H);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (stats) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, s);
    }
    int64_t launches = 0;
    // LJ_RENDER_PROFILE: an event pair around every kernel, grouped by class
    const bool profile = stats && (params->flags & LJ_RENDER_PROFILE);
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
    int64_t class_launches[LJ_KERNEL_CLASSES] = {};
    // LJ_RENDER_COUNT_BVH: rays / nodes / prims of the closest-hit queues
    const bool count_bvh = stats && (params->flags & LJ_RENDER_COUNT_BVH);
    unsigned long long *bvhc = nullptr;
    if (count_bvh) {
        LJ_CUDA_TRY(cudaMallocAsync(&bvhc, 3 * sizeof(unsigned long long), s));
        LJ_CUDA_TRY(cudaMemsetAsync(bvhc, 0, 3 * sizeof(unsigned long long), s));
    }
    auto mark_begin = [&](int cls) {
        class_launches[cls]++;
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
    for (int sb = 0; sb < spp; sb += nsamp) {
        int ns = std::min(nsamp, spp - sb);
        int Pb = num_pixels * ns;
        k_vol_set_counts<<<1, 1, 0, s>>>(q.counts, Pb);
        class_launches[LJ_KERNEL_OTHER]++;
        mark_begin(LJ_KERNEL_CAMERA);
        k_vol_camera<<<(Pb + 255) / 256, 256, 0, s>>>(sc, ps, q, Pb, num_pixels, params->sample_offset + sb,
                                                      params->seed);
        mark_end();
        launches += 2;
        int curq = 0;
        for (int pass = 0; pass < passes; pass++) {
            k_vol_zero<<<1, 1, 0, s>>>(q.counts, curq ^ 1);
            class_launches[LJ_KERNEL_OTHER]++;
            mark_begin(LJ_KERNEL_TRACE);
            k_vol_trace<<<g_trace, 128, 0, s>>>(sc.bvh, q.ray[curq], q.hit, q.counts + curq, q.counts + 8,
                                                q.stats + 0, ctx->d_status);
            mark_end();
            if (count_bvh)
                launch_trace_counters_queue(sc.bvh, q.ray[curq], q.counts + curq, Pb, LJ_COUNT_BVH_STRIDE, false,
                                            bvhc, ctx->d_status, s);
            mark_begin(LJ_KERNEL_MEDIUM);
            k_vol_a<<<g_a, 128, 0, s>>>(sc, ps, q, curq, spread0, ctx->d_status);
            mark_end();
            mark_begin(LJ_KERNEL_NEE);
            k_vol_b<<<g_b, 128, 0, s>>>(sc, ps, q, curq, spread0, ctx->d_status);
            mark_end();
            mark_begin(LJ_KERNEL_MEDIUM);
            k_cs<<<g_cs, 128, 0, s>>>(sc, ps, q, curq, spread0);
            mark_end();
            launches += 5;
            curq ^= 1;
            // stop once every path of the batch has ended
            if ((pass & 3) == 3 && pass + 1 < passes) {
                int c = 0;
                LJ_CUDA_TRY(cudaMemcpyAsync(&c, q.counts + curq, sizeof(int), cudaMemcpyDeviceToHost, s));
                LJ_CUDA_TRY(cudaStreamSynchronize(s));
                if (c == 0) break;
            }
        }
        k_vol_resolve<<<(num_pixels + 255) / 256, 256, 0, s>>>(ps.L, num_pixels, ns, d_out);
        launches++;
        class_launches[LJ_KERNEL_OTHER]++;
    }
    int64_t nfl = 3 * (int64_t)num_pixels;
    k_vol_scale<<<(int)((nfl + 255) / 256), 256, 0, s>>>(d_out, nfl, 1.0f / spp);
    launches++;
    class_launches[LJ_KERNEL_OTHER]++;
    LJ_CUDA_TRY(cudaGetLastError());
    if (stats) {
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
        stats->null_collisions = (int64_t)st[3];
        stats->real_collisions = (int64_t)st[4];
        stats->kernel_launches = launches;
        if (count_bvh) {
            unsigned long long c[3];
            LJ_CUDA_TRY(cudaMemcpyAsync(c, bvhc, sizeof(c), cudaMemcpyDeviceToHost, s));
            LJ_CUDA_TRY(cudaFreeAsync(bvhc, s));
            LJ_CUDA_TRY(cudaStreamSynchronize(s));
            stats->bvh_rays[0] = (int64_t)c[0];
            stats->bvh_nodes[0] = (int64_t)c[1];
            stats->bvh_prims[0] = (int64_t)c[2];
        }
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
            for (int c = 0; c < LJ_KERNEL_CLASSES; c++)
                if (c != LJ_KERNEL_OTHER) other -= stats->class_ms[c];
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
    return LJ_OK;
}

}  // namespace lj
