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
// Path state travels with its queue entry (every kernel reads its queue
// contiguously); an ended path leaves its radiance in its sample slot, and
// the slots are reduced per pixel in sample order, so the image is
// deterministic.
#include <algorithm>
#include <cstring>
#include <vector>

#include "lj_host.h"
#include "lj_trace_queue.cuh"
#include "lj_wavefront.cuh"

namespace lj {

namespace {

__global__ void k_camera(DevScene sc, Queues q, int P, int num_pixels, int sample_base, uint64_t seed) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const PathSoA &ps = q.st[0];
    int pixel = p % num_pixels;
    int sample = sample_base + p / num_pixels;
    Pcg rng = pcg_keyed(seed, (uint64_t)pixel, (uint64_t)sample);
    int x = pixel % sc.cam.w, y = pixel / sc.cam.w;
    float r1 = pcg_uniform(rng), r2 = pcg_uniform(rng);
    V3 o, d;
    camera_ray(sc.cam, (x + r1) / sc.cam.w, (y + r2) / sc.cam.h, o, d);
    q.ray[0][2 * p] = make_float4(o.x, o.y, o.z, 0.0f);
    q.ray[0][2 * p + 1] = make_float4(d.x, d.y, d.z, __int_as_float(0x7f800000));
    ps.slot[p] = p;
    ps.pixel[p] = pixel;
    ps.rng[p] = rng.state;
    ps.beta[p] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    ps.L[p] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    ps.prev[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    ps.nv[p] = 2;
}

// Persistent warps with dynamic ray fetch (lj_trace_queue.cuh); *fetch is
// zeroed before each launch.
__global__ void __launch_bounds__(128, 8) k_trace_queue(DevBvh bvh, const float4 *rays, float4 *hits,
                                                     const int *count, int *fetch, unsigned long long *stat,
                                                     int *status) {
    const int n = *count;
    if (blockIdx.x == 0 && threadIdx.x == 0 && stat) atomicAdd(stat, (unsigned long long)n);
    ClosestQueueIO io{bvh, rays, hits};
    trace_queue<false, 128>(io, n, fetch, status);
}

// Lnext: the radiance of the next queue's entries (the paths that go on)
__global__ void __launch_bounds__(128, 8) k_trace_shadow(DevBvh bvh, const float4 *rays, const int *targets,
                                                      const float4 *contrib, const int *count, int *fetch,
                                                      float4 *Lnext, float4 *Lres, unsigned long long *stat,
                                                      int *status) {
    const int n = *count;
    if (blockIdx.x == 0 && threadIdx.x == 0 && stat) atomicAdd(stat, (unsigned long long)n);
    ShadowQueueIO io{bvh, rays, targets, contrib, Lnext, Lres};
    trace_queue<true, 128>(io, n, fetch, status);
}

// One instance per material set (kMats): a scene of Lambertian surfaces only
// runs a much smaller kernel than one that may meet every Disney lobe, and a
// scene of combined Disney BSDFs alone one without the other eight types.
template <uint32_t kMats>
// (8 blocks per SM (64 registers) for the instances with Disney code, 6 for
// the others: spilled registers cost less than the warps fewer blocks would
// lose -- the shade step waits on memory; the Lambertian / classic
// instances at 6 are -6 to -11 % against 4 and 5 blocks and gain nothing at
// 8, the Disney-BSDF instance at 8 shades the full terrain 9 % faster than
// at 6, and 6 % faster at 6 than the every-type instance at 5)
__global__ void __launch_bounds__(128, (kMats & ~kClassicMats) != 0 ? 8 : 6) k_shade(DevScene sc, Queues q, int cur, float spread0,
                                                                         int *status) {
    const int n = q.counts[cur];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(q.stats + 2, (unsigned long long)n);
    const ShadeCfg cfg{sc.max_depth, sc.rr_depth, spread0};
    const OrderedPaths paths{q, cur};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        shade_segment<kMats>(sc, paths, i, cfg, status);
}
using ShadeKernel = void (*)(DevScene, Queues, int, float, int *);

// Paths still in queue cur when the passes end: their radiance to their slots.
__global__ void k_flush(Queues q, int cur) {
    const int n = q.counts[cur];
    const PathSoA &s = q.state(cur);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) q.Lres[s.slot[i]] = s.L[i];
}
// the smallest instance whose material set covers the scene's
ShadeKernel shade_kernel_for(uint32_t mat_mask) {
    if ((mat_mask & ~kLambertMats) == 0) return k_shade<kLambertMats>;
    if ((mat_mask & ~kClassicMats) == 0) return k_shade<kClassicMats>;
    if ((mat_mask & ~kDisneyBsdfMats) == 0) return k_shade<kDisneyBsdfMats>;
    return k_shade<kAllMats>;
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

// counts: [0], [1] ray queues, [2] shadow queue, [8], [9] ray fetch
// counters of the closest / shadow traversal kernels
__global__ void k_set_counts(int *counts, int c0) {
    counts[0] = c0;
    counts[1] = 0;
    counts[2] = 0;
    counts[8] = 0;
    counts[9] = 0;
}
__global__ void k_zero2(int *counts, int a, int b) {
    counts[a] = 0;
    counts[b] = 0;
    counts[8] = 0;
    counts[9] = 0;
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
    for (int k = 0; k < 2; k++) {   // state of queue k: slot, pixel, rng, beta, L, prev, nv
        add(P * 4); add(P * 4); add(P * 8); add(P * 16); add(P * 16); add(P * 16); add(P * 4);
    }
    add(P * 32); add(P * 32); add(P * 16);   // rays of both queues, hits
    add(P * 32); add(P * 4); add(P * 16);    // shadow rays, targets, contributions
    add(P * 16);                             // radiance per sample slot
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
                lj_stats *stats, bool sync_stats, const lj_job_desc *job) {
    lj_ctx *ctx = scene->ctx;
    DevScene sc = scene->dev;   // job overrides: resolution (camera) and depth options
    int W = scene->width, H = scene->height;
    int max_depth = scene->options.max_depth;
    if (job && job->width > 0 && job->height > 0) {
        W = job->width;
        H = job->height;
        make_cam_rec(scene->camera, W, H, sc.cam);
    }
    if (job && job->override_depth) {
        if (job->max_depth < -1) return set_error(ctx, LJ_ERR_INVALID_ARG, "render: max_depth must be >= -1");
        sc.max_depth = max_depth = job->max_depth;
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
    Queues q;
    for (int k = 0; k < 2; k++) {
        PathSoA &ps = q.st[k];
        ps.slot = carve<int>(cur, P);
        ps.pixel = carve<int>(cur, P);
        ps.rng = carve<uint64_t>(cur, P);
        ps.beta = carve<float4>(cur, P);
        ps.L = carve<float4>(cur, P);
        ps.prev = carve<float4>(cur, P);
        ps.nv = carve<int>(cur, P);
    }
    q.ray[0] = carve<float4>(cur, 2 * P);
    q.ray[1] = carve<float4>(cur, 2 * P);
    q.hit = carve<float4>(cur, P);
    q.sray = carve<float4>(cur, 2 * P);
    q.starget = carve<int>(cur, P);
    q.scontrib = carve<float4>(cur, P);
    q.Lres = carve<float4>(cur, P);
    q.counts = carve<int>(cur, 16);
    q.stats = carve<unsigned long long>(cur, 8);

    LJ_CUDA_TRY(cudaMemsetAsync(q.stats, 0, 8 * sizeof(unsigned long long), s));
    LJ_CUDA_TRY(cudaMemsetAsync(d_out, 0, sizeof(float) * 3 * (size_t)num_pixels, s));
    const int g_trace = grid_persistent((const void *)k_trace_queue, 128);
    const int g_shadow = grid_persistent((const void *)k_trace_shadow, 128);
    const ShadeKernel shade = shade_kernel_for(scene->mat_mask);
    const int g_shade = grid_persistent((const void *)shade, 128);
    const int passes = max_depth == -1 ? LJ_MAX_BOUNCES + 1 : std::max(1, max_depth);
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
    int64_t class_launches[LJ_KERNEL_CLASSES] = {};
    // LJ_RENDER_COUNT_BVH: rays / nodes / prims of closest [0..2] and shadow [3..5] queues
    const bool count_bvh = timed && (params->flags & LJ_RENDER_COUNT_BVH);
    unsigned long long *bvhc = nullptr;
    if (count_bvh) {
        LJ_CUDA_TRY(cudaMallocAsync(&bvhc, 6 * sizeof(unsigned long long), s));
        LJ_CUDA_TRY(cudaMemsetAsync(bvhc, 0, 6 * sizeof(unsigned long long), s));
    }
    for (int sb = 0; sb < spp; sb += nsamp) {
        int ns = std::min(nsamp, spp - sb);
        int Pb = num_pixels * ns;
        k_set_counts<<<1, 1, 0, s>>>(q.counts, Pb);
        mark_begin(LJ_KERNEL_CAMERA);
        k_camera<<<(Pb + 255) / 256, 256, 0, s>>>(sc, q, Pb, num_pixels, params->sample_offset + sb,
                                                  params->seed);
        mark_end();
        launches += 2;
        class_launches[LJ_KERNEL_OTHER]++;
        class_launches[LJ_KERNEL_CAMERA]++;
        int curq = 0;
        for (int pass = 0; pass < passes; pass++) {
            k_zero2<<<1, 1, 0, s>>>(q.counts, curq ^ 1, 2);
            mark_begin(LJ_KERNEL_TRACE);
            k_trace_queue<<<g_trace, 128, 0, s>>>(sc.bvh, q.ray[curq], q.hit, q.counts + curq, q.counts + 8,
                                                  q.stats + 0, ctx->d_status);
            mark_end();
            if (count_bvh)
                launch_trace_counters_queue(sc.bvh, q.ray[curq], q.counts + curq, Pb, LJ_COUNT_BVH_STRIDE, false,
                                            bvhc, ctx->d_status, s);
            mark_begin(LJ_KERNEL_SHADE);
            shade<<<g_shade, 128, 0, s>>>(sc, q, curq, spread0, ctx->d_status);
            mark_end();
            mark_begin(LJ_KERNEL_SHADOW);
            k_trace_shadow<<<g_shadow, 128, 0, s>>>(sc.bvh, q.sray, q.starget, q.scontrib, q.counts + 2,
                                                    q.counts + 9, q.st[curq ^ 1].L, q.Lres, q.stats + 1,
                                                    ctx->d_status);
            mark_end();
            if (count_bvh)
                launch_trace_counters_queue(sc.bvh, q.sray, q.counts + 2, Pb, LJ_COUNT_BVH_STRIDE, true, bvhc + 3,
                                            ctx->d_status, s);
            launches += 4;
            class_launches[LJ_KERNEL_OTHER]++;
            class_launches[LJ_KERNEL_TRACE]++;
            class_launches[LJ_KERNEL_SHADE]++;
            class_launches[LJ_KERNEL_SHADOW]++;
            curq ^= 1;
            // stop early once every path of the batch has ended (paths end
            // well before a large max_depth through escapes and roulette)
            if ((max_depth == -1 || max_depth > 8) && (pass & 3) == 3 && pass + 1 < passes) {
                int c = 0;
                LJ_CUDA_TRY(cudaMemcpyAsync(&c, q.counts + curq, sizeof(int), cudaMemcpyDeviceToHost, s));
                LJ_CUDA_TRY(cudaStreamSynchronize(s));
                if (c == 0) break;
            }
        }
        // paths the pass limit stopped: their radiance to their slots
        k_flush<<<g_shade, 128, 0, s>>>(q, curq);
        k_resolve<<<(num_pixels + 255) / 256, 256, 0, s>>>(q.Lres, num_pixels, ns, d_out);
        launches += 2;
        class_launches[LJ_KERNEL_OTHER] += 2;
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
        if (count_bvh) {
            unsigned long long c[6];
            LJ_CUDA_TRY(cudaMemcpyAsync(c, bvhc, sizeof(c), cudaMemcpyDeviceToHost, s));
            LJ_CUDA_TRY(cudaFreeAsync(bvhc, s));
            LJ_CUDA_TRY(cudaStreamSynchronize(s));
            for (int k = 0; k < 2; k++) {
                stats->bvh_rays[k] = (int64_t)c[3 * k];
                stats->bvh_nodes[k] = (int64_t)c[3 * k + 1];
                stats->bvh_prims[k] = (int64_t)c[3 * k + 2];
            }
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
    cudaStream_t s = (cudaStream_t)stream;   // NULL: the legacy default stream
    if (stats) memset(stats, 0, sizeof(*stats));
    // integrator dispatch, src/render.cpp:155-170
    if (scene->options.integrator == LJ_INTEGRATOR_PATH)
        return render_path(scene, params, d_out_rgb, s, stats, stats != nullptr, nullptr);
    if (scene->options.integrator == LJ_INTEGRATOR_VOLPATH) {
        // versions 1-5 are simplifications of 6 for homework; 0 and 6 select the full one
        if (scene->options.vol_path_version != 0 && scene->options.vol_path_version != 6)
            return set_error(scene->ctx, LJ_ERR_UNSUPPORTED, "render: only vol_path_version 0 / 6 is built");
        return render_volpath(scene, params, d_out_rgb, s, stats, nullptr);
    }
    if (scene->options.integrator >= LJ_INTEGRATOR_DEPTH && scene->options.integrator <= LJ_INTEGRATOR_MIPMAP_LEVEL)
        return render_aux(scene, params, d_out_rgb, s, stats);
    return set_error(scene->ctx, LJ_ERR_UNSUPPORTED, "render: unknown integrator");
}

int lj_gpu_render_job_device(lj_scene *scene, const lj_job_desc *job, float *d_out_rgb, void *stream,
                             lj_stats *stats) {
    if (!scene || !job || !d_out_rgb) return LJ_ERR_INVALID_ARG;
    const bool vol = scene->options.integrator == LJ_INTEGRATOR_VOLPATH &&
                     (scene->options.vol_path_version == 0 || scene->options.vol_path_version == 6);
    if (scene->options.integrator != LJ_INTEGRATOR_PATH && !vol)
        return set_error(scene->ctx, LJ_ERR_UNSUPPORTED, "render_job: path and volpath (v6) scenes only");
    if ((job->width > 0) != (job->height > 0))
        return set_error(scene->ctx, LJ_ERR_INVALID_ARG, "render_job: give both width and height, or neither");
    cudaSetDevice(scene->ctx->device);
    if (stats) memset(stats, 0, sizeof(*stats));
    lj_render_params p{};
    p.seed = job->seed;
    p.spp = job->spp;
    p.sample_offset = job->sample_offset;
    p.flags = job->flags;
    if (vol) return render_volpath(scene, &p, d_out_rgb, (cudaStream_t)stream, stats, job);
    return render_path(scene, &p, d_out_rgb, (cudaStream_t)stream, stats, stats != nullptr, job);
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
