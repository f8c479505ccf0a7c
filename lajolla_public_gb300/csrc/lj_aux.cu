// Auxiliary buffers: the GPU form of aux_render (src/render.cpp:12-69).
// One thread per pixel: a ray through the pixel centre, closest hit, then
// the quantity the integrator names (depth, shading normal, mean curvature,
// ray differential, mipmap level); black where nothing is hit.  No random
// numbers are used, so the image does not depend on the seed or spp.
#include <cstring>

#include "lj_host.h"
#include "lj_shade.cuh"
#include "lj_trace.cuh"

namespace lj {

namespace {

__global__ void __launch_bounds__(128) k_aux(DevScene sc, int integrator, float *out, int *status) {
    const int w = sc.cam.w, h = sc.cam.h;
    int pixel = blockIdx.x * blockDim.x + threadIdx.x;
    if (pixel >= w * h) return;
    int x = pixel % w, y = pixel / w;
    V3 o, d;
    camera_ray(sc.cam, (x + 0.5f) / w, (y + 0.5f) / h, o, d);
    const float spread = 0.25f / (float)max(w, h);   // init_ray_differential, src/ray.h:35-37
    TraceHit hit{0.0f, -1, 0.0f, 0.0f};
    int ovf = 0;
    bool found = trace_bvh<false>(sc.bvh, o, d, 0.0f, __int_as_float(0x7f800000), hit, &ovf);
    if (ovf) atomicOr(status, kStatusStackOverflow);
    V3 c{0.0f, 0.0f, 0.0f};
    if (found) {
        Vertex vx = make_vertex(sc, o, d, hit.t, hit.prim, hit.u, hit.v, spread);
        switch (integrator) {
        case LJ_INTEGRATOR_DEPTH: {
            float dist = length(vx.p - o);
            c = V3{dist, dist, dist};
            break;
        }
        case LJ_INTEGRATOR_SHADING_NORMAL: c = vx.frame.n; break;
        case LJ_INTEGRATOR_MEAN_CURVATURE: c = V3{vx.mean_curvature, vx.mean_curvature, vx.mean_curvature}; break;
        case LJ_INTEGRATOR_RAY_DIFFERENTIAL: c = V3{0.0f, spread, 0.0f}; break;
        case LJ_INTEGRATOR_MIPMAP_LEVEL: {
            // get_texture: slot 0 of every material; DisneyClearcoat gives a
            // constant (src/materials/disney_clearcoat.inl:51-53)
            const MatRec &m = sc.mats[vx.material];
            if (m.type != LJ_MAT_DISNEY_CLEARCOAT && m.tex[0].kind == LJ_TEX_IMAGE) {
                const MipLevel &l0 = sc.image_levels[m.tex[0].image_id * 8];
                float scaled = (float)max(l0.w, l0.h) * fmaxf(m.tex[0].us, m.tex[0].vs) * vx.uv_screen_size;
                float level = log2f(fmaxf(scaled, 1e-8f));
                c = V3{level, level, level};
            }
            break;
        }
        default: break;
        }
    }
    out[3 * pixel] = c.x;
    out[3 * pixel + 1] = c.y;
    out[3 * pixel + 2] = c.z;
}

}  // namespace

int render_aux(lj_scene *scene, const lj_render_params *params, float *d_out, cudaStream_t s,
               lj_stats *stats) {
    (void)params;
    lj_ctx *ctx = scene->ctx;
    std::string e;
    std::string *err = &e;
    const int num_pixels = scene->width * scene->height;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (stats) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, s);
    }
    k_aux<<<(num_pixels + 127) / 128, 128, 0, s>>>(scene->dev, scene->options.integrator, d_out,
                                                   ctx->d_status);
    LJ_CUDA_TRY(cudaGetLastError());
    if (stats) {
        cudaEventRecord(e1, s);
        LJ_CUDA_TRY(cudaStreamSynchronize(s));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        stats->device_ms = ms;
        stats->samples = num_pixels;
        stats->rays_closest = num_pixels;
        stats->path_segments = num_pixels;
        stats->kernel_launches = 1;
        stats->class_launches[LJ_KERNEL_TRACE] = 1;
        stats->class_ms[LJ_KERNEL_TRACE] = ms;
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
