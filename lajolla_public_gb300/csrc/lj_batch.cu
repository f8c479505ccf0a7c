// Batch entry points for per-function parity tests and microbenchmarks:
//   lj_gpu_bsdf_batch          eval / sample_bsdf / pdf_sample_bsdf (src/material.cpp:90-119)
//   lj_gpu_light_sample_batch  sample_light + sample_point_on_light + pdfs
//                              (src/scene.cpp:61-67, src/light.cpp:56-77)
//   lj_gpu_phase_batch         Henyey-Greenstein / isotropic (src/phase_function.cpp:30-47)
//   lj_gpu_light_emission_batch  emission (src/light.cpp:56-77)
//   lj_gpu_camera_ray_batch    sample_primary + pixel filters (src/camera.cpp:23-47)
//   lj_gpu_medium_batch        get_sigma_a / get_sigma_s / get_majorant (src/medium.cpp:27-37)
// One thread per query; inputs and outputs are flat FP32 arrays in HBM.
#include "lj_host.h"
#include "lj_phase.cuh"
#include "lj_shade.cuh"
#include "lj_volwave.cuh"

namespace lj {
namespace {

// The vertex of src/tests/materials.cpp:55-60: n = ng = +z, frame from n.
__device__ BsdfVertex local_vertex() {
    BsdfVertex v;
    v.ng = V3{0, 0, 1};
    v.frame = frame_from_n(V3{0, 0, 1});
    return v;
}

__global__ void k_bsdf_batch(lj_bsdf_batch b, int np, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *pp = b.d_params + i * np;
    MatParams m;
    m.type = b.material_type;
    int k = 0;
#pragma unroll
    for (int s = 0; s < kMatSlots; s++) {
        int w = slot_width(b.material_type, s);
        if (w == 3) {
            m.s[s] = V3{pp[k], pp[k + 1], pp[k + 2]};
            k += 3;
        } else if (w == 1) {
            m.s[s] = V3{pp[k], pp[k], pp[k]};
            k += 1;
        } else {
            m.s[s] = V3{0, 0, 0};
        }
    }
    m.eta = pp[k];
    BsdfVertex v = local_vertex();
    V3 wi{b.d_dir_in[3 * i], b.d_dir_in[3 * i + 1], b.d_dir_in[3 * i + 2]};
    if (b.op == LJ_BSDF_OP_EVAL) {
        V3 wo{b.d_dir_out[3 * i], b.d_dir_out[3 * i + 1], b.d_dir_out[3 * i + 2]};
        V3 f = bsdf_eval(m, v, wi, wo, b.transport_to_view != 0);
        b.d_out_value[3 * i] = f.x;
        b.d_out_value[3 * i + 1] = f.y;
        b.d_out_value[3 * i + 2] = f.z;
    } else if (b.op == LJ_BSDF_OP_PDF) {
        V3 wo{b.d_dir_out[3 * i], b.d_dir_out[3 * i + 1], b.d_dir_out[3 * i + 2]};
        b.d_out_pdf[i] = bsdf_pdf(m, v, wi, wo);
    } else {
        BsdfSample s = bsdf_sample(m, v, wi, b.d_rnd[3 * i], b.d_rnd[3 * i + 1], b.d_rnd[3 * i + 2]);
        b.d_out_dir[3 * i] = s.dir.x;
        b.d_out_dir[3 * i + 1] = s.dir.y;
        b.d_out_dir[3 * i + 2] = s.dir.z;
        if (b.d_out_eta) b.d_out_eta[i] = s.eta;
        if (b.d_out_roughness) b.d_out_roughness[i] = s.roughness;
        if (b.d_out_valid) b.d_out_valid[i] = s.valid ? 1 : 0;
    }
}

__global__ void k_light_batch(DevScene sc, const float *ref, const float *rnd, int32_t *out_light,
                              float *out_point, float *out_normal, float *out_pdf, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V3 p{ref[3 * i], ref[3 * i + 1], ref[3 * i + 2]};
    const float *r = rnd + 4 * i;
    int lid = sample_light(sc, r[0]);
    PN pn = sample_point_on_light(sc, lid, p, r[1], r[2], r[3]);
    out_light[i] = lid;
    out_point[3 * i] = pn.p.x; out_point[3 * i + 1] = pn.p.y; out_point[3 * i + 2] = pn.p.z;
    out_normal[3 * i] = pn.n.x; out_normal[3 * i + 1] = pn.n.y; out_normal[3 * i + 2] = pn.n.z;
    out_pdf[i] = __ldg(sc.light_pmf + lid) * pdf_point_on_light(sc, lid, pn, p);
}

__global__ void k_phase_batch(int kind, float g, const float *din, const float *dout, const float *rnd,
                              float *val, float *pdf, float *dir, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V3 wi{din[3 * i], din[3 * i + 1], din[3 * i + 2]};
    if (dout && (val || pdf)) {
        V3 wo{dout[3 * i], dout[3 * i + 1], dout[3 * i + 2]};
        float v = phase_eval(kind, g, wi, wo);
        if (val) val[i] = v;
        if (pdf) pdf[i] = v;
    }
    if (dir && rnd) {
        V3 d = phase_sample(kind, g, wi, rnd[2 * i], rnd[2 * i + 1]);
        dir[3 * i] = d.x; dir[3 * i + 1] = d.y; dir[3 * i + 2] = d.z;
    }
}

__global__ void k_emission_batch(DevScene sc, const int32_t *light, const float *view, const float *point,
                                 const float *normal, float *out, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int lid = light[i];
    V3 e;
    if (lid < 0 || lid >= sc.num_lights) {
        e = V3{__int_as_float(0x7fc00000), __int_as_float(0x7fc00000), __int_as_float(0x7fc00000)};
    } else {
        const V3 vd{view[3 * i], view[3 * i + 1], view[3 * i + 2]};
        PN pn{V3{point[3 * i], point[3 * i + 1], point[3 * i + 2]},
              V3{normal[3 * i], normal[3 * i + 1], normal[3 * i + 2]}};
        e = light_emission(sc, lid, vd, pn);
    }
    out[3 * i] = e.x; out[3 * i + 1] = e.y; out[3 * i + 2] = e.z;
}

__global__ void k_camera_batch(CamRec cam, const float *screen, float *org, float *dir, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V3 o, d;
    camera_ray(cam, screen[2 * i], screen[2 * i + 1], o, d);
    org[3 * i] = o.x; org[3 * i + 1] = o.y; org[3 * i + 2] = o.z;
    dir[3 * i] = d.x; dir[3 * i + 1] = d.y; dir[3 * i + 2] = d.z;
}

// sigma_a = density * (1 - albedo), sigma_s = density * albedo
// (src/media/heterogeneous.inl:11-21); the constants of a homogeneous medium.
__global__ void k_medium_batch(const MediumRec *media, int mid, const float *pts, const float *dirs, float *sa,
                               float *ss, float *maj, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const MediumRec &m = media[mid];
    const V3 p{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    if (sa || ss) {
        V3 a, s;
        if (m.kind == LJ_MEDIUM_HOMOGENEOUS) {
            a = V3{m.sigma_a[0], m.sigma_a[1], m.sigma_a[2]};
            s = V3{m.sigma_s[0], m.sigma_s[1], m.sigma_s[2]};
        } else {
            const V3 d = vol_lookup(m.density, p), al = vol_lookup(m.albedo, p);
            s = d * al;
            a = d * (V3{1, 1, 1} - al);
        }
        if (sa) { sa[3 * i] = a.x; sa[3 * i + 1] = a.y; sa[3 * i + 2] = a.z; }
        if (ss) { ss[3 * i] = s.x; ss[3 * i + 1] = s.y; ss[3 * i + 2] = s.z; }
    }
    if (maj) {
        const V3 d{dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]};
        const V3 mj = majorant(m, p, d);
        maj[3 * i] = mj.x; maj[3 * i + 1] = mj.y; maj[3 * i + 2] = mj.z;
    }
}

inline int blocks(int64_t n) { return (int)((n + 255) / 256); }

}  // namespace
}  // namespace lj

using namespace lj;

extern "C" {

int lj_gpu_bsdf_param_count(int32_t type) {
    if (type < 0 || type >= LJ_MAT_COUNT) return -1;
    return bsdf_param_count(type);
}

int lj_gpu_bsdf_batch(lj_ctx *ctx, const lj_bsdf_batch *b, int64_t n, void *stream) {
    if (!ctx || !b || n < 0) return LJ_ERR_INVALID_ARG;
    if (b->material_type < 0 || b->material_type >= LJ_MAT_COUNT)
        return set_error(ctx, LJ_ERR_INVALID_ARG, "bsdf_batch: unknown material type");
    if (b->op < LJ_BSDF_OP_EVAL || b->op > LJ_BSDF_OP_SAMPLE)
        return set_error(ctx, LJ_ERR_INVALID_ARG, "bsdf_batch: unknown op");
    if (n == 0) return LJ_OK;
    bool ok = b->d_params && b->d_dir_in;
    if (b->op == LJ_BSDF_OP_EVAL) ok = ok && b->d_dir_out && b->d_out_value;
    if (b->op == LJ_BSDF_OP_PDF) ok = ok && b->d_dir_out && b->d_out_pdf;
    if (b->op == LJ_BSDF_OP_SAMPLE) ok = ok && b->d_rnd && b->d_out_dir;
    if (!ok) return set_error(ctx, LJ_ERR_INVALID_ARG, "bsdf_batch: missing buffer for this op");
    cudaSetDevice(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;   // NULL: the legacy default stream
    k_bsdf_batch<<<blocks(n), 256, 0, s>>>(*b, bsdf_param_count(b->material_type), n);
    if (cudaGetLastError() != cudaSuccess) return set_error(ctx, LJ_ERR_CUDA, "bsdf_batch launch failed");
    return LJ_OK;
}

int lj_gpu_light_sample_batch(lj_scene *sc, const float *ref, const float *rnd, int32_t *out_light,
                              float *out_point, float *out_normal, float *out_pdf, int64_t n, void *stream) {
    if (!sc || n < 0 || (n > 0 && (!ref || !rnd || !out_light || !out_point || !out_normal || !out_pdf)))
        return LJ_ERR_INVALID_ARG;
    if (sc->dev.num_lights == 0) return set_error(sc->ctx, LJ_ERR_INVALID_ARG, "light_sample_batch: scene has no lights");
    if (n == 0) return LJ_OK;
    cudaSetDevice(sc->ctx->device);
    cudaStream_t s = (cudaStream_t)stream;   // NULL: the legacy default stream
    k_light_batch<<<blocks(n), 256, 0, s>>>(sc->dev, ref, rnd, out_light, out_point, out_normal, out_pdf, n);
    if (cudaGetLastError() != cudaSuccess) return set_error(sc->ctx, LJ_ERR_CUDA, "light_sample_batch launch failed");
    return LJ_OK;
}

int lj_gpu_phase_batch(lj_ctx *ctx, int32_t kind, float g, const float *d_dir_in, const float *d_dir_out,
                       const float *d_rnd, float *d_out_value, float *d_out_pdf, float *d_out_dir, int64_t n,
                       void *stream) {
    if (!ctx || n < 0 || (kind != LJ_PHASE_ISOTROPIC && kind != LJ_PHASE_HG)) return LJ_ERR_INVALID_ARG;
    if (n > 0 && !d_dir_in) return LJ_ERR_INVALID_ARG;
    if (n == 0) return LJ_OK;
    cudaSetDevice(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;   // NULL: the legacy default stream
    k_phase_batch<<<blocks(n), 256, 0, s>>>(kind, g, d_dir_in, d_dir_out, d_rnd, d_out_value, d_out_pdf,
                                            d_out_dir, n);
    if (cudaGetLastError() != cudaSuccess) return set_error(ctx, LJ_ERR_CUDA, "phase_batch launch failed");
    return LJ_OK;
}

int lj_gpu_light_emission_batch(lj_scene *sc, const int32_t *d_light, const float *d_view_dir, const float *d_point,
                                const float *d_normal, float *d_out, int64_t n, void *stream) {
    if (!sc || n < 0 || (n > 0 && (!d_light || !d_view_dir || !d_point || !d_normal || !d_out)))
        return LJ_ERR_INVALID_ARG;
    if (n == 0) return LJ_OK;
    cudaSetDevice(sc->ctx->device);
    cudaStream_t s = (cudaStream_t)stream;   // NULL: the legacy default stream
    k_emission_batch<<<blocks(n), 256, 0, s>>>(sc->dev, d_light, d_view_dir, d_point, d_normal, d_out, n);
    if (cudaGetLastError() != cudaSuccess) return set_error(sc->ctx, LJ_ERR_CUDA, "light_emission_batch launch failed");
    return LJ_OK;
}

int lj_gpu_camera_ray_batch(lj_scene *sc, const float *d_screen, float *d_out_org, float *d_out_dir, int64_t n,
                            void *stream) {
    if (!sc || n < 0 || (n > 0 && (!d_screen || !d_out_org || !d_out_dir))) return LJ_ERR_INVALID_ARG;
    if (n == 0) return LJ_OK;
    cudaSetDevice(sc->ctx->device);
    cudaStream_t s = (cudaStream_t)stream;   // NULL: the legacy default stream
    k_camera_batch<<<blocks(n), 256, 0, s>>>(sc->dev.cam, d_screen, d_out_org, d_out_dir, n);
    if (cudaGetLastError() != cudaSuccess) return set_error(sc->ctx, LJ_ERR_CUDA, "camera_ray_batch launch failed");
    return LJ_OK;
}

int lj_gpu_medium_batch(lj_scene *sc, int32_t medium_id, const float *d_points, const float *d_dirs,
                        float *d_out_sigma_a, float *d_out_sigma_s, float *d_out_majorant, int64_t n,
                        void *stream) {
    if (!sc || n < 0) return LJ_ERR_INVALID_ARG;
    if (medium_id < 0 || medium_id >= sc->dev.num_media)
        return set_error(sc->ctx, LJ_ERR_INVALID_ARG, "medium_batch: medium id out of range");
    if (n > 0 && (!d_points || (d_out_majorant && !d_dirs)))
        return set_error(sc->ctx, LJ_ERR_INVALID_ARG, "medium_batch: missing input buffer");
    if (n == 0 || (!d_out_sigma_a && !d_out_sigma_s && !d_out_majorant)) return LJ_OK;
    cudaSetDevice(sc->ctx->device);
    cudaStream_t s = (cudaStream_t)stream;   // NULL: the legacy default stream
    k_medium_batch<<<blocks(n), 256, 0, s>>>(sc->dev.media, medium_id, d_points, d_dirs, d_out_sigma_a,
                                             d_out_sigma_s, d_out_majorant, n);
    if (cudaGetLastError() != cudaSuccess) return set_error(sc->ctx, LJ_ERR_CUDA, "medium_batch launch failed");
    return LJ_OK;
}

}  // extern "C"
