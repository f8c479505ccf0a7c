// C ABI entry points (include/lj_gpu.h): context, scene upload + device BVH
// build, batch ray casting, Morton sort.  The host-side preparation mirrors
// Scene::Scene (src/scene.cpp:4-53): triangle area tables
// (src/shapes/triangle_mesh.inl:60-75), light power table (src/scene.cpp:47-52,
// src/lights/*.inl light_power), envmap mipmaps and 2D sampling table
// (src/mipmap.h:25-48, src/lights/envmap.inl:75-98), camera matrices
// (src/camera.cpp:7-21), bounding sphere and epsilons (src/scene.cpp:29-34,
// src/scene.h:99-105).  Tables are built in double precision, as the
// reference does, and stored as FP32.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <thread>

#include "lj_host.h"

using namespace lj;

namespace lj {

int set_error(lj_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->last_error = msg;
    return code;
}

}  // namespace lj

namespace {

struct M4d {
    double m[16];
};
M4d m4_mul(const M4d &a, const M4d &b) {
    M4d r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double s = 0;
            for (int k = 0; k < 4; k++) s += a.m[i * 4 + k] * b.m[k * 4 + j];
            r.m[i * 4 + j] = s;
        }
    return r;
}
// Gauss-Jordan inverse with partial pivoting.
M4d m4_inverse(const M4d &a) {
    double t[4][8];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 8; j++) t[i][j] = j < 4 ? a.m[i * 4 + j] : (j - 4 == i ? 1.0 : 0.0);
    for (int c = 0; c < 4; c++) {
        int p = c;
        for (int r = c + 1; r < 4; r++)
            if (std::fabs(t[r][c]) > std::fabs(t[p][c])) p = r;
        for (int j = 0; j < 8; j++) std::swap(t[c][j], t[p][j]);
        double d = t[c][c];
        if (d == 0) return M4d{};
        for (int j = 0; j < 8; j++) t[c][j] /= d;
        for (int r = 0; r < 4; r++) {
            if (r == c) continue;
            double f = t[r][c];
            for (int j = 0; j < 8; j++) t[r][j] -= f * t[c][j];
        }
    }
    M4d r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) r.m[i * 4 + j] = t[i][j + 4];
    return r;
}

double luminance_d(double r, double g, double b) { return r * 0.212671 + g * 0.715160 + b * 0.072169; }

// make_table_dist_1d semantics, src/table_dist.cpp:3-25.
void table_1d(const std::vector<double> &f, std::vector<float> &pmf, std::vector<float> &cdf) {
    size_t n = f.size();
    std::vector<double> c(n + 1, 0.0);
    for (size_t i = 0; i < n; i++) c[i + 1] = c[i] + f[i];
    double total = c[n];
    pmf.resize(n);
    cdf.resize(n + 1);
    if (total > 0) {
        for (size_t i = 0; i < n; i++) {
            pmf[i] = (float)(f[i] / total);
            cdf[i] = (float)(c[i] / total);
        }
        cdf[n] = (float)(c[n] / total);
    } else {
        for (size_t i = 0; i < n; i++) {
            pmf[i] = (float)(1.0 / n);
            cdf[i] = (float)((double)i / n);
        }
        cdf[n] = 1.0f;
    }
}

struct HostImg {
    int w = 0, h = 0;
    std::vector<double> px;   // rgb
};
// 2x2 box pyramid, <= 8 levels: src/mipmap.h:25-48.  Where the previous
// level is one texel high (or wide) and the other side is larger, the
// reference's 2x2 box reads a row (column) past the image; here that read
// takes the edge texel instead, which changes no read that is in bounds.
std::vector<HostImg> make_mips(const lj_image_desc &im) {
    std::vector<HostImg> lv;
    HostImg l0;
    l0.w = im.width;
    l0.h = im.height;
    l0.px.resize((size_t)im.width * im.height * 3);
    for (size_t p = 0; p < (size_t)im.width * im.height; p++)
        for (int c = 0; c < 3; c++)
            l0.px[p * 3 + c] = im.channels == 3 ? im.data[p * 3 + c] : im.data[p];
    lv.push_back(l0);
    int size = std::max(im.width, im.height);
    int levels = std::min((int)std::ceil(std::log2((double)size) + 1), 8);
    for (int i = 1; i < levels; i++) {
        const HostImg &p = lv.back();
        HostImg n;
        n.w = std::max(p.w / 2, 1);
        n.h = std::max(p.h / 2, 1);
        n.px.resize((size_t)n.w * n.h * 3);
        for (int y = 0; y < n.h; y++)
            for (int x = 0; x < n.w; x++)
                for (int c = 0; c < 3; c++) {
                    auto at = [&](int xx, int yy) {
                        xx = std::min(xx, p.w - 1);
                        yy = std::min(yy, p.h - 1);
                        return p.px[((size_t)yy * p.w + xx) * 3 + c];
                    };
                    n.px[((size_t)y * n.w + x) * 3 + c] =
                        (at(2 * x, 2 * y) + at(2 * x + 1, 2 * y) + at(2 * x, 2 * y + 1) + at(2 * x + 1, 2 * y + 1)) / 4.0;
                }
        lv.push_back(n);
    }
    return lv;
}
int mod_i(int a, int b) {
    int r = a % b;
    return r < 0 ? r + b : r;
}
// bilinear lookup at level 0, src/mipmap.h:52-72
void lookup0(const HostImg &im, double u, double v, double out[3]) {
    u = u * im.w - 0.5;
    v = v * im.h - 0.5;
    int uf = mod_i((int)u, im.w), vf = mod_i((int)v, im.h);
    int uc = mod_i(uf + 1, im.w), vc = mod_i(vf + 1, im.h);
    double uo = u - uf, vo = v - vf;
    for (int c = 0; c < 3; c++) {
        auto at = [&](int x, int y) { return im.px[((size_t)y * im.w + x) * 3 + c]; };
        out[c] = at(uf, vf) * (1 - uo) * (1 - vo) + at(uf, vc) * (1 - uo) * vo + at(uc, vf) * uo * (1 - vo) +
                 at(uc, vc) * uo * vo;
    }
}

// Host -> device copy of a caller's (pageable) array.  Large arrays are
// page-locked for the copy (cudaHostRegister, read-only where the device
// allows it) and released after it: a pageable copy of tens of MB runs at
// a fraction of the link's rate.  Memory that is already page-locked, or
// that cannot be registered, is copied as it is.  One copy at a time in the
// process (scene creations may run on several threads): a range locked for
// one copy is never seen, half-released, by a copy of an overlapping range
// that a caller's two descriptions share.
std::mutex g_h2d_mutex;
int h2d(void *dst, const void *src, size_t bytes, cudaStream_t s, std::string *err) {
    std::lock_guard<std::mutex> lock(g_h2d_mutex);
    if (bytes >= ((size_t)4 << 20)) {
        void *h = const_cast<void *>(src);
        cudaError_t e = cudaHostRegister(h, bytes, cudaHostRegisterReadOnly);
        if (e != cudaSuccess) {
            cudaGetLastError();
            e = cudaHostRegister(h, bytes, cudaHostRegisterDefault);
        }
        if (e == cudaSuccess) {
            cudaError_t c = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
            cudaError_t w = cudaStreamSynchronize(s);
            cudaHostUnregister(h);
            LJ_CUDA_TRY(c);
            LJ_CUDA_TRY(w);
            return 0;
        }
        cudaGetLastError();
    }
    LJ_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
    return 0;
}

template <typename T>
int upload(lj_scene *sc, const T *src, size_t n, const T **dst, std::string *err) {
    *dst = nullptr;
    if (n == 0) return 0;
    void *p = nullptr;
    LJ_CUDA_TRY(cudaMalloc(&p, sizeof(T) * n));
    sc->allocs.push_back(p);
    if (h2d(p, src, sizeof(T) * n, sc->upload_stream, err)) return -2;
    *dst = (const T *)p;
    sc->info.device_bytes += (int64_t)(sizeof(T) * n);
    return 0;
}

// Per-channel maximum of a grid volume's values and at least zero (the
// reference's load_volume starts its maximum at zero, src/volume.cpp:72-97),
// and for three channels the one-float4-per-voxel layout.  mx: 3 uints,
// zeroed; non-negative floats order like their bit patterns.
__global__ void k_grid_prep(const float *src, size_t n, int channels, float4 *rgb, unsigned int *mx) {
    float m[3] = {0.0f, 0.0f, 0.0f};
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
        if (channels == 1) {
            m[0] = fmaxf(m[0], src[p]);
        } else {
            const float x = src[3 * p], y = src[3 * p + 1], z = src[3 * p + 2];
            m[0] = fmaxf(m[0], x);
            m[1] = fmaxf(m[1], y);
            m[2] = fmaxf(m[2], z);
            rgb[p] = make_float4(x, y, z, 0.0f);
        }
    }
    for (int c = 0; c < 3; c++) {
        float v = m[c];
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (!(v > 0.0f)) v = 0.0f;   // also turns -0 into +0
        if ((threadIdx.x & 31) == 0 && v > 0.0f) atomicMax(mx + c, __float_as_uint(v));
    }
}
template <typename T>
int upload(lj_scene *sc, const std::vector<T> &v, const T **dst, std::string *err) {
    return upload(sc, v.data(), v.size(), dst, err);
}

__global__ void k_iota(uint32_t *p, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = (uint32_t)i;
}
int fill_iota(uint32_t *p, int64_t n, cudaStream_t s) {
    k_iota<<<(int)((n + 255) / 256), 256, 0, s>>>(p, n);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int check_desc(const lj_scene_desc *d, std::string &msg) {
    if (d->camera.width <= 0 || d->camera.height <= 0) { msg = "camera width/height must be positive"; return -1; }
    if (d->num_shapes < 0 || d->num_materials < 0 || d->num_lights < 0 || d->num_media < 0 || d->num_images < 0) {
        msg = "negative element count"; return -1;
    }
    for (int i = 0; i < d->num_shapes; i++) {
        const lj_shape_desc &s = d->shapes[i];
        if (s.kind == LJ_SHAPE_MESH) {
            if (s.num_triangles < 0 || s.num_vertices < 0 || (s.num_triangles > 0 && (!s.positions || !s.indices))) {
                msg = "mesh " + std::to_string(i) + ": missing positions/indices"; return -1;
            }
            for (int t = 0; t < s.num_triangles * 3; t++)
                if (s.indices[t] < 0 || s.indices[t] >= s.num_vertices) {
                    msg = "mesh " + std::to_string(i) + ": vertex index out of range"; return -1;
                }
        } else if (s.kind == LJ_SHAPE_SPHERE) {
            if (!(s.radius > 0)) { msg = "sphere " + std::to_string(i) + ": radius must be positive"; return -1; }
        } else {
            msg = "shape " + std::to_string(i) + ": unknown kind"; return -1;
        }
        // material -1: an index-matching surface (volumetric integrator only)
        if (s.material_id < -1 || s.material_id >= d->num_materials ||
            (s.material_id == -1 && d->options.integrator != LJ_INTEGRATOR_VOLPATH)) {
            msg = "shape " + std::to_string(i) + ": material id out of range"; return -1;
        }
        if (s.area_light_id < -1 || s.area_light_id >= d->num_lights) {
            msg = "shape " + std::to_string(i) + ": light id out of range"; return -1;
        }
        if (s.interior_medium_id < -1 || s.exterior_medium_id < -1 || s.interior_medium_id >= d->num_media ||
            s.exterior_medium_id >= d->num_media) {
            msg = "shape " + std::to_string(i) + ": medium id out of range"; return -1;
        }
    }
    for (int i = 0; i < d->num_images; i++) {
        const lj_image_desc &im = d->images[i];
        if (im.width <= 0 || im.height <= 0 || !im.data || (im.channels != 1 && im.channels != 3)) {
            msg = "image " + std::to_string(i) + ": bad size, channel count or data"; return -1;
        }
    }
    for (int i = 0; i < d->num_materials; i++) {
        if (d->materials[i].type < 0 || d->materials[i].type >= LJ_MAT_COUNT) {
            msg = "material " + std::to_string(i) + ": unknown type"; return -1;
        }
        for (int k = 0; k < LJ_MAT_SLOTS; k++) {
            const lj_texture_desc &t = d->materials[i].tex[k];
            if (t.kind != LJ_TEX_CONST && t.kind != LJ_TEX_IMAGE && t.kind != LJ_TEX_CHECKER) {
                msg = "material " + std::to_string(i) + ": unknown texture kind"; return -1;
            }
            if (t.kind == LJ_TEX_IMAGE && (t.image_id < 0 || t.image_id >= d->num_images)) {
                msg = "material " + std::to_string(i) + ": texture image id out of range"; return -1;
            }
        }
    }
    for (int i = 0; i < d->num_lights; i++) {
        const lj_light_desc &l = d->lights[i];
        if (l.kind != LJ_LIGHT_AREA && l.kind != LJ_LIGHT_ENVMAP) {
            msg = "light " + std::to_string(i) + ": unknown kind"; return -1;
        }
        if (l.kind == LJ_LIGHT_AREA && (l.shape_id < 0 || l.shape_id >= d->num_shapes)) {
            msg = "light " + std::to_string(i) + ": shape id out of range"; return -1;
        }
        if (l.kind == LJ_LIGHT_ENVMAP && (l.image_id < 0 || l.image_id >= d->num_images)) {
            msg = "light " + std::to_string(i) + ": image id out of range"; return -1;
        }
    }
    if (d->envmap_light_id < -1 || d->envmap_light_id >= d->num_lights) {
        msg = "envmap light id out of range"; return -1;
    }
    if (d->camera.medium_id >= d->num_media || d->camera.medium_id < -1) { msg = "camera medium id out of range"; return -1; }
    for (int i = 0; i < d->num_media; i++) {
        const lj_medium_desc &m = d->media[i];
        if (m.kind != LJ_MEDIUM_HOMOGENEOUS && m.kind != LJ_MEDIUM_HETEROGENEOUS) { msg = "medium: unknown kind"; return -1; }
        if (m.phase_kind != LJ_PHASE_ISOTROPIC && m.phase_kind != LJ_PHASE_HG) { msg = "medium: unknown phase"; return -1; }
        const lj_volume_desc *vols[2] = {&m.albedo, &m.density};
        for (int k = 0; k < 2 && m.kind == LJ_MEDIUM_HETEROGENEOUS; k++) {
            const lj_volume_desc &v = *vols[k];
            if (v.kind != LJ_VOL_CONST && v.kind != LJ_VOL_GRID) {
                msg = "medium " + std::to_string(i) + ": unknown volume kind"; return -1;
            }
            if (v.kind == LJ_VOL_GRID && (v.res[0] <= 0 || v.res[1] <= 0 || v.res[2] <= 0 || !v.data ||
                                          (v.channels != 1 && v.channels != 3))) {
                msg = "medium " + std::to_string(i) + ": bad grid volume"; return -1;
            }
        }
    }
    return 0;
}

}  // namespace

namespace lj {
// Camera (src/camera.cpp:7-21) at resolution width x height.
void make_cam_rec(const lj_camera_desc &c, int width, int height, CamRec &cam) {
    double aspect = (double)width / (double)height;
    M4d sc_m{}, tr{}, persp{};
    sc_m.m[0] = -0.5; sc_m.m[5] = -0.5 * aspect; sc_m.m[10] = 1.0; sc_m.m[15] = 1;
    tr.m[0] = 1; tr.m[5] = 1; tr.m[10] = 1; tr.m[15] = 1; tr.m[3] = -1.0; tr.m[7] = -1.0 / aspect;
    double cot = 1.0 / std::tan((M_PI / 180.0) * (c.fov / 2.0));
    persp.m[0] = cot; persp.m[5] = cot; persp.m[10] = 1; persp.m[11] = -1; persp.m[14] = 1;
    M4d s2c = m4_inverse(m4_mul(m4_mul(sc_m, tr), persp));
    for (int k = 0; k < 16; k++) {
        cam.sample_to_cam[k] = (float)s2c.m[k];
        cam.cam_to_world[k] = (float)c.cam_to_world[k];
    }
    // xform_point(cam_to_world, 0) with the homogeneous divide
    double w = c.cam_to_world[15];
    for (int k = 0; k < 3; k++) cam.org[k] = (float)(c.cam_to_world[k * 4 + 3] / w);
    cam.w = width;
    cam.h = height;
    cam.filter_kind = c.filter_kind;
    cam.filter_param = c.filter_param;
}
}  // namespace lj

extern "C" {

int lj_gpu_abi_version(void) { return LJ_GPU_ABI_VERSION; }

int lj_gpu_init(int device, lj_ctx **out) {
    if (!out) return LJ_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return LJ_ERR_NO_DEVICE;
    if (device < 0 || device >= n) return LJ_ERR_INVALID_ARG;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return LJ_ERR_CUDA;
    if (prop.major * 10 + prop.minor < 100) return LJ_ERR_NO_DEVICE;   // built for sm_103a
    if (cudaSetDevice(device) != cudaSuccess) return LJ_ERR_CUDA;
    lj_ctx *ctx = new (std::nothrow) lj_ctx();
    if (!ctx) return LJ_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&ctx->d_status, sizeof(int)) != cudaSuccess ||
        cudaMemset(ctx->d_status, 0, sizeof(int)) != cudaSuccess) {
        delete ctx;
        return LJ_ERR_CUDA;
    }
    *out = ctx;
    return LJ_OK;
}

void lj_gpu_shutdown(lj_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    while (!ctx->servers.empty()) lj_gpu_server_stop(ctx->servers.back());
    while (!ctx->scenes.empty()) lj_gpu_scene_destroy(ctx->scenes.back());
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->d_status) cudaFree(ctx->d_status);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char *lj_gpu_last_error(lj_ctx *ctx) { return ctx ? ctx->last_error.c_str() : ""; }

int lj_gpu_scene_validate(const lj_scene_desc *d, char *msg, int msg_size) {
    std::string m;
    int rc = LJ_OK;
    if (!d) {
        m = "null scene description";
        rc = LJ_ERR_INVALID_ARG;
    } else if (check_desc(d, m)) {
        rc = LJ_ERR_INVALID_ARG;
    }
    if (msg && msg_size > 0) {
        size_t n = std::min(m.size(), (size_t)msg_size - 1);
        memcpy(msg, m.data(), n);
        msg[n] = 0;
    }
    return rc;
}

namespace {

// Frees a scene that never joined its context's list (its creation failed,
// or another scene of the same lj_gpu_scene_create_many call did).
void discard_scene(lj_scene *sc) {
    cudaStreamSynchronize(sc->upload_stream);
    for (void *p : sc->allocs) cudaFree(p);
    delete sc;
}

// A scene under construction: discarded on every way out but success
// (an error code or an exception).
struct SceneGuard {
    lj_scene *sc = nullptr;
    bool keep = false;
    ~SceneGuard() {
        if (sc && !keep) discard_scene(sc);
    }
};

// One scene from a checked description, every copy and kernel on `stream`,
// the host-side tables built on the calling thread.  Touches nothing of the
// context but its device and stream-independent settings, so that several
// run at once; on failure the scene's allocations are freed and msg says why.
int create_scene_body(lj_ctx *ctx, const lj_scene_desc *d, cudaStream_t stream, lj_scene **out, std::string &msg,
                      SceneGuard &guard) {
    cudaSetDevice(ctx->device);
    lj_scene *sc = new lj_scene();
    guard.sc = sc;
    sc->ctx = ctx;
    sc->upload_stream = stream;
    sc->options = d->options;
    sc->width = d->camera.width;
    sc->height = d->camera.height;
    std::string err;
    auto fail = [&](int code) {   // the guard frees the scene
        msg = err.empty() ? "scene upload failed" : err;
        return code;
    };
    DevScene &ds = sc->dev;

    // ---- geometry: global vertex arrays, triangles, spheres ----
    std::vector<float> vpos, vnrm, vuv, spheres;
    std::vector<int> tri_vidx, prim_shape;
    std::vector<ShapeRec> shapes(d->num_shapes);
    std::vector<float> tri_cdf;
    int num_tris = 0, num_spheres = 0;
    for (int i = 0; i < d->num_shapes; i++)
        if (d->shapes[i].kind == LJ_SHAPE_MESH) num_tris += d->shapes[i].num_triangles;
        else num_spheres++;
    sc->num_spheres = num_spheres;
    sc->shape_prim_base.assign(d->num_shapes, 0);
    sc->shape_vbase.assign(d->num_shapes, -1);
    sc->shape_nverts.assign(d->num_shapes, 0);
    sc->emitter_indices.assign(d->num_shapes, {});
    int tri_base = 0, sphere_ord = 0;
    prim_shape.assign((size_t)num_tris + num_spheres, 0);
    tri_vidx.resize((size_t)num_tris * 3);
    // shapes an area light emits from: they need their triangle areas
    std::vector<char> emits(d->num_shapes, 0);
    for (int l = 0; l < d->num_lights; l++)
        if (d->lights[l].kind == LJ_LIGHT_AREA) emits[d->lights[l].shape_id] = 1;
    for (int i = 0; i < d->num_shapes; i++) {
        const lj_shape_desc &s = d->shapes[i];
        ShapeRec &r = shapes[i];
        memset(&r, 0, sizeof(r));
        r.kind = s.kind;
        r.material_id = s.material_id;
        r.area_light_id = s.area_light_id;
        r.interior_medium_id = s.interior_medium_id;
        r.exterior_medium_id = s.exterior_medium_id;
        if (s.kind == LJ_SHAPE_MESH) {
            int vbase = (int)(vpos.size() / 3);
            sc->shape_vbase[i] = vbase;
            sc->shape_nverts[i] = s.num_vertices;
            if (emits[i] || s.area_light_id >= 0)
                sc->emitter_indices[i].assign(s.indices, s.indices + (size_t)s.num_triangles * 3);
            vpos.insert(vpos.end(), s.positions, s.positions + (size_t)s.num_vertices * 3);
            if (s.normals) vnrm.insert(vnrm.end(), s.normals, s.normals + (size_t)s.num_vertices * 3);
            else vnrm.insert(vnrm.end(), (size_t)s.num_vertices * 3, 0.0f);
            if (s.uvs) vuv.insert(vuv.end(), s.uvs, s.uvs + (size_t)s.num_vertices * 2);
            else vuv.insert(vuv.end(), (size_t)s.num_vertices * 2, 0.0f);
            r.has_normals = s.normals != nullptr;
            r.has_uvs = s.uvs != nullptr;
            r.tri_begin = tri_base;
            r.num_tris = s.num_triangles;
            int *tv = tri_vidx.data() + (size_t)tri_base * 3;
            for (int t = 0; t < 3 * s.num_triangles; t++) tv[t] = vbase + s.indices[t];
            std::fill(prim_shape.begin() + tri_base, prim_shape.begin() + tri_base + s.num_triangles, i);
            // triangle areas: only an emissive mesh samples by area and needs
            // its total (its light pdf)
            std::vector<double> areas(s.area_light_id >= 0 || emits[i] ? s.num_triangles : 0);
            double total = 0;
            for (int t = 0; t < (int)areas.size(); t++) {
                int a = s.indices[t * 3], b = s.indices[t * 3 + 1], c = s.indices[t * 3 + 2];
                const float *p0 = s.positions + a * 3, *p1 = s.positions + b * 3, *p2 = s.positions + c * 3;
                double e1[3] = {(double)p1[0] - p0[0], (double)p1[1] - p0[1], (double)p1[2] - p0[2]};
                double e2[3] = {(double)p2[0] - p0[0], (double)p2[1] - p0[1], (double)p2[2] - p0[2]};
                double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                       cz = e1[0] * e2[1] - e1[1] * e2[0];
                areas[t] = std::sqrt(cx * cx + cy * cy + cz * cz) / 2;
                total += areas[t];
            }
            r.total_area = (float)total;
            if (s.area_light_id >= 0) {
                std::vector<float> pmf, cdf;
                table_1d(areas, pmf, cdf);
                r.sampler_offset = (int)tri_cdf.size();
                tri_cdf.insert(tri_cdf.end(), cdf.begin(), cdf.end());
            } else {
                r.sampler_offset = -1;
            }
            sc->shape_prim_base[i] = tri_base;
            tri_base += s.num_triangles;
        } else {
            r.cx = s.center[0]; r.cy = s.center[1]; r.cz = s.center[2]; r.radius = s.radius;
            r.total_area = (float)(4 * M_PI * (double)s.radius * s.radius);
            int g = num_tris + sphere_ord++;
            prim_shape[g] = i;
            sc->shape_prim_base[i] = g;
            spheres.insert(spheres.end(), {s.center[0], s.center[1], s.center[2], s.radius});
        }
    }
    sc->prim_shape_host = prim_shape;
    if (upload(sc, vpos, &ds.vpos, &err) || upload(sc, vnrm, &ds.vnrm, &err) || upload(sc, vuv, &ds.vuv, &err) ||
        upload(sc, tri_vidx, &ds.tri_vidx, &err) || upload(sc, prim_shape, &ds.prim_shape, &err) ||
        upload(sc, shapes, &ds.shapes, &err) || upload(sc, tri_cdf, &ds.tri_cdf, &err))
        return fail(LJ_ERR_CUDA);
    const float *d_spheres = nullptr;
    if (upload(sc, spheres, &d_spheres, &err)) return fail(LJ_ERR_CUDA);
    sc->d_spheres = d_spheres;
    sc->shapes_host = shapes;
    ds.num_tris = num_tris;
    ds.num_prims = num_tris + num_spheres;
    ds.num_shapes = d->num_shapes;

    // ---- BVH ----
    BvhInput bin{ds.vpos, ds.tri_vidx, d_spheres, num_tris, num_spheres};
    BvhOutput bout;
    int rc = build_bvh(bin, &bout, stream, &err);
    if (bout.nodes) sc->allocs.push_back(bout.nodes);
    if (bout.prims) sc->allocs.push_back(bout.prims);
    if (rc) return fail(rc == -5 ? LJ_ERR_DEVICE_LIMIT : LJ_ERR_CUDA);
    ds.bvh.nodes = bout.nodes;
    ds.bvh.prims = bout.prims;
    ds.bvh.num_nodes = bout.num_nodes;
    ds.bvh.num_leaf_prims = ds.num_prims;
    sc->bvh_levels = bout.level_start;
    sc->info.num_wide_nodes = bout.num_nodes;
    sc->info.num_binary_nodes = bout.num_binary;
    sc->info.build_ms = bout.build_ms;
    sc->info.device_bytes += (int64_t)bout.num_nodes * 80 + (int64_t)ds.num_prims * 48;
    for (int k = 0; k < 3; k++) {
        sc->info.bounds_lower[k] = ds.num_prims ? bout.lo[k] : 0.f;
        sc->info.bounds_upper[k] = ds.num_prims ? bout.hi[k] : 0.f;
    }
    // bounding sphere, src/scene.cpp:29-34; epsilon, src/scene.h:99-105
    {
        double lb[3], ub[3], dd = 0;
        for (int k = 0; k < 3; k++) {
            lb[k] = sc->info.bounds_lower[k];
            ub[k] = sc->info.bounds_upper[k];
            dd += (ub[k] - lb[k]) * (ub[k] - lb[k]);
        }
        sc->info.bsphere_radius = std::sqrt(dd) / 2;
        for (int k = 0; k < 3; k++) sc->info.bsphere_center[k] = (lb[k] + ub[k]) / 2;
        ds.bradius = (float)sc->info.bsphere_radius;
        for (int k = 0; k < 3; k++) ds.bcenter[k] = (float)sc->info.bsphere_center[k];
        ds.eps = (float)std::min(sc->info.bsphere_radius * 1e-5, 0.01);
    }
    sc->info.num_triangles = num_tris;
    sc->info.num_prims = ds.num_prims;

    // ---- materials ----
    std::vector<MatRec> mats(d->num_materials);
    for (int i = 0; i < d->num_materials; i++) sc->mat_mask |= 1u << d->materials[i].type;
    for (int i = 0; i < d->num_materials; i++) {
        const lj_material_desc &m = d->materials[i];
        MatRec &r = mats[i];
        memset(&r, 0, sizeof(r));
        r.type = m.type;
        r.eta = m.eta;
        for (int k = 0; k < LJ_MAT_SLOTS; k++) {
            const lj_texture_desc &t = m.tex[k];
            TexRec &x = r.tex[k];
            x.kind = t.kind;
            x.image_id = t.image_id;
            for (int c = 0; c < 3; c++) { x.v0[c] = t.value0[c]; x.v1[c] = t.value1[c]; }
            x.us = t.uscale; x.vs = t.vscale; x.uo = t.uoffset; x.vo = t.voffset;
            if (t.kind != LJ_TEX_CONST) r.textured |= 1 << k;
        }
    }
    if (upload(sc, mats, &ds.mats, &err)) return fail(LJ_ERR_CUDA);
    ds.num_mats = d->num_materials;

    // ---- images (mip pyramids) ----
    std::vector<std::vector<HostImg>> mips(d->num_images);
    std::vector<MipLevel> levels((size_t)std::max(1, d->num_images) * 8);
    std::vector<int> nlev(std::max(1, d->num_images), 0);
    for (int i = 0; i < d->num_images; i++) {
        mips[i] = make_mips(d->images[i]);
        nlev[i] = (int)mips[i].size();
        for (size_t l = 0; l < mips[i].size(); l++) {
            std::vector<float> f(mips[i][l].px.begin(), mips[i][l].px.end());
            const float *p = nullptr;
            if (upload(sc, f, &p, &err)) return fail(LJ_ERR_CUDA);
            levels[i * 8 + l] = MipLevel{p, mips[i][l].w, mips[i][l].h};
        }
    }
    if (d->num_images > 0) {
        if (upload(sc, levels, &ds.image_levels, &err) || upload(sc, nlev, &ds.image_num_levels, &err))
            return fail(LJ_ERR_CUDA);
    }

    // ---- lights + power table (src/scene.cpp:47-52) ----
    std::vector<LightRec> lights(d->num_lights);
    std::vector<double> power(d->num_lights);
    sc->light_factor.assign(d->num_lights, 0.0);
    ds.env.light_id = -1;
    for (int i = 0; i < d->num_lights; i++) {
        const lj_light_desc &l = d->lights[i];
        LightRec &r = lights[i];
        memset(&r, 0, sizeof(r));
        r.kind = l.kind;
        r.shape_id = l.shape_id;
        for (int c = 0; c < 3; c++) r.intensity[c] = l.intensity[c];
        r.scale = l.scale;
        r.image_id = l.image_id;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                r.to_world[a * 3 + b] = (float)l.to_world[a * 4 + b];
                r.to_local[a * 3 + b] = (float)l.to_local[a * 4 + b];
            }
        if (l.kind == LJ_LIGHT_AREA) {
            double area = shapes[l.shape_id].total_area;
            if (d->shapes[l.shape_id].kind == LJ_SHAPE_SPHERE)
                area = 4 * M_PI * (double)d->shapes[l.shape_id].radius * d->shapes[l.shape_id].radius;
            sc->light_factor[i] = luminance_d(l.intensity[0], l.intensity[1], l.intensity[2]) * M_PI;
            power[i] = sc->light_factor[i] * area;
        } else {
            // envmap sampling table from luminance * sin(elevation) at level 0
            const HostImg &im = mips[l.image_id][0];
            int w = im.w, h = im.h;
            std::vector<double> cdf_rows((size_t)h * (w + 1)), pdf_rows((size_t)h * w), f((size_t)w * h);
            for (int y = 0; y < h; y++) {
                double v = (y + 0.5) / h, se = std::sin(M_PI * v);
                for (int x = 0; x < w; x++) {
                    double rgb[3];
                    lookup0(im, (x + 0.5) / w, v, rgb);
                    f[(size_t)y * w + x] = luminance_d(rgb[0], rgb[1], rgb[2]) * se;
                }
            }
            // make_table_dist_2d, src/table_dist.cpp:40-114
            std::vector<double> row_int(h);
            for (int y = 0; y < h; y++) {
                double *cr = &cdf_rows[(size_t)y * (w + 1)];
                cr[0] = 0;
                for (int x = 0; x < w; x++) cr[x + 1] = cr[x] + f[(size_t)y * w + x];
                double integral = cr[w];
                row_int[y] = integral;
                if (integral > 0) {
                    for (int x = 0; x < w; x++) cr[x] /= integral;
                    for (int x = 0; x < w; x++) pdf_rows[(size_t)y * w + x] = f[(size_t)y * w + x] / integral;
                } else {
                    for (int x = 0; x < w; x++) { pdf_rows[(size_t)y * w + x] = 1.0 / w; cr[x] = (double)x / w; }
                    cr[w] = 1;
                    row_int[y] = 1;
                }
            }
            std::vector<double> cdf_m(h + 1, 0.0), pdf_m(h);
            for (int y = 0; y < h; y++) cdf_m[y + 1] = cdf_m[y] + row_int[y];
            double total = cdf_m[h];
            if (total > 0) {
                for (int y = 0; y < h; y++) cdf_m[y] /= total;
                cdf_m[h] = 1;
                for (int y = 0; y < h; y++) pdf_m[y] = row_int[y] / total;
            } else {
                for (int y = 0; y < h; y++) { pdf_m[y] = 1.0 / h; cdf_m[y] = (double)y / h; }
                cdf_m[h] = 1;
            }
            for (int y = 0; y < h; y++) cdf_rows[(size_t)y * (w + 1) + w] = 1;
            auto tof = [](const std::vector<double> &v) { return std::vector<float>(v.begin(), v.end()); };
            if (upload(sc, tof(cdf_rows), &ds.env.cdf_rows, &err) || upload(sc, tof(pdf_rows), &ds.env.pdf_rows, &err) ||
                upload(sc, tof(cdf_m), &ds.env.cdf_marg, &err) || upload(sc, tof(pdf_m), &ds.env.pdf_marg, &err))
                return fail(LJ_ERR_CUDA);
            ds.env.tw = w;
            ds.env.th = h;
            ds.env.light_id = i;
            ds.env.num_levels = (int)mips[l.image_id].size();
            for (int k = 0; k < ds.env.num_levels; k++) ds.env.levels[k] = levels[l.image_id * 8 + k];
            sc->light_factor[i] = M_PI * total / ((double)w * h);
            power[i] = sc->light_factor[i] * sc->info.bsphere_radius * sc->info.bsphere_radius;
        }
    }
    if (d->envmap_light_id >= 0 && ds.env.light_id != d->envmap_light_id)
        ds.env.light_id = d->envmap_light_id;
    std::vector<float> lpmf, lcdf;
    table_1d(power, lpmf, lcdf);
    if (upload(sc, lights, &ds.lights, &err) || upload(sc, lpmf, &ds.light_pmf, &err) ||
        upload(sc, lcdf, &ds.light_cdf, &err))
        return fail(LJ_ERR_CUDA);
    ds.num_lights = d->num_lights;

    sc->camera = d->camera;
    make_cam_rec(d->camera, d->camera.width, d->camera.height, ds.cam);
    ds.max_depth = d->options.max_depth;
    ds.rr_depth = d->options.rr_depth;
    sc->has_media = d->num_media > 0;

    // ---- media (src/medium.h, src/volume.h; .vol data as load_volume gives it) ----
    {
        std::vector<MediumRec> media(d->num_media);
        for (int i = 0; i < d->num_media; i++) {
            const lj_medium_desc &m = d->media[i];
            MediumRec &r = media[i];
            memset(&r, 0, sizeof(r));
            r.kind = m.kind;
            r.phase_kind = m.phase_kind;
            r.g = m.g;
            for (int c = 0; c < 3; c++) { r.sigma_a[c] = m.sigma_a[c]; r.sigma_s[c] = m.sigma_s[c]; }
            const lj_volume_desc *src[2] = {&m.albedo, &m.density};
            VolRec *dst[2] = {&r.albedo, &r.density};
            for (int k = 0; k < 2 && m.kind == LJ_MEDIUM_HETEROGENEOUS; k++) {
                const lj_volume_desc &v = *src[k];
                VolRec &o = *dst[k];
                o.kind = v.kind;
                o.scale = v.scale;
                if (v.kind == LJ_VOL_CONST) {
                    for (int c = 0; c < 3; c++) o.value[c] = o.max_value[c] = v.value[c];
                    continue;
                }
                size_t n = (size_t)v.res[0] * v.res[1] * v.res[2];
                if (n == 0 || !v.data || (v.channels != 1 && v.channels != 3)) {
                    err = "medium " + std::to_string(i) + ": bad grid volume";
                    return fail(LJ_ERR_INVALID_ARG);
                }
                const bool cs_set = v.channel_scale[0] != 0.0f || v.channel_scale[1] != 0.0f ||
                                    v.channel_scale[2] != 0.0f;
                float mx[3] = {0, 0, 0};
                o.channels = v.channels;
                // the caller's values to the device as they are; maxima (and
                // the float4 layout of three channels) computed there
                unsigned int *d_mx = nullptr, h_mx[3] = {0, 0, 0};
                const float *raw = nullptr;
                float4 *rgb = nullptr;
                const int gblocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
                bool ok = cudaMalloc(&d_mx, sizeof(h_mx)) == cudaSuccess &&
                          cudaMemsetAsync(d_mx, 0, sizeof(h_mx), stream) == cudaSuccess;
                if (ok && v.channels == 1) {   // one float per voxel, uploaded from the caller's array
                    ok = upload(sc, v.data, n, &o.data1, &err) == 0;
                    raw = o.data1;
                } else if (ok) {
                    void *tmp = nullptr;
                    ok = cudaMalloc(&tmp, sizeof(float) * 3 * n) == cudaSuccess &&
                         h2d(tmp, v.data, sizeof(float) * 3 * n, stream, &err) == 0 &&
                         cudaMalloc((void **)&rgb, sizeof(float4) * n) == cudaSuccess;
                    if (rgb) {
                        sc->allocs.push_back(rgb);
                        sc->info.device_bytes += (int64_t)(sizeof(float4) * n);
                        o.data = rgb;
                    }
                    raw = (const float *)tmp;
                }
                if (ok) {
                    k_grid_prep<<<gblocks, 256, 0, stream>>>(raw, n, v.channels, rgb, d_mx);
                    ok = cudaGetLastError() == cudaSuccess &&
                         cudaMemcpyAsync(h_mx, d_mx, sizeof(h_mx), cudaMemcpyDeviceToHost, stream) ==
                             cudaSuccess &&
                         cudaStreamSynchronize(stream) == cudaSuccess;
                }
                if (v.channels == 3 && raw) cudaFree(const_cast<float *>(raw));
                if (d_mx) cudaFree(d_mx);
                if (!ok) {
                    cudaGetLastError();
                    if (err.empty()) err = "medium " + std::to_string(i) + ": grid upload failed";
                    return fail(LJ_ERR_CUDA);
                }
                for (int c = 0; c < 3; c++) {
                    float f;
                    memcpy(&f, &h_mx[v.channels == 1 ? 0 : c], sizeof(f));
                    mx[c] = f;
                }
                for (int c = 0; c < 3; c++) {
                    o.res[c] = v.res[c];
                    o.pmin[c] = v.p_min[c];
                    o.pmax[c] = v.p_max[c];
                    o.cscale[c] = cs_set ? v.channel_scale[c] : 1.0f;
                    o.max_value[c] = v.scale * mx[c] * o.cscale[c];
                    o.gscale[c] = (float)((double)(v.res[c] - 1) / ((double)v.p_max[c] - (double)v.p_min[c]));
                }
            }
        }
        if (upload(sc, media, &ds.media, &err)) return fail(LJ_ERR_CUDA);
        ds.num_media = d->num_media;
        ds.camera_medium = d->camera.medium_id;
        ds.max_null_collisions = d->options.max_null_collisions;
    }
    if (cudaStreamSynchronize(stream) != cudaSuccess) {
        err = "scene upload: stream synchronize failed";
        return fail(LJ_ERR_CUDA);
    }
    sc->upload_stream = ctx->stream;   // later copies (none yet) go to the context's stream
    guard.keep = true;
    *out = sc;
    return LJ_OK;
}

// create_scene_body with no exception leaving it (a host allocation that
// fails becomes LJ_ERR_OUT_OF_MEMORY): it runs on threads of its own and
// under the C ABI.
int create_scene(lj_ctx *ctx, const lj_scene_desc *d, cudaStream_t stream, lj_scene **out, std::string &msg) {
    *out = nullptr;
    try {
        SceneGuard guard;
        return create_scene_body(ctx, d, stream, out, msg, guard);
    } catch (const std::bad_alloc &) {
        msg = "host allocation failed";
        return LJ_ERR_OUT_OF_MEMORY;
    } catch (...) {
        msg = "scene creation failed";
        return LJ_ERR_CUDA;
    }
}

constexpr int kCreateThreads = 8;   // host threads of one lj_gpu_scene_create_many call at most

}  // namespace

int lj_gpu_scene_create(lj_ctx *ctx, const lj_scene_desc *d, lj_scene **out) {
    if (!ctx || !d || !out) return LJ_ERR_INVALID_ARG;
    *out = nullptr;
    std::string msg;
    if (check_desc(d, msg)) return set_error(ctx, LJ_ERR_INVALID_ARG, msg);
    lj_scene *sc = nullptr;
    const int rc = create_scene(ctx, d, ctx->stream, &sc, msg);
    if (rc != LJ_OK) return set_error(ctx, rc, msg);
    ctx->scenes.push_back(sc);
    *out = sc;
    return LJ_OK;
}

int lj_gpu_scene_create_many(lj_ctx *ctx, int32_t n, const lj_scene_desc *const *descs, lj_scene **out) {
    if (!ctx || n < 0 || (n > 0 && (!descs || !out))) return LJ_ERR_INVALID_ARG;
    for (int i = 0; i < n; i++) out[i] = nullptr;
    for (int i = 0; i < n; i++) {
        std::string msg = "NULL description";
        if (!descs[i] || check_desc(descs[i], msg))
            return set_error(ctx, LJ_ERR_INVALID_ARG, "scene_create_many: description " + std::to_string(i) + ": " + msg);
    }
    if (n == 0) return LJ_OK;
    cudaSetDevice(ctx->device);
    std::vector<cudaStream_t> streams(n, nullptr);
    for (int i = 0; i < n; i++) {
        if (cudaStreamCreateWithFlags(&streams[i], cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            for (int k = 0; k < i; k++) cudaStreamDestroy(streams[k]);
            return set_error(ctx, LJ_ERR_CUDA, "scene_create_many: stream creation failed");
        }
    }
    std::vector<lj_scene *> made(n, nullptr);
    std::vector<int> rc(n, LJ_OK);
    std::vector<std::string> msg(n);
    std::atomic<int> next{0};
    auto work = [&]() {
        for (int i = next++; i < n; i = next++) rc[i] = create_scene(ctx, descs[i], streams[i], &made[i], msg[i]);
    };
    std::vector<std::thread> helpers;
    for (int t = 1; t < std::min(n, kCreateThreads); t++) {
        try {
            helpers.emplace_back(work);
        } catch (...) {   // no more threads: the ones started (and this one) take the rest
            break;
        }
    }
    work();
    for (std::thread &t : helpers) t.join();
    for (cudaStream_t s : streams) cudaStreamDestroy(s);   // each creation synchronized its stream
    for (int i = 0; i < n; i++) {
        if (rc[i] == LJ_OK) continue;
        for (lj_scene *sc : made)
            if (sc) discard_scene(sc);
        return set_error(ctx, rc[i], "scene_create_many: description " + std::to_string(i) + ": " + msg[i]);
    }
    for (int i = 0; i < n; i++) {
        ctx->scenes.push_back(made[i]);
        out[i] = made[i];
    }
    return LJ_OK;
}

int lj_gpu_scene_update_mesh(lj_scene *sc, int32_t shape_id, const float *positions, const float *normals,
                             int32_t num_vertices, int32_t mode) {
    if (!sc) return LJ_ERR_INVALID_ARG;
    lj_ctx *ctx = sc->ctx;
    if (shape_id < 0 || shape_id >= (int)sc->shapes_host.size() || sc->shapes_host[shape_id].kind != LJ_SHAPE_MESH)
        return set_error(ctx, LJ_ERR_INVALID_ARG, "scene_update_mesh: shape_id is not a mesh of the scene");
    if (!positions || num_vertices != sc->shape_nverts[shape_id])
        return set_error(ctx, LJ_ERR_INVALID_ARG, "scene_update_mesh: positions must hold the mesh's " +
                                                      std::to_string(sc->shape_nverts[shape_id]) + " vertices");
    if (mode != LJ_UPDATE_REFIT && mode != LJ_UPDATE_REBUILD)
        return set_error(ctx, LJ_ERR_INVALID_ARG, "scene_update_mesh: unknown mode");
    if (normals && !sc->shapes_host[shape_id].has_normals)
        return set_error(ctx, LJ_ERR_INVALID_ARG, "scene_update_mesh: the mesh was created without normals");
    if (sc->server_refs.load() > 0)
        return set_error(ctx, LJ_ERR_INVALID_ARG, "scene_update_mesh: the scene is registered with a running server");
    const size_t nv = (size_t)num_vertices;
    for (size_t k = 0; k < nv * 3; k++)
        if (!std::isfinite(positions[k]))
            return set_error(ctx, LJ_ERR_INVALID_ARG, "scene_update_mesh: a position is not finite");
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    std::string err;
    // work queued on any stream may still read the scene
    if (cudaDeviceSynchronize() != cudaSuccess) return set_error(ctx, LJ_ERR_CUDA, "scene_update_mesh: device error");
    DevScene &ds = sc->dev;
    const size_t vbase = (size_t)sc->shape_vbase[shape_id];
    if (cudaMemcpyAsync(const_cast<float *>(ds.vpos) + vbase * 3, positions, sizeof(float) * nv * 3,
                        cudaMemcpyHostToDevice, s) != cudaSuccess ||
        (normals && cudaMemcpyAsync(const_cast<float *>(ds.vnrm) + vbase * 3, normals, sizeof(float) * nv * 3,
                                    cudaMemcpyHostToDevice, s) != cudaSuccess))
        return set_error(ctx, LJ_ERR_CUDA, "scene_update_mesh: upload failed");

    // ---- BVH: refit in place, or rebuild ----
    BvhInput bin{ds.vpos, ds.tri_vidx, sc->d_spheres, ds.num_tris, sc->num_spheres};
    float lo[3], hi[3];
    if (mode == LJ_UPDATE_REFIT) {
        if (refit_bvh(bin, const_cast<uint4 *>(ds.bvh.nodes), const_cast<float4 *>(ds.bvh.prims), ds.num_prims,
                      sc->bvh_levels, lo, hi, s, &err))
            return set_error(ctx, LJ_ERR_CUDA, "scene_update_mesh: " + err);
    } else {
        BvhOutput bout;
        int rc = build_bvh(bin, &bout, s, &err);
        if (rc) {
            if (bout.nodes) cudaFree(bout.nodes);
            if (bout.prims) cudaFree(bout.prims);
            return set_error(ctx, rc == -5 ? LJ_ERR_DEVICE_LIMIT : LJ_ERR_CUDA, "scene_update_mesh: " + err);
        }
        for (void *&a : sc->allocs) {
            if (a == (void *)ds.bvh.nodes) {
                cudaFree(a);
                a = bout.nodes;
            } else if (a == (void *)ds.bvh.prims) {
                cudaFree(a);
                a = bout.prims;
            }
        }
        sc->info.device_bytes += ((int64_t)bout.num_nodes - ds.bvh.num_nodes) * 80;
        ds.bvh.nodes = bout.nodes;
        ds.bvh.prims = bout.prims;
        ds.bvh.num_nodes = bout.num_nodes;
        sc->bvh_levels = bout.level_start;
        sc->info.num_wide_nodes = bout.num_nodes;
        sc->info.num_binary_nodes = bout.num_binary;
        sc->info.build_ms = bout.build_ms;
        for (int k = 0; k < 3; k++) {
            lo[k] = bout.lo[k];
            hi[k] = bout.hi[k];
        }
    }
    // ---- bounds, bounding sphere and shadow epsilon (src/scene.cpp:29-34,
    // src/scene.h:99-105) follow the new geometry ----
    {
        double dd = 0;
        for (int k = 0; k < 3; k++) {
            sc->info.bounds_lower[k] = lo[k];
            sc->info.bounds_upper[k] = hi[k];
            dd += ((double)hi[k] - lo[k]) * ((double)hi[k] - lo[k]);
        }
        sc->info.bsphere_radius = std::sqrt(dd) / 2;
        for (int k = 0; k < 3; k++) sc->info.bsphere_center[k] = ((double)lo[k] + hi[k]) / 2;
        ds.bradius = (float)sc->info.bsphere_radius;
        for (int k = 0; k < 3; k++) ds.bcenter[k] = (float)sc->info.bsphere_center[k];
        ds.eps = (float)std::min(sc->info.bsphere_radius * 1e-5, 0.01);
    }
    // ---- an emitting mesh's triangle areas and sampling table ----
    ShapeRec &r = sc->shapes_host[shape_id];
    const std::vector<int32_t> &idx = sc->emitter_indices[shape_id];
    if (!idx.empty()) {
        const int nt = (int)(idx.size() / 3);
        std::vector<double> areas(nt);
        double total = 0;
        for (int t = 0; t < nt; t++) {
            const float *p0 = positions + idx[t * 3] * 3, *p1 = positions + idx[t * 3 + 1] * 3,
                        *p2 = positions + idx[t * 3 + 2] * 3;
            double e1[3] = {(double)p1[0] - p0[0], (double)p1[1] - p0[1], (double)p1[2] - p0[2]};
            double e2[3] = {(double)p2[0] - p0[0], (double)p2[1] - p0[1], (double)p2[2] - p0[2]};
            double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                   cz = e1[0] * e2[1] - e1[1] * e2[0];
            areas[t] = std::sqrt(cx * cx + cy * cy + cz * cz) / 2;
            total += areas[t];
        }
        r.total_area = (float)total;
        if (cudaMemcpyAsync(const_cast<ShapeRec *>(ds.shapes) + shape_id, &r, sizeof(ShapeRec),
                            cudaMemcpyHostToDevice, s) != cudaSuccess)
            return set_error(ctx, LJ_ERR_CUDA, "scene_update_mesh: upload failed");
        if (r.sampler_offset >= 0) {
            std::vector<float> pmf, cdf;
            table_1d(areas, pmf, cdf);
            if (cudaMemcpyAsync(const_cast<float *>(ds.tri_cdf) + r.sampler_offset, cdf.data(),
                                sizeof(float) * cdf.size(), cudaMemcpyHostToDevice, s) != cudaSuccess)
                return set_error(ctx, LJ_ERR_CUDA, "scene_update_mesh: upload failed");
        }
    }
    // ---- light-selection table (src/scene.cpp:47-52): area lights by their
    // shapes' areas, the envmap by the bounding radius ----
    if (ds.num_lights > 0) {
        std::vector<double> power(ds.num_lights);
        std::vector<LightRec> lr(ds.num_lights);
        if (cudaMemcpyAsync(lr.data(), ds.lights, sizeof(LightRec) * lr.size(), cudaMemcpyDeviceToHost, s) !=
                cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return set_error(ctx, LJ_ERR_CUDA, "scene_update_mesh: light table read failed");
        for (int i = 0; i < ds.num_lights; i++) {
            if (lr[i].kind == LJ_LIGHT_AREA) {
                const ShapeRec &sh = sc->shapes_host[lr[i].shape_id];
                double area = sh.kind == LJ_SHAPE_SPHERE ? 4 * M_PI * (double)sh.radius * sh.radius : sh.total_area;
                power[i] = sc->light_factor[i] * area;
            } else {
                power[i] = sc->light_factor[i] * sc->info.bsphere_radius * sc->info.bsphere_radius;
            }
        }
        std::vector<float> lpmf, lcdf;
        table_1d(power, lpmf, lcdf);
        if (cudaMemcpyAsync(const_cast<float *>(ds.light_pmf), lpmf.data(), sizeof(float) * lpmf.size(),
                            cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(const_cast<float *>(ds.light_cdf), lcdf.data(), sizeof(float) * lcdf.size(),
                            cudaMemcpyHostToDevice, s) != cudaSuccess)
            return set_error(ctx, LJ_ERR_CUDA, "scene_update_mesh: upload failed");
    }
    if (cudaStreamSynchronize(s) != cudaSuccess)
        return set_error(ctx, LJ_ERR_CUDA, "scene_update_mesh: stream synchronize failed");
    return LJ_OK;
}

void lj_gpu_scene_destroy(lj_scene *sc) {
    if (!sc) return;
    if (sc->server_refs.load() > 0) {
        set_error(sc->ctx, LJ_ERR_INVALID_ARG, "scene_destroy: the scene is registered with a running server");
        return;
    }
    auto &live = sc->ctx->scenes;
    live.erase(std::remove(live.begin(), live.end(), sc), live.end());
    cudaSetDevice(sc->ctx->device);
    cudaDeviceSynchronize();   // kernels on any stream may still read the scene
    for (void *p : sc->allocs) cudaFree(p);
    if (sc->path.block) cudaFree(sc->path.block);
    delete sc;
}

int lj_gpu_scene_info(lj_scene *sc, lj_scene_info *out) {
    if (!sc || !out) return LJ_ERR_INVALID_ARG;
    *out = sc->info;
    return LJ_OK;
}

int lj_gpu_prim_to_shape(lj_scene *sc, int32_t prim, int32_t *shape_id, int32_t *local_prim) {
    if (!sc || !shape_id || !local_prim) return LJ_ERR_INVALID_ARG;
    if (prim < 0 || prim >= (int32_t)sc->prim_shape_host.size()) return LJ_ERR_INVALID_ARG;
    int s = sc->prim_shape_host[prim];
    *shape_id = s;
    *local_prim = prim - sc->shape_prim_base[s];
    return LJ_OK;
}

int lj_gpu_bvh_leaf_prims(lj_scene *sc, int32_t *out, int64_t capacity, int64_t *count) {
    if (!sc || !count) return LJ_ERR_INVALID_ARG;
    const int64_t n = sc->dev.bvh.num_leaf_prims;
    *count = n;
    if (!out) return LJ_OK;
    if (capacity < n) return set_error(sc->ctx, LJ_ERR_SIZE_LIMIT, "bvh_leaf_prims: capacity below the primitive count");
    if (n == 0) return LJ_OK;
    cudaSetDevice(sc->ctx->device);
    std::vector<float4> rec((size_t)n * kPrimF4);
    if (cudaMemcpy(rec.data(), sc->dev.bvh.prims, sizeof(float4) * rec.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
        return set_error(sc->ctx, LJ_ERR_CUDA, "bvh_leaf_prims: copy failed");
    for (int64_t i = 0; i < n; i++) {
        float w = rec[(size_t)i * kPrimF4].w;
        int32_t id;
        memcpy(&id, &w, sizeof(id));
        out[i] = id;
    }
    return LJ_OK;
}

static int check_status(lj_ctx *ctx, cudaStream_t s, const char *what) {
    int st = 0;
    if (cudaMemcpyAsync(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return set_error(ctx, LJ_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(cudaGetLastError()));
    if (st) {
        cudaMemsetAsync(ctx->d_status, 0, sizeof(int), s);
        return set_error(ctx, LJ_ERR_DEVICE_LIMIT, std::string(what) + ": device loop bound reached (status " +
                                                       std::to_string(st) + ")");
    }
    return LJ_OK;
}

int lj_gpu_trace_closest(lj_scene *sc, const lj_ray *d_rays, lj_hit *d_hits, int64_t n, void *stream) {
    if (!sc || n < 0 || (n > 0 && (!d_rays || !d_hits))) return LJ_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;   // NULL: the legacy default stream
    cudaSetDevice(sc->ctx->device);
    if (launch_trace_closest(sc->dev.bvh, d_rays, d_hits, n, sc->ctx->d_status, s))
        return set_error(sc->ctx, LJ_ERR_CUDA, "trace_closest launch failed");
    return LJ_OK;
}

int lj_gpu_trace_any(lj_scene *sc, const lj_ray *d_rays, uint8_t *d_occluded, int64_t n, void *stream) {
    if (!sc || n < 0 || (n > 0 && (!d_rays || !d_occluded))) return LJ_ERR_INVALID_ARG;
    cudaStream_t s = (cudaStream_t)stream;   // NULL: the legacy default stream
    cudaSetDevice(sc->ctx->device);
    if (launch_trace_any(sc->dev.bvh, d_rays, d_occluded, n, sc->ctx->d_status, s))
        return set_error(sc->ctx, LJ_ERR_CUDA, "trace_any launch failed");
    return LJ_OK;
}

int lj_gpu_trace_counters(lj_scene *sc, const lj_ray *d_rays, int64_t n, int32_t any_hit,
                          int64_t *nodes_fetched, int64_t *prims_tested) {
    if (!sc || n < 0 || (n > 0 && !d_rays) || !nodes_fetched || !prims_tested) return LJ_ERR_INVALID_ARG;
    cudaSetDevice(sc->ctx->device);
    cudaStream_t s = sc->ctx->stream;
    unsigned long long *d = nullptr, h[2] = {0, 0};
    if (cudaMallocAsync(&d, sizeof(h), s) != cudaSuccess)
        return set_error(sc->ctx, LJ_ERR_OUT_OF_MEMORY, "trace_counters: allocation failed");
    cudaMemsetAsync(d, 0, sizeof(h), s);
    int rc = launch_trace_counters(sc->dev.bvh, d_rays, n, any_hit != 0, d, sc->ctx->d_status, s);
    cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(d, s);
    if (rc || cudaStreamSynchronize(s) != cudaSuccess)
        return set_error(sc->ctx, LJ_ERR_CUDA, "trace_counters failed");
    *nodes_fetched = (int64_t)h[0];
    *prims_tested = (int64_t)h[1];
    return check_status(sc->ctx, s, "trace_counters");
}

int lj_gpu_morton_sort(lj_ctx *ctx, const float *d_tri_vertices, int64_t n, uint32_t *d_codes,
                       uint32_t *d_order, void *stream) {
    if (!ctx || n < 0 || (n > 0 && (!d_tri_vertices || !d_codes || !d_order))) return LJ_ERR_INVALID_ARG;
    if (n > (int64_t)1 << 31) return set_error(ctx, LJ_ERR_INVALID_ARG, "morton_sort: n too large");
    if (n == 0) return LJ_OK;
    cudaSetDevice(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;   // NULL: the legacy default stream
    std::string err;
    // scratch: bounds (64 B), sorted keys (n), tmp keys (n), tmp vals (n), histogram
    size_t hist = radix_hist_entries(n);
    size_t need = 64 + sizeof(uint32_t) * (3 * (size_t)n + hist);
    if (need > ctx->scratch_bytes) {
        if (ctx->scratch) cudaFree(ctx->scratch);
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
        if (cudaMalloc(&ctx->scratch, need) != cudaSuccess)
            return set_error(ctx, LJ_ERR_OUT_OF_MEMORY, "morton_sort: scratch allocation failed");
        ctx->scratch_bytes = need;
    }
    uint32_t *bounds = (uint32_t *)ctx->scratch;
    uint32_t *keys = bounds + 16;
    uint32_t *tk = keys + n, *tv = tk + n, *h = tv + n;
    if (morton_codes_tris(d_tri_vertices, n, d_codes, bounds, s, &err))
        return set_error(ctx, LJ_ERR_CUDA, err);
    if (cudaMemcpyAsync(keys, d_codes, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return set_error(ctx, LJ_ERR_CUDA, "morton_sort: copy failed");
    // values = 0..n-1
    if (fill_iota(d_order, n, s)) return set_error(ctx, LJ_ERR_CUDA, "morton_sort: iota failed");
    if (radix_sort_pairs(keys, d_order, tk, tv, h, n, s, &err)) return set_error(ctx, LJ_ERR_CUDA, err);
    return LJ_OK;
}

}  // extern "C"
