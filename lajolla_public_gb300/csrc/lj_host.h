// Host-side handle types behind the opaque lj_ctx / lj_scene of lj_gpu.h.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <string>
#include <vector>

#include "../../include/lj_gpu.h"
#include "lj_internal.h"

struct lj_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    int *d_status = nullptr;      // device status word (bounded-loop flags)
    // grow-only scratch for the Morton / radix-sort entry point
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    // live scenes and servers of this context: lj_gpu_shutdown stops and
    // destroys what is left
    std::vector<struct lj_scene *> scenes;
    std::vector<struct lj_server *> servers;
};

// Wavefront buffers owned by a scene, grown on demand (lj_path.cu).
struct PathBuffers {
    size_t capacity = 0;
    void *block = nullptr;
    size_t bytes = 0;
};

struct lj_scene {
    lj_ctx *ctx = nullptr;
    cudaStream_t upload_stream = nullptr;   // the stream the scene's creation copies and builds on
    lj::DevScene dev{};
    std::vector<void *> allocs;   // device allocations freed on destroy
    lj_scene_info info{};
    lj_render_options options{};
    int width = 0, height = 0;
    int num_spheres = 0;
    std::vector<int> shape_prim_base;   // shape -> first global prim
    std::vector<int> prim_shape_host;   // global prim -> shape
    PathBuffers path;
    bool has_media = false;
    lj_camera_desc camera{};
    uint32_t mat_mask = 0;             // bit t: a material of type t exists
    std::atomic<int> server_refs{0};   // servers this scene is registered with
    // kept for lj_gpu_scene_update_mesh: the BVH's levels and sphere records,
    // where each mesh's vertices start, the host copy of the shape records
    // and the triangle indices of emitting meshes (their areas feed the
    // light tables), and each light's power factor (area light: luminance x
    // pi, times its shape's area; envmap: pi x mean table value, times the
    // bounding radius squared)
    const float *d_spheres = nullptr;
    std::vector<int> bvh_levels;
    std::vector<int> shape_vbase, shape_nverts;
    std::vector<lj::ShapeRec> shapes_host;
    std::vector<std::vector<int32_t>> emitter_indices;
    std::vector<double> light_factor;
};

namespace lj {
int set_error(lj_ctx *ctx, int code, const std::string &msg);
// lj_capi.cu: camera record (src/camera.cpp:7-21) at a given resolution
void make_cam_rec(const lj_camera_desc &c, int width, int height, CamRec &cam);
// lj_path.cu
int render_path(lj_scene *scene, const lj_render_params *params, float *d_out, cudaStream_t s,
                lj_stats *stats, bool sync_stats, const lj_job_desc *job);
// lj_volpath.cu
int render_volpath(lj_scene *scene, const lj_render_params *params, float *d_out, cudaStream_t s,
                   lj_stats *stats, const lj_job_desc *job);
// lj_aux.cu
int render_aux(lj_scene *scene, const lj_render_params *params, float *d_out, cudaStream_t s,
               lj_stats *stats);
}  // namespace lj
