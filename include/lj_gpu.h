/*
 * lj_gpu.h -- C ABI of the GB300 (sm_103a) rendering hot path for lajolla.
 *
 * This is the drop-in boundary.  In the reference renderer the hot path sits
 * behind three C++ seams:
 *   - Image3 render(const Scene &scene)                     src/render.h:9
 *   - intersect()/occluded() over Embree's rtcIntersect1 /
 *     rtcOccluded1                                           src/intersection.h:39-44,
 *                                                            src/intersection.cpp:7-85
 *   - the BSDF / light / phase functors dispatched through
 *     std::visit                                             src/material.cpp:90-119,
 *                                                            src/light.cpp:56-77,
 *                                                            src/phase_function.cpp:30-47
 * Every entry point below replaces one of them; the comment on each names the
 * reference interface it stands in for.
 *
 * Conventions (all entry points):
 *   - return LJ_OK (0) on success, a negative LJ_ERR_* code on failure; no C++
 *     exception ever crosses this boundary (the reference throws fl_exception,
 *     src/flexception.h:8-24; here that becomes an error code plus
 *     lj_gpu_last_error()).
 *   - descriptors are read during the call and copied; the caller keeps
 *     ownership of every pointer it passes in.
 *   - all device memory is owned by an lj_ctx or lj_scene handle.
 *   - a context is used from one host thread at a time; contexts are
 *     independent of each other.
 *   - "d_" pointers are device pointers (cudaMalloc'd or torch tensors),
 *     everything else is host memory.  `stream` is a cudaStream_t (NULL = the
 *     legacy default stream).
 *   - every device loop is bounded (BVH stack depth, bounces, null
 *     collisions); a kernel that reaches a bound writes a status word which
 *     the host turns into LJ_ERR_DEVICE_LIMIT.
 */
#ifndef LJ_GPU_H
#define LJ_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2: lj_volume_desc.channel_scale, the volumetric kernel classes
 * (LJ_KERNEL_MEDIUM, LJ_KERNEL_NEE) and the volumetric counters of
 * lj_server_stats
 * 3: the emission, camera-ray and medium batches; LJ_RENDER_COUNT_BVH and
 * the lj_stats.bvh_* counters; lj_gpu_scene_update_mesh
 * 4: lj_gpu_scene_create_many */
#define LJ_GPU_ABI_VERSION 4

/* ---- error codes -------------------------------------------------------- */
#define LJ_OK                 0
#define LJ_ERR_INVALID_ARG   -1  /* null handle, bad size, bad enum, bad index */
#define LJ_ERR_CUDA          -2  /* a CUDA runtime call failed                 */
#define LJ_ERR_OUT_OF_MEMORY -3  /* device allocation or HBM budget exceeded   */
#define LJ_ERR_UNSUPPORTED   -4  /* feature not available in this library      */
#define LJ_ERR_DEVICE_LIMIT  -5  /* a bounded device loop hit its limit        */
#define LJ_ERR_NO_DEVICE     -6  /* no CUDA device / wrong architecture        */
#define LJ_ERR_QUEUE_FULL    -7  /* server admission queue is full             */
#define LJ_ERR_NOT_FOUND     -8  /* unknown job id                             */
#define LJ_ERR_TIMEOUT       -9  /* a host-side wait ran out of time           */
#define LJ_ERR_CANCELLED    -10  /* the job was cancelled                      */
#define LJ_ERR_SIZE_LIMIT   -11  /* request larger than a fixed-size buffer    */

typedef struct lj_ctx lj_ctx;
typedef struct lj_scene lj_scene;
typedef struct lj_server lj_server;

/* ---- scene description (flat POD view of the reference's Scene) ---------- */

/* Texture<T> variant, src/texture.h:80-113 (ConstantTexture, ImageTexture,
 * CheckerboardTexture).  Scalar textures use value0[0] / value1[0]. */
enum { LJ_TEX_CONST = 0, LJ_TEX_IMAGE = 1, LJ_TEX_CHECKER = 2 };
typedef struct lj_texture_desc {
    int32_t kind;
    int32_t image_id;          /* LJ_TEX_IMAGE: index into lj_scene_desc.images */
    float value0[3];           /* constant value / checkerboard color0          */
    float value1[3];           /* checkerboard color1                           */
    float uscale, vscale, uoffset, voffset;
} lj_texture_desc;             /* 48 bytes */

/* Material variant, same order as src/material.h:102-110. */
enum {
    LJ_MAT_LAMBERTIAN = 0,
    LJ_MAT_ROUGHPLASTIC = 1,
    LJ_MAT_ROUGHDIELECTRIC = 2,
    LJ_MAT_DISNEY_DIFFUSE = 3,
    LJ_MAT_DISNEY_METAL = 4,
    LJ_MAT_DISNEY_GLASS = 5,
    LJ_MAT_DISNEY_CLEARCOAT = 6,
    LJ_MAT_DISNEY_SHEEN = 7,
    LJ_MAT_DISNEY_BSDF = 8,
    LJ_MAT_COUNT = 9
};
#define LJ_MAT_SLOTS 12
/* Texture slot meaning per material type (struct member order of
 * src/material.h:12-100):
 *   LAMBERTIAN        0 reflectance
 *   ROUGHPLASTIC      0 diffuse_reflectance 1 specular_reflectance 2 roughness
 *   ROUGHDIELECTRIC   0 specular_reflectance 1 specular_transmittance 2 roughness
 *   DISNEY_DIFFUSE    0 base_color 1 roughness 2 subsurface
 *   DISNEY_METAL      0 base_color 1 roughness 2 anisotropic
 *   DISNEY_GLASS      0 base_color 1 roughness 2 anisotropic
 *   DISNEY_CLEARCOAT  0 clearcoat_gloss
 *   DISNEY_SHEEN      0 base_color 1 sheen_tint
 *   DISNEY_BSDF       0 base_color 1 specular_transmission 2 metallic
 *                     3 subsurface 4 specular 5 roughness 6 specular_tint
 *                     7 anisotropic 8 sheen 9 sheen_tint 10 clearcoat
 *                     11 clearcoat_gloss
 */
typedef struct lj_material_desc {
    int32_t type;
    float eta;                 /* interior IOR / exterior IOR (plastic, dielectric, glass, bsdf) */
    lj_texture_desc tex[LJ_MAT_SLOTS];
} lj_material_desc;

/* Shape variant, src/shape.h:21-54 (Sphere, TriangleMesh). */
enum { LJ_SHAPE_MESH = 0, LJ_SHAPE_SPHERE = 1 };
typedef struct lj_shape_desc {
    int32_t kind;
    int32_t material_id;
    int32_t area_light_id;       /* -1 if not emissive */
    int32_t interior_medium_id;  /* -1 = none */
    int32_t exterior_medium_id;
    int32_t num_vertices;
    int32_t num_triangles;
    int32_t pad0;
    const float *positions;      /* num_vertices * 3 (FP32, as Embree receives them) */
    const int32_t *indices;      /* num_triangles * 3 */
    const float *normals;        /* num_vertices * 3 or NULL */
    const float *uvs;            /* num_vertices * 2 or NULL */
    float center[3];             /* sphere */
    float radius;
} lj_shape_desc;

/* Light variant, src/light.h:15-36 (DiffuseAreaLight, Envmap). */
enum { LJ_LIGHT_AREA = 0, LJ_LIGHT_ENVMAP = 1 };
typedef struct lj_light_desc {
    int32_t kind;
    int32_t shape_id;            /* area light: emitting shape              */
    float intensity[3];          /* area light radiance                     */
    int32_t image_id;            /* envmap: RGB image (mip level 0)         */
    float scale;                 /* envmap scale                            */
    int32_t pad0;
    double to_world[16];         /* envmap, row-major 4x4 */
    double to_local[16];
} lj_light_desc;

/* RGB or single-channel FP32 image, row-major, channels interleaved. */
typedef struct lj_image_desc {
    int32_t width, height, channels, pad0;
    const float *data;
} lj_image_desc;

/* Volume<T> variant, src/volume.h:12-30 (ConstantVolume, GridVolume). */
enum { LJ_VOL_CONST = 0, LJ_VOL_GRID = 1 };
typedef struct lj_volume_desc {
    int32_t kind;
    int32_t res[3];              /* x, y, z */
    int32_t channels;            /* 1 or 3 */
    float value[3];              /* constant volume */
    float p_min[3], p_max[3];
    float scale;
    const float *data;           /* res.x*res.y*res.z*channels, x fastest */
    /* Grid value of channel c = data (the one channel, or channel c) *
     * scale * channel_scale[c]: a scalar grid with a chromatic factor
     * (density times a colour), stored at one float per voxel.  All zero
     * means (1, 1, 1), the reference's GridVolume.  No counterpart in the
     * reference, whose chromatic grids hold three values per voxel. */
    float channel_scale[3];
} lj_volume_desc;

/* Medium variant, src/medium.h:10-22; PhaseFunction src/phase_function.h:9-16. */
enum { LJ_MEDIUM_HOMOGENEOUS = 0, LJ_MEDIUM_HETEROGENEOUS = 1 };
enum { LJ_PHASE_ISOTROPIC = 0, LJ_PHASE_HG = 1 };
typedef struct lj_medium_desc {
    int32_t kind;
    int32_t phase_kind;
    float g;
    float sigma_a[3], sigma_s[3];
    lj_volume_desc albedo, density;
} lj_medium_desc;

/* Camera, src/camera.h:9-25, and Filter variant src/filter.h:31-45. */
enum { LJ_FILTER_BOX = 0, LJ_FILTER_TENT = 1, LJ_FILTER_GAUSSIAN = 2 };
typedef struct lj_camera_desc {
    double cam_to_world[16];     /* row-major */
    double fov;                  /* degrees */
    int32_t width, height;
    int32_t filter_kind;
    float filter_param;          /* box/tent width, gaussian stddev */
    int32_t medium_id;
    int32_t pad0;
} lj_camera_desc;

/* Integrator enum and RenderOptions, src/scene.h:13-31. */
enum {
    LJ_INTEGRATOR_DEPTH = 0,
    LJ_INTEGRATOR_SHADING_NORMAL = 1,
    LJ_INTEGRATOR_MEAN_CURVATURE = 2,
    LJ_INTEGRATOR_RAY_DIFFERENTIAL = 3,
    LJ_INTEGRATOR_MIPMAP_LEVEL = 4,
    LJ_INTEGRATOR_PATH = 5,
    LJ_INTEGRATOR_VOLPATH = 6
};
typedef struct lj_render_options {
    int32_t integrator;
    int32_t samples_per_pixel;
    int32_t max_depth;           /* -1 = Russian roulette only (device cap LJ_MAX_BOUNCES) */
    int32_t rr_depth;
    int32_t vol_path_version;
    int32_t max_null_collisions;
} lj_render_options;

typedef struct lj_scene_desc {
    lj_camera_desc camera;
    lj_render_options options;
    int32_t num_shapes, num_materials, num_lights, num_media, num_images;
    int32_t envmap_light_id;     /* -1 if none */
    const lj_shape_desc *shapes;
    const lj_material_desc *materials;
    const lj_light_desc *lights;
    const lj_medium_desc *media;
    const lj_image_desc *images;
} lj_scene_desc;

/* Hard cap on path length when max_depth == -1 (the reference relies on
 * Russian roulette alone; a device loop must be bounded). */
#define LJ_MAX_BOUNCES 1024

/* ---- context -------------------------------------------------------------- */

/* Replaces rtcNewDevice (src/main.cpp:30) + parallel_init (src/main.cpp:31). */
int lj_gpu_init(int device, lj_ctx **out);
/* Replaces rtcReleaseDevice + parallel_cleanup (src/main.cpp:47-48).
 * Destroys the context's remaining scenes: their handles are invalid after. */
void lj_gpu_shutdown(lj_ctx *ctx);
/* Message of the last failing call on this context ("" if none). */
const char *lj_gpu_last_error(lj_ctx *ctx);
int lj_gpu_abi_version(void);

/* ---- scene ---------------------------------------------------------------- */

/* Replaces Scene::Scene's Embree registration + rtcCommitScene + sampling
 * table construction (src/scene.cpp:4-53).  Copies the description to the
 * device and builds the BVH there (LBVH -> 8-wide compressed BVH). */
int lj_gpu_scene_create(lj_ctx *ctx, const lj_scene_desc *desc, lj_scene **out);
/* n scenes at once, each exactly as lj_gpu_scene_create makes it (the same
 * BVH, tables and device records), with their copies and device builds on
 * streams of their own and their host-side tables on threads of their own
 * (up to 8), so that a server's resident pool loads in about the time of
 * its largest scene: a BVH build is a chain of small dependent launches,
 * and the chains of several scenes overlap.  Every description is checked
 * first (lj_gpu_scene_validate's checks); on any error no scene is kept,
 * out[0..n) are all NULL and the message names the failing description's
 * index.  Returns when every scene is on the device.  Replaces n
 * Scene::Scene constructions (src/scene.cpp:4-53), one per scene file a
 * server keeps resident. */
int lj_gpu_scene_create_many(lj_ctx *ctx, int32_t n, const lj_scene_desc *const *descs, lj_scene **out);
/* The checks lj_gpu_scene_create makes before it touches the device, with no
 * context and no device needed: indices in range (shapes -> materials,
 * lights, media; lights -> shapes, images; textures -> images), known kinds,
 * positive sizes.  Returns LJ_OK, or LJ_ERR_INVALID_ARG with the reason in
 * msg (NUL-terminated, at most msg_size bytes; msg may be NULL).  Where the
 * reference's parser throws fl_exception (src/flexception.h:24,
 * src/parsers/parse_scene.cpp) on such input. */
int lj_gpu_scene_validate(const lj_scene_desc *desc, char *msg, int msg_size);
/* New vertex positions (and, when not NULL, normals) of mesh `shape_id`
 * of a resident scene, num_vertices * 3 host floats (the mesh's vertex count
 * at creation), with the BVH brought up to date on the device without
 * uploading the scene again: LJ_UPDATE_REFIT keeps the tree's topology and
 * recomputes its boxes bottom-up (fast; traversal slows down as the motion
 * grows), LJ_UPDATE_REBUILD builds a new tree from the new positions.  The
 * scene's bounds, bounding sphere, shadow epsilon, the mesh's emitter areas
 * and the light-selection table follow the new positions, so the scene
 * renders as one created with them would.  Waits for the device's queued
 * work first.  Refused (LJ_ERR_INVALID_ARG) while the scene is registered
 * with a running server.  Replaces rtcUpdateGeometryBuffer +
 * rtcCommitGeometry + rtcCommitScene, Embree's path for moved geometry (the
 * reference builds its Embree scene once, src/scene.cpp:19-34). */
enum { LJ_UPDATE_REFIT = 0, LJ_UPDATE_REBUILD = 1 };
int lj_gpu_scene_update_mesh(lj_scene *scene, int32_t shape_id, const float *positions, const float *normals,
                             int32_t num_vertices, int32_t mode);
/* Replaces Scene::~Scene / rtcReleaseScene (src/scene.cpp:55-59). */
void lj_gpu_scene_destroy(lj_scene *scene);

typedef struct lj_scene_info {
    float bounds_lower[3], bounds_upper[3]; /* rtcGetSceneBounds (src/scene.cpp:29-34) */
    double bsphere_radius;                  /* Scene::bounds.radius */
    double bsphere_center[3];
    int64_t num_triangles;                  /* all meshes */
    int64_t num_prims;                      /* triangles + spheres */
    int64_t num_wide_nodes;                 /* compressed 8-wide BVH nodes (80 B each) */
    int64_t num_binary_nodes;               /* LBVH internal nodes */
    int64_t device_bytes;                   /* HBM held by this scene */
    double build_ms;                        /* device BVH build time */
} lj_scene_info;
int lj_gpu_scene_info(lj_scene *scene, lj_scene_info *out);

/* ---- render -------------------------------------------------------------- */

/* lj_render_params.flags */
#define LJ_RENDER_PROFILE 1      /* time each kernel class with CUDA events (adds event records) */
#define LJ_RENDER_COUNT_BVH 2    /* after each traversal launch, an instrumented traversal of every
                                    LJ_COUNT_BVH_STRIDE-th queue entry counts the BVH bytes it reads
                                    (lj_stats.bvh_*; measurement only: extra launches) */
#define LJ_COUNT_BVH_STRIDE 16

typedef struct lj_render_params {
    uint64_t seed;               /* job seed; RNG is keyed on (seed, pixel, sample) */
    int32_t spp;                 /* 0 = scene options.samples_per_pixel */
    int32_t sample_offset;       /* first sample index (resume / split renders) */
    int32_t max_paths_in_flight; /* 0 = library default (wavefront width) */
    int32_t flags;               /* LJ_RENDER_* bits */
} lj_render_params;

/* Kernel classes of the wavefront, for LJ_RENDER_PROFILE. */
enum {
    LJ_KERNEL_CAMERA = 0,        /* ray generation                      */
    LJ_KERNEL_TRACE = 1,         /* closest-hit traversal               */
    LJ_KERNEL_SHADE = 2,         /* shading / NEE / BSDF sampling       */
    LJ_KERNEL_SHADOW = 3,        /* shadow any-hit traversal            */
    LJ_KERNEL_OTHER = 4,         /* resolve, scale, queue bookkeeping   */
    LJ_KERNEL_MEDIUM = 5,        /* volpath: delta tracking, emission,
                                    phase / BSDF sampling              */
    LJ_KERNEL_NEE = 6,           /* volpath: NEE shadow loop (closest
                                    hits + ratio tracking)             */
    LJ_KERNEL_CLASSES = 7
};

typedef struct lj_stats {
    double device_ms;            /* kernel time of the render (CUDA events)   */
    int64_t samples;             /* camera samples traced                     */
    int64_t rays_closest;        /* closest-hit rays traced                   */
    int64_t rays_shadow;         /* shadow rays traced                        */
    int64_t path_segments;       /* shade-kernel invocations                  */
    int64_t kernel_launches;     /* kernels launched by this call             */
    int64_t null_collisions;     /* volpath: null-collision events            */
    int64_t real_collisions;     /* volpath: real scattering events           */
    double class_ms[LJ_KERNEL_CLASSES];        /* LJ_RENDER_PROFILE only */
    int64_t class_launches[LJ_KERNEL_CLASSES]; /* LJ_RENDER_PROFILE only */
    /* LJ_RENDER_COUNT_BVH only, [0] closest-hit queues, [1] shadow-ray
     * queues (the path tracer's; the volumetric NEE loop is not counted):
     * rays counted, 80-byte wide nodes fetched and 48-byte leaf records
     * tested by those rays. */
    int64_t bvh_rays[2], bvh_nodes[2], bvh_prims[2];
} lj_stats;

/* Replaces Image3 render(const Scene&) (src/render.cpp:155-170).  Writes the
 * W*H*3 FP32 image (the per-pixel mean over spp samples, HWC) into host
 * memory `out_rgb`.  Host<->device copies are part of the call. */
int lj_gpu_render(lj_scene *scene, const lj_render_params *params,
                  float *out_rgb, lj_stats *stats);

/* Same as lj_gpu_render but leaves the image in device memory `d_out_rgb`
 * (W*H*3 floats) and runs on `stream`; stats->device_ms is 0 unless `stats`
 * is non-NULL, in which case the call synchronizes.  With max_depth -1 or
 * above 8 the call also reads the live-path count back every 4 bounces (a
 * stream synchronization) to stop once every path has ended. */
int lj_gpu_render_device(lj_scene *scene, const lj_render_params *params,
                         float *d_out_rgb, void *stream, lj_stats *stats);

/* ---- batch kernels (oracle tests and microbenchmarks) -------------------- */

/* Ray layout: 32 bytes, FP32, as RTCRay's first two float4s (rtcore_ray.h). */
typedef struct lj_ray {
    float org[3];
    float tnear;
    float dir[3];
    float tfar;
} lj_ray;

/* Hit layout: 16 bytes.  prim = global primitive index (triangles of all
 * meshes in shape order, then spheres), -1 on miss. u, v = barycentrics
 * (Embree convention: p = (1-u-v) p0 + u p1 + v p2).  Primitives at exactly
 * the same distance resolve to the lower index, whatever the traversal
 * order. */
typedef struct lj_hit {
    float t;
    int32_t prim;
    float u, v;
} lj_hit;

/* Replaces rtcIntersect1 (src/intersection.cpp:32) for n rays at once. */
int lj_gpu_trace_closest(lj_scene *scene, const lj_ray *d_rays, lj_hit *d_hits,
                         int64_t n, void *stream);
/* Replaces rtcOccluded1 (src/intersection.cpp:83) for n rays at once;
 * d_occluded[i] = 1 if any primitive lies in (tnear, tfar). */
int lj_gpu_trace_any(lj_scene *scene, const lj_ray *d_rays, uint8_t *d_occluded,
                     int64_t n, void *stream);
/* Maps a global primitive index to (shape id, primitive id within shape). */
int lj_gpu_prim_to_shape(lj_scene *scene, int32_t prim, int32_t *shape_id,
                         int32_t *local_prim);
/* Primitive index of every leaf record of the scene's BVH, in leaf order
 * (host array of capacity entries; *count = number of records; out = NULL
 * only reports the count).  For structural checks (every primitive exactly
 * once).  No reference counterpart. */
int lj_gpu_bvh_leaf_prims(lj_scene *scene, int32_t *out, int64_t capacity, int64_t *count);

/* Instrumented traversal (a separate, slower kernel; for byte accounting):
 * for n rays, the total number of 80-byte wide nodes fetched and 48-byte leaf
 * primitive records tested by closest-hit (any_hit = 0) or any-hit traversal.
 * No reference counterpart (Embree exposes no traversal counters). */
int lj_gpu_trace_counters(lj_scene *scene, const lj_ray *d_rays, int64_t n, int32_t any_hit,
                          int64_t *nodes_fetched, int64_t *prims_tested);

/* 30-bit Morton codes (10 bits per axis) of triangle centroids over the
 * centroid bounding box, and the stable sort order of those codes -- the
 * first two stages of the LBVH build (replaces the BVH build behind
 * rtcCommitScene, src/scene.cpp:27).  d_tri_vertices: n*9 floats
 * (v0, v1, v2).  Outputs: d_codes[n] (unsorted, per triangle) and
 * d_order[n] (triangle indices in ascending code order, ties by index). */
int lj_gpu_morton_sort(lj_ctx *ctx, const float *d_tri_vertices, int64_t n,
                       uint32_t *d_codes, uint32_t *d_order, void *stream);

/* Same results as lj_gpu_morton_sort, for callers that cannot allocate
 * device memory when they call it (no counterpart in the reference, which
 * has no GPU path).  It takes no context and calls no allocator: its working
 * memory is one fixed 2 MiB array inside this library, held on every GPU
 * that loads the library until the process exits.  Hence the limit:
 * n <= LJ_NOALLOC_MORTON_MAX_TRIANGLES, else LJ_ERR_SIZE_LIMIT (nothing is
 * queued).  The first call in each CUDA context (a device's primary
 * context, or a driver-API context current on the calling thread) looks up
 * the array's device address in that context and caches it under the
 * context's unique id; a context created anew (e.g. after cudaDeviceReset)
 * gets a new id and a fresh lookup.  Make the first call in a context before
 * any stream capture begins.  Every call reuses the same array, so
 * calls that overlap on the GPU race: order them (same stream, or events).
 * Errors are returned as codes only (there is no context for a message). */
#define LJ_NOALLOC_MORTON_MAX_TRIANGLES 65536
int lj_gpu_morton_sort_noalloc(const float *d_tri_vertices, int64_t n, uint32_t *d_codes,
                               uint32_t *d_order, void *stream);

/* BSDF batch: replaces eval / sample_bsdf / pdf_sample_bsdf
 * (src/material.cpp:90-119) for n independent queries in the local shading
 * frame of a vertex whose geometric and shading normal are +z (the setup of
 * the reference's src/tests/materials.cpp:55-60).
 *   params:  n * lj_gpu_bsdf_param_count(type) floats: per query the
 *            material's texture slots above packed in slot order (RGB slots
 *            3 floats, scalar slots 1 float), followed by eta.
 *   dir_in/dir_out: n*3, rnd: n*3 (uv, w).
 *   eval -> out_value n*3; pdf -> out_pdf n; sample -> out_dir n*3,
 *   out_eta n, out_roughness n, out_valid n (0/1). */
enum { LJ_BSDF_OP_EVAL = 0, LJ_BSDF_OP_PDF = 1, LJ_BSDF_OP_SAMPLE = 2 };
/* Packed parameter count per query for a material type, -1 if unknown. */
int lj_gpu_bsdf_param_count(int32_t material_type);
typedef struct lj_bsdf_batch {
    int32_t material_type;
    int32_t op;
    int32_t transport_to_view;   /* 0 = TransportDirection::TO_LIGHT */
    int32_t pad0;
    const float *d_params;
    const float *d_dir_in;
    const float *d_dir_out;
    const float *d_rnd;
    float *d_out_value;
    float *d_out_pdf;
    float *d_out_dir;
    float *d_out_eta;
    float *d_out_roughness;
    int32_t *d_out_valid;
} lj_bsdf_batch;
int lj_gpu_bsdf_batch(lj_ctx *ctx, const lj_bsdf_batch *batch, int64_t n, void *stream);

/* Light batch: replaces sample_light + sample_point_on_light +
 * pdf_point_on_light + light_pmf (src/scene.cpp:61-67, src/light.cpp:56-77)
 * for n reference points of a scene.  rnd: n*4 (light_w, uv, shape_w) in the
 * order src/path_tracing.h:98-100 consumes them.
 * Outputs: light id, point n*3, normal n*3, pdf = light_pmf * pdf_point. */
int lj_gpu_light_sample_batch(lj_scene *scene, const float *d_ref_points,
                              const float *d_rnd, int32_t *d_out_light,
                              float *d_out_point, float *d_out_normal,
                              float *d_out_pdf, int64_t n, void *stream);

/* Emission batch: replaces emission(light, view_dir, view_footprint,
 * point_on_light, scene) (src/light.cpp:56-77; area light
 * src/lights/diffuse_area_light.inl:15-20, envmap src/lights/envmap.inl:44-73)
 * for n queries.  d_light: light ids; d_view_dir n*3 (pointing from the
 * light, as the reference's view_dir); d_point / d_normal n*3 the point on
 * the light and its normal (an envmap ignores them).  out n*3.  The
 * reference's envmap footprint never leaves mip level 0 (it is computed from
 * the direction alone and clamped), so there is no footprint argument.  A
 * light id outside [0, num_lights) gives NaN. */
int lj_gpu_light_emission_batch(lj_scene *scene, const int32_t *d_light, const float *d_view_dir,
                                const float *d_point, const float *d_normal, float *d_out_emission,
                                int64_t n, void *stream);

/* Camera batch: replaces sample_primary (src/camera.cpp:23-47) with the
 * scene camera's pixel filter (box / tent / Gaussian, src/filters/*.inl)
 * for n screen positions d_screen (n*2, in [0,1)^2, x right, y down).
 * Outputs: ray origins and unit directions, n*3 each. */
int lj_gpu_camera_ray_batch(lj_scene *scene, const float *d_screen, float *d_out_org,
                            float *d_out_dir, int64_t n, void *stream);

/* Medium batch: replaces get_sigma_a / get_sigma_s (src/medium.cpp:31-37,
 * src/media/*.inl, with the GridVolume trilinear lookup of
 * src/volume.h:44-81) at n points d_points (n*3), and get_majorant
 * (src/medium.cpp:27-29, the grid box slab test src/volume.h:124-144) for
 * the n rays (d_points[i], d_dirs[i], tfar = inf), of medium `medium_id` of
 * the scene.  Outputs n*3 each; any output may be NULL. */
int lj_gpu_medium_batch(lj_scene *scene, int32_t medium_id, const float *d_points, const float *d_dirs,
                        float *d_out_sigma_a, float *d_out_sigma_s, float *d_out_majorant,
                        int64_t n, void *stream);

/* Phase batch: replaces eval / sample_phase_function / pdf_sample_phase
 * (src/phase_function.cpp:30-47) for Henyey-Greenstein (g) or isotropic
 * (phase_kind).  out_value n (eval), out_pdf n, out_dir n*3 (sample). */
int lj_gpu_phase_batch(lj_ctx *ctx, int32_t phase_kind, float g,
                       const float *d_dir_in, const float *d_dir_out,
                       const float *d_rnd, float *d_out_value, float *d_out_pdf,
                       float *d_out_dir, int64_t n, void *stream);

/* ---- serving: continuous batching of render jobs ------------------------ */
/* No counterpart in the reference, whose main.cpp renders one scene per
 * process.  A server keeps scenes, BVHs and per-job accumulators resident and
 * runs the paths of every live job in one pool of wavefront queues: when a
 * path ends, its slot is refilled with a sample of the next job in the
 * scheduling order, so jobs that arrive while others run are admitted as
 * slots and memory free up and their work overlaps on the device.  Each
 * wave (ray generation, closest hit, shade, shadow rays, retire) is replayed
 * from a captured CUDA graph.  Samples are keyed on (job seed, pixel,
 * sample) as in lj_gpu_render and summed in 64-bit fixed point (2^-32
 * units), so a job's image is bit-identical whatever else runs beside it.
 * Path and volumetric path (v6) scenes; each class of job has its own queue
 * and shade kernel (other integrators: LJ_ERR_UNSUPPORTED).  A sample with a
 * non-finite channel is dropped and counted in samples_dropped.
 * The server runs a host thread of its own; its functions may be called
 * from any one client thread at a time.  A scene submitted to a server stays
 * registered with it until lj_gpu_server_stop; lj_gpu_scene_destroy leaves
 * such a scene alive (and sets the context's error message). */
enum { LJ_SCHED_FIFO = 0, LJ_SCHED_SRPT = 1 };  /* SRPT: fewest remaining samples first */
typedef struct lj_server_options {
    int64_t hbm_budget_bytes;    /* scenes + live jobs + path pool; 0 = 120 GiB            */
    int64_t path_pool;           /* paths in flight over all jobs; 0 = 1 << 22             */
    int32_t block_size;          /* 64, 128 or 256; 0 = 128                                */
    int32_t max_live_jobs;       /* job table size, <= 4096; 0 = 256                       */
    int32_t max_queued_jobs;     /* submissions waiting for admission; 0 = 65536           */
    int32_t waves_per_poll;      /* waves between host completion checks; 0 = 8            */
    int32_t policy;              /* LJ_SCHED_*                                             */
    int32_t use_graphs;          /* 1 = replay captured CUDA graphs, 0 = plain launches    */
    int32_t flags;               /* LJ_SERVER_PROFILE: time each kernel class with CUDA
                                    events (plain launches, a host sync per poll)          */
    int32_t tune_objective;      /* lj_gpu_server_autotune: LJ_TUNE_*                      */
} lj_server_options;
/* Autotuner objectives.  BALANCED: among the candidates within 3% of the
 * highest throughput, the one with the lowest median job latency (a larger
 * path pool often buys a little throughput with much later small jobs);
 * THROUGHPUT: the highest Msamples/s; LATENCY: the lowest median latency. */
enum { LJ_TUNE_BALANCED = 0, LJ_TUNE_THROUGHPUT = 1, LJ_TUNE_LATENCY = 2 };
#define LJ_SERVER_PROFILE 1
#define LJ_SERVER_ONE_SHADE_KERNEL 2   /* every job through the all-materials shade kernel */

typedef struct lj_job_desc {
    uint64_t seed;               /* RNG key, as lj_render_params.seed                      */
    int32_t spp;                 /* 0 = scene options.samples_per_pixel                    */
    int32_t sample_offset;
    int32_t width, height;       /* 0 = the scene camera's resolution (same fov)           */
    int32_t override_depth;      /* 1 = use max_depth / rr_depth below                     */
    int32_t max_depth, rr_depth;
    int32_t flags;               /* lj_gpu_render_job_device: LJ_RENDER_* bits             */
} lj_job_desc;

enum { LJ_JOB_QUEUED = 0, LJ_JOB_RUNNING = 1, LJ_JOB_DONE = 2, LJ_JOB_FAILED = 3, LJ_JOB_CANCELLED = 4 };
typedef struct lj_job_status {
    int32_t state;               /* LJ_JOB_*                                               */
    int32_t error;               /* LJ_ERR_* when FAILED                                   */
    int32_t width, height;
    int64_t samples_total;
    int64_t samples_done;        /* as of the server's last completion check              */
    int64_t samples_dropped;     /* non-finite samples left out of the sum                 */
    double submit_ms, admit_ms, finish_ms;   /* server clock (ms since start)              */
} lj_job_status;

typedef struct lj_server_stats {
    int64_t jobs_submitted, jobs_done, jobs_failed, jobs_cancelled;
    int64_t waves;               /* wavefront passes launched                              */
    int64_t graph_launches;
    int64_t samples_done;
    int64_t bytes_resident;      /* scenes + live jobs + path pool                         */
    double busy_ms;              /* host time with paths in flight                         */
    int64_t rays_closest, rays_shadow, path_segments;   /* device counters, last poll     */
    int64_t kernel_launches;
    double class_ms[LJ_KERNEL_CLASSES];        /* LJ_SERVER_PROFILE only (regen = CAMERA,
                                                  plan + retire = OTHER)                   */
    int64_t class_launches[LJ_KERNEL_CLASSES];
    int64_t vol_segments, nee_requests;        /* volpath device counters, last poll       */
    int64_t null_collisions, real_collisions;
} lj_server_stats;

int lj_gpu_server_start(lj_ctx *ctx, const lj_server_options *options, lj_server **out);
/* Queues a render of `scene` (LJ_ERR_QUEUE_FULL when max_queued_jobs are
 * waiting; LJ_ERR_OUT_OF_MEMORY when the job cannot fit the budget even
 * alone).  *job_id identifies it in the calls below. */
int lj_gpu_server_submit(lj_server *server, lj_scene *scene, const lj_job_desc *job, int64_t *job_id);
int lj_gpu_server_poll(lj_server *server, int64_t job_id, lj_job_status *status);
/* Waits until the job is no longer queued or running (timeout_s < 0: no
 * limit; LJ_ERR_TIMEOUT otherwise).  When it is DONE and out_rgb is not
 * NULL, copies its W*H*3 FP32 image (mean over spp) there and forgets the
 * job.  Returns LJ_ERR_CANCELLED / the job's error for those states. */
int lj_gpu_server_wait(lj_server *server, int64_t job_id, double timeout_s, float *out_rgb,
                       lj_job_status *status);
/* Stops issuing the job's samples; paths already in flight finish. */
int lj_gpu_server_cancel(lj_server *server, int64_t job_id);
int lj_gpu_server_stats(lj_server *server, lj_server_stats *stats);
const char *lj_gpu_server_last_error(lj_server *server);
/* Cancels what is left, waits for the device, frees everything. */
int lj_gpu_server_stop(lj_server *server);

/* One job through the single-scene wavefront renderer (no batching): the
 * same samples a server job of this description traces, into device memory
 * `d_out_rgb` (W*H*3 floats at the job's resolution) on `stream`.  Stats as
 * lj_gpu_render_device.  No counterpart in the reference. */
int lj_gpu_render_job_device(lj_scene *scene, const lj_job_desc *job, float *d_out_rgb, void *stream,
                             lj_stats *stats);

/* Autotuner: runs the given job mix (job i renders scenes[job_scene[i]],
 * all submitted at once) once per candidate path pool x block size, then
 * waves between polls for the best of those, and writes the choice that
 * options->tune_objective ranks first into *options (other fields are
 * kept).  With cache_path, results are read from and stored in that JSON
 * file, keyed by device, objective and workload (total samples, largest
 * scene, share of volumetric samples, mean max depth). */
int lj_gpu_server_autotune(lj_ctx *ctx, lj_scene *const *scenes, const lj_job_desc *jobs,
                           const int32_t *job_scene, int32_t n_jobs, const char *cache_path,
                           lj_server_options *options);

#ifdef __cplusplus
}
#endif

#endif /* LJ_GPU_H */
