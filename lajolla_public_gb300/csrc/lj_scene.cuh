// Device-resident scene layout (HBM) for the GB300 hot path.
//
// The reference keeps the scene in std::vectors of std::variant records
// (src/scene.h:42-82, src/shape.h:39-49) and hands FP32 copies of the
// triangles to Embree (src/shapes/triangle_mesh.inl:1-22).  Here everything
// is flattened to structure-of-arrays buffers owned by one lj_scene handle:
//
//   nodes    compressed 8-wide BVH, 80 B/node = 5 x uint4 (one 128-bit load each)
//   prims    leaf primitive records in BVH leaf order, 48 B = 3 x float4:
//              triangle: (v0, prim) (e1, 0) (e2, 0)
//              sphere:   (center, prim) (radius, 1 [kind]) (0)
//   shading  per-triangle vertex indices + per-vertex positions / normals /
//            uvs (FP32), per-prim shape id, per-shape records
//   materials, lights, light/triangle sampling tables, envmap mips + tables
#pragma once

#include <cstdint>

#include "lj_common.cuh"

namespace lj {

constexpr int kWideNodeU4 = 5;      // 80-byte node
constexpr int kPrimF4 = 3;          // 48-byte leaf primitive record
constexpr int kTraversalStack = 64; // node groups; depth of an 8-wide tree of 2^31 prims is < 12

struct DevBvh {
    const uint4 *nodes;
    const float4 *prims;
    int num_nodes;
    int num_leaf_prims;
};

// Wide node (decoded view of the 5 x uint4):
//   u4[0] = p.x, p.y, p.z (float bits), e.x | e.y << 8 | e.z << 16 | imask << 24
//   u4[1] = child_base, prim_base, meta[0..3], meta[4..7]
//   u4[2] = qlo.x[0..7], qlo.y[0..7]     (8-bit quantized planes)
//   u4[3] = qlo.z[0..7], qhi.x[0..7]
//   u4[4] = qhi.y[0..7], qhi.z[0..7]
// meta byte per child slot: 0 = empty; internal: 0b001 << 5 | (24 + slot);
// leaf: unary(count) << 5 | prim offset (count 1..3, offset 0..23).

struct ShapeRec {
    int kind;               // LJ_SHAPE_MESH / LJ_SHAPE_SPHERE
    int material_id;
    int area_light_id;
    int interior_medium_id;
    int exterior_medium_id;
    int has_normals, has_uvs;
    int tri_begin;          // mesh: first global triangle index
    int num_tris;
    int sampler_offset;     // mesh: offset into tri_cdf (num_tris + 1 entries)
    float total_area;       // mesh: sum of triangle areas
    float cx, cy, cz, radius;  // sphere
};

struct TexRec {
    int kind;               // LJ_TEX_CONST / LJ_TEX_IMAGE / LJ_TEX_CHECKER
    int image_id;
    float v0[3], v1[3];
    float us, vs, uo, vo;
};

struct MatRec {
    int type;
    float eta;
    int textured;           // bitmask of non-constant slots
    int pad;
    TexRec tex[12];
};

struct LightRec {
    int kind;
    int shape_id;
    float intensity[3];
    float scale;
    int image_id;
    float to_world[9], to_local[9];   // 3x3 linear part (row-major)
};

struct MipLevel {
    const float *rgb;   // w*h*3
    int w, h;
};

struct EnvRec {
    int light_id;       // -1: no envmap
    int num_levels;
    MipLevel levels[8];
    int tw, th;         // sampling table size (level 0)
    const float *cdf_rows;   // th * (tw + 1)
    const float *pdf_rows;   // th * tw
    const float *cdf_marg;   // th + 1
    const float *pdf_marg;   // th
};

// Volume<Spectrum> (src/volume.h:12-30): constant value or an FP32 grid,
// (z, y, x, rgb) with x fastest, trilinear lookup, scale applied on lookup.
struct VolRec {
    int kind;              // LJ_VOL_CONST / LJ_VOL_GRID
    int res[3];
    float value[3];
    float pmin[3], pmax[3];
    float scale;
    float max_value[3];    // scale * channel scale * max over the grid (or the constant)
    float gscale[3];       // (res - 1) / (pmax - pmin): world offset -> grid coordinate
    float cscale[3];       // channel scale (lj_volume_desc.channel_scale; 1 when unset)
    int channels;          // 1: data1, one float per voxel; 3: data
    const float4 *data;    // one float4 per voxel (xyz = the channels, w = 0): one 16-byte load per corner
    const float *data1;
};

// Medium (src/medium.h) + phase function.
struct MediumRec {
    int kind;              // LJ_MEDIUM_HOMOGENEOUS / LJ_MEDIUM_HETEROGENEOUS
    int phase_kind;        // LJ_PHASE_ISOTROPIC / LJ_PHASE_HG
    float g;
    float sigma_a[3], sigma_s[3];
    VolRec albedo, density;
};

struct CamRec {
    float sample_to_cam[16];  // row-major
    float cam_to_world[16];
    float org[3];
    int w, h;
    int filter_kind;
    float filter_param;
};

struct DevScene {
    DevBvh bvh;
    // shading geometry
    const int *prim_shape;        // global prim -> shape
    const int *tri_vidx;          // global triangle -> 3 global vertex indices
    const float *vpos;            // global vertex positions (3 floats)
    const float *vnrm;            // global vertex normals (3 floats; meshes with has_normals)
    const float *vuv;             // global vertex uvs (2 floats; meshes with has_uvs)
    const ShapeRec *shapes;
    int num_tris, num_prims, num_shapes;
    // materials
    const MatRec *mats;
    int num_mats;
    // lights
    const LightRec *lights;
    const float *light_pmf;
    const float *light_cdf;       // num_lights + 1
    int num_lights;
    const float *tri_cdf;         // per-mesh area cdfs (normalized), packed
    EnvRec env;
    // images (textures other than the envmap)
    const MipLevel *image_levels; // image i, level l -> image_levels[i * 8 + l]
    const int *image_num_levels;
    // participating media
    const MediumRec *media;
    int num_media;
    int camera_medium;
    int max_null_collisions;
    // camera + options
    CamRec cam;
    float eps;                    // min(radius * 1e-5, 0.01): src/scene.h:99-105
    float bradius;
    float bcenter[3];
    int max_depth, rr_depth;
};

}  // namespace lj
