// Host-side declarations shared by the .cu translation units of liblj_gpu.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "lj_scene.cuh"

namespace lj {

// Paths in flight of one wavefront batch of the single-scene renderers when
// the caller does not say (lj_render_params.max_paths_in_flight = 0): 16 Mi
// paths (~4.8 GB of path state and queues for the path tracer, ~6 GB for
// the volumetric one).  Larger batches spread each bounce's launch and its
// last, half-empty warps over more paths: the 1080p x 256 spp terrain
// renders 16 % faster than with 4 Mi, 32 Mi adds 2 % more.
constexpr int64_t kDefaultPathsInFlight = (int64_t)1 << 24;

// Status word bits written by bounded device loops.
enum : int {
    kStatusStackOverflow = 1,
    kStatusBounceCap = 2,
    kStatusNullCollisionCap = 4,
    kStatusQueueOverflow = 8,
};

#define LJ_CUDA_TRY(expr)                                                      \
    do {                                                                       \
        cudaError_t _e = (expr);                                               \
        if (_e != cudaSuccess) {                                               \
            if (err) *err = std::string(#expr) + ": " + cudaGetErrorString(_e); \
            return -2;                                                         \
        }                                                                      \
    } while (0)

// ---- radix sort (lj_bvh.cu) ----
// Keys per tile of the sort's block passes: 256 threads x 8 keys.
constexpr int kRadixThreads = 256;
constexpr int kRadixItems = 8;
constexpr int kRadixTile = kRadixThreads * kRadixItems;
// Histogram entries the sort needs for n keys: 256 buckets per tile.
constexpr size_t radix_hist_entries(int64_t n) {
    return (size_t)256 * (size_t)(n > 0 ? (n + kRadixTile - 1) / kRadixTile : 1);
}
// Stable LSD sort of (key, value) pairs on bits [0, 32) of the key, 8 bits
// per pass.  tmp_keys/tmp_vals: n entries; hist: radix_hist_entries(n).
int radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *tmp_keys, uint32_t *tmp_vals,
                     uint32_t *hist, int64_t n, cudaStream_t s, std::string *err);

// Morton codes of triangle centroids (n x 9 floats) over their centroid box.
// `bounds_scratch`: 8 uint32.
int morton_codes_tris(const float *tri_vertices, int64_t n, uint32_t *codes,
                      uint32_t *bounds_scratch, cudaStream_t s, std::string *err);
// Same, with the caller's centroid buffer (n float4): allocates nothing.
int morton_codes_tris_into(const float *tri_vertices, int64_t n, uint32_t *codes, uint32_t *bounds,
                           float4 *cent, cudaStream_t s);

// ---- BVH build (lj_bvh.cu) ----
struct BvhInput {
    const float *vpos;      // device, global vertex positions
    const int *tri_vidx;    // device, 3 per triangle
    const float *spheres;   // device, 4 floats (c, r) per sphere (prims num_tris ..)
    int num_tris, num_spheres;
    int karras = 0;         // 1: Karras radix tree over the Morton order, 0: PLOC clustering
    int treelet_passes = 3; // PLOC: treelet restructuring passes before the collapse
};
struct BvhOutput {
    uint4 *nodes = nullptr;     // device, owned by the scene
    float4 *prims = nullptr;    // device
    int num_nodes = 0;
    int num_binary = 0;
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // scene AABB (rtcGetSceneBounds)
    double build_ms = 0;
    // wide nodes level by level: level l is [level_start[l], level_start[l + 1])
    std::vector<int> level_start;
};
int build_bvh(const BvhInput &in, BvhOutput *out, cudaStream_t s, std::string *err);
// Refit of a built tree to moved vertices (in.vpos): leaf records rewritten,
// node boxes recomputed level by level from the deepest, topology kept;
// lo / hi receive the new root box.
int refit_bvh(const BvhInput &in, uint4 *nodes, float4 *prims, int num_prims, const std::vector<int> &level_start,
              float lo[3], float hi[3], cudaStream_t s, std::string *err);

// ---- batch trace (lj_bvh.cu) ----
int launch_trace_closest(const DevBvh &bvh, const void *rays, void *hits, int64_t n,
                         int *d_status, cudaStream_t s);
int launch_trace_any(const DevBvh &bvh, const void *rays, uint8_t *occ, int64_t n,
                     int *d_status, cudaStream_t s);
// instrumented traversal: d_counts[0] += nodes fetched, d_counts[1] += prims tested
int launch_trace_counters(const DevBvh &bvh, const void *rays, int64_t n, bool any,
                          unsigned long long *d_counts, int *d_status, cudaStream_t s);
// the same over every stride-th entry of a ray queue whose length is in
// device memory (*d_count <= cap): d_counts[0] += rays counted, [1] += nodes
// fetched, [2] += prims tested
int launch_trace_counters_queue(const DevBvh &bvh, const void *rays, const int *d_count, int64_t cap, int stride,
                                bool any, unsigned long long *d_counts, int *d_status, cudaStream_t s);

}  // namespace lj
