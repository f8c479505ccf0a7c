/*
 * lj_bytes_model.h -- algorithmic bytes per unit of work of the wavefront
 * kernels, the numerator of every roofline figure this project reports
 * (bench.py mirrors these constants).  "Algorithmic" = what the algorithm
 * must move between HBM and the SMs at least once per unit, counted from the
 * data layout (lj_scene.cuh, lj_path.cu); measured DRAM traffic (ncu
 * dram__bytes_read.sum + dram__bytes_write.sum) is reported beside it.
 *
 * No counterpart in the reference (it publishes no performance model).
 */
#ifndef LJ_BYTES_MODEL_H
#define LJ_BYTES_MODEL_H

/* ray queue entry: org, tnear, dir, tfar (FP32) */
#define LJ_BYTES_RAY 32
/* closest hit: t, prim, u, v */
#define LJ_BYTES_HIT 16
/* compressed 8-wide BVH node (5 x 16 B) */
#define LJ_BYTES_WIDE_NODE 80
/* leaf primitive record: v0 + prim id, e1, e2 (3 x 16 B) */
#define LJ_BYTES_LEAF_PRIM 48
/* path state: pixel 4 + rng 8 + throughput/rr 16 + radiance/eta 16 +
 * previous vertex/pdf 16 + num_vertices 4 */
#define LJ_BYTES_PATH_STATE 64
/* shading geometry of a triangle hit: 3 vertex indices + 3 positions
 * (+ prim -> shape id); normals / uvs add 36 / 24 when present */
#define LJ_BYTES_SHADE_GEOM 52
/* constant-texture material record as read by the shade kernel:
 * type, eta, textured mask, 12 RGB slot values */
#define LJ_BYTES_SHADE_MATERIAL 160
/* shadow queue entry: ray 32 + path id 4 + NEE contribution 16 */
#define LJ_BYTES_SHADOW_ENTRY 52

/* per closest-hit ray: ray in, hit out, plus the BVH bytes of that ray
 * (nodes * 80 + primitive records * 48, counted by lj_gpu_trace_counters) */
#define LJ_BYTES_TRACE_CLOSEST(bvh_bytes) (LJ_BYTES_RAY + LJ_BYTES_HIT + (bvh_bytes))
/* per shadow ray: entry in, radiance read-modify-write (32), BVH bytes */
#define LJ_BYTES_TRACE_SHADOW(bvh_bytes) (LJ_BYTES_SHADOW_ENTRY + 32 + (bvh_bytes))
/* per shade segment: queue entry + hit + path id + state + geometry +
 * material read; state + next ray + path id written; plus one shadow entry
 * written per shadow ray emitted (counted separately) */
#define LJ_BYTES_SHADE_SEGMENT                                                   \
    (LJ_BYTES_RAY + LJ_BYTES_HIT + 4 + LJ_BYTES_PATH_STATE + LJ_BYTES_SHADE_GEOM + \
     LJ_BYTES_SHADE_MATERIAL + LJ_BYTES_PATH_STATE + LJ_BYTES_RAY + 4)

/* volumetric path state (server layout): job 4 + pixel 4 + rng 8 +
 * throughput 16 + radiance 16 + NEE vertex 16 + two pdf products 32 +
 * medium / bounces / flags 16 */
#define LJ_BYTES_VOL_STATE 112
/* NEE request: entry 4 + origin, direction, light point, light normal,
 * sigma_s (5 x 16) + media / bounces / pixel 16 + rng 8 */
#define LJ_BYTES_NEE_REQUEST 108
/* NEE result: transmittance, two pdf products (3 x 16) + rng 8 */
#define LJ_BYTES_NEE_RESULT 56
/* per volumetric segment (a step): ray + hit + state in, state out (or the
 * next ray and state), one NEE request written; the c step reads the
 * request, result, ray, hit and state again and writes state + next ray.
 * Density-grid lookups are excluded (they hit L1/L2 mostly). */
#define LJ_BYTES_VOL_SEGMENT                                                                 \
    (2 * (LJ_BYTES_RAY + LJ_BYTES_HIT + LJ_BYTES_VOL_STATE) + 2 * (LJ_BYTES_VOL_STATE + LJ_BYTES_RAY) + \
     2 * LJ_BYTES_NEE_REQUEST + LJ_BYTES_NEE_RESULT)
/* per NEE request (b step): request in, result out (grid lookups and BVH
 * bytes excluded) */
#define LJ_BYTES_NEE_SHADOW_LOOP (LJ_BYTES_NEE_REQUEST + LJ_BYTES_NEE_RESULT)

#endif /* LJ_BYTES_MODEL_H */
