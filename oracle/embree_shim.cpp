// ORACLE / TEST INFRASTRUCTURE -- not part of the product.
//
// A CPU implementation of the 20 Embree 4 API functions the reference renderer
// calls (src/scene.cpp:20-34, src/shapes/triangle_mesh.inl:2-20,
// src/shapes/sphere.inl:151-162, src/intersection.cpp:32,83, src/main.cpp:30,48).
// The Embree 4.3.0 binary is missing from the reference mount
// (.MISSING_LARGE_BLOBS) and its source is not vendored, so this shim lets the
// unmodified reference sources link into a working `lajolla` and into the
// golden-vector harness.  Only the public header types are used (names and
// signatures); the implementation is ours:
//   - triangles: the FP32 test of ljo_geom.h (the same arithmetic the GPU uses)
//   - user geometry (spheres): the registered bounds/intersect/occluded callbacks
//   - acceleration: a median-split binary BVH (ljo_geom.h)
// Hit semantics follow rtcIntersect1/rtcOccluded1 as the reference relies on
// them: geomID/primID/u/v/Ng/tfar written on the closest hit; occluded sets
// tfar = -inf.
#include <embree4/rtcore.h>

#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

#include "ljo_geom.h"

using ljo::f3;

struct RTCDeviceTy {
    int refs = 1;
};

struct RTCGeometryTy {
    RTCGeometryType type;
    int refs = 1;
    std::vector<float> vertices;     // 4 floats per vertex (16-byte stride)
    std::vector<uint32_t> indices;   // 3 per triangle
    size_t num_vertices = 0, num_triangles = 0;
    unsigned int user_prims = 0;
    void *user_ptr = nullptr;
    RTCBoundsFunction bounds_fn = nullptr;
    RTCIntersectFunctionN intersect_fn = nullptr;
    RTCOccludedFunctionN occluded_fn = nullptr;
};

struct Prim {
    uint32_t geom;
    uint32_t prim;
};

struct RTCSceneTy {
    int refs = 1;
    std::vector<RTCGeometryTy *> geoms;
    std::vector<Prim> prims;
    std::vector<ljo::TriPre> tri_pre;   // parallel to prims (unused for user prims)
    ljo::CpuBvh bvh;
    ljo::Box bounds;
};

extern "C" {

RTCDevice rtcNewDevice(const char *) { return new RTCDeviceTy(); }
void rtcReleaseDevice(RTCDevice d) {
    if (d && --d->refs == 0) delete d;
}

RTCScene rtcNewScene(RTCDevice) { return new RTCSceneTy(); }
void rtcSetSceneBuildQuality(RTCScene, enum RTCBuildQuality) {}
void rtcSetSceneFlags(RTCScene, enum RTCSceneFlags) {}

void rtcReleaseScene(RTCScene s) {
    if (!s || --s->refs > 0) return;
    for (RTCGeometryTy *g : s->geoms)
        if (--g->refs == 0) delete g;
    delete s;
}

RTCGeometry rtcNewGeometry(RTCDevice, enum RTCGeometryType type) {
    RTCGeometryTy *g = new RTCGeometryTy();
    g->type = type;
    return g;
}

unsigned int rtcAttachGeometry(RTCScene s, RTCGeometry g) {
    g->refs++;
    s->geoms.push_back(g);
    return (unsigned int)(s->geoms.size() - 1);
}

void *rtcSetNewGeometryBuffer(RTCGeometry g, enum RTCBufferType type, unsigned int,
                              enum RTCFormat, size_t byteStride, size_t itemCount) {
    if (type == RTC_BUFFER_TYPE_VERTEX) {
        if (byteStride != 16) std::abort();
        g->num_vertices = itemCount;
        g->vertices.assign(itemCount * 4 + 4, 0.f);
        return g->vertices.data();
    } else if (type == RTC_BUFFER_TYPE_INDEX) {
        if (byteStride != 12) std::abort();
        g->num_triangles = itemCount;
        g->indices.assign(itemCount * 3, 0u);
        return g->indices.data();
    }
    std::abort();
}

void rtcSetGeometryVertexAttributeCount(RTCGeometry, unsigned int) {}
void rtcSetGeometryUserPrimitiveCount(RTCGeometry g, unsigned int n) { g->user_prims = n; }
void rtcSetGeometryUserData(RTCGeometry g, void *ptr) { g->user_ptr = ptr; }
void rtcSetGeometryBoundsFunction(RTCGeometry g, RTCBoundsFunction f, void *) { g->bounds_fn = f; }
void rtcSetGeometryIntersectFunction(RTCGeometry g, RTCIntersectFunctionN f) { g->intersect_fn = f; }
void rtcSetGeometryOccludedFunction(RTCGeometry g, RTCOccludedFunctionN f) { g->occluded_fn = f; }
void rtcCommitGeometry(RTCGeometry) {}
void rtcReleaseGeometry(RTCGeometry g) {
    if (g && --g->refs == 0) delete g;
}

static f3 vtx(const RTCGeometryTy *g, uint32_t i) {
    return f3{g->vertices[i * 4 + 0], g->vertices[i * 4 + 1], g->vertices[i * 4 + 2]};
}

void rtcCommitScene(RTCScene s) {
    s->prims.clear();
    s->tri_pre.clear();
    std::vector<ljo::Box> boxes;
    s->bounds.reset();
    for (uint32_t gi = 0; gi < s->geoms.size(); gi++) {
        RTCGeometryTy *g = s->geoms[gi];
        if (g->type == RTC_GEOMETRY_TYPE_TRIANGLE) {
            for (uint32_t t = 0; t < g->num_triangles; t++) {
                f3 p0 = vtx(g, g->indices[t * 3 + 0]);
                f3 p1 = vtx(g, g->indices[t * 3 + 1]);
                f3 p2 = vtx(g, g->indices[t * 3 + 2]);
                ljo::Box b;
                b.lo[0] = std::min(p0.x, std::min(p1.x, p2.x));
                b.lo[1] = std::min(p0.y, std::min(p1.y, p2.y));
                b.lo[2] = std::min(p0.z, std::min(p1.z, p2.z));
                b.hi[0] = std::max(p0.x, std::max(p1.x, p2.x));
                b.hi[1] = std::max(p0.y, std::max(p1.y, p2.y));
                b.hi[2] = std::max(p0.z, std::max(p1.z, p2.z));
                boxes.push_back(b);
                s->prims.push_back(Prim{gi, t});
                s->tri_pre.push_back(ljo::tri_pre(p0, p1, p2));
                s->bounds.grow(b);
            }
        } else if (g->type == RTC_GEOMETRY_TYPE_USER) {
            for (uint32_t p = 0; p < g->user_prims; p++) {
                RTCBounds rb;
                RTCBoundsFunctionArguments args;
                args.geometryUserPtr = g->user_ptr;
                args.primID = p;
                args.timeStep = 0;
                args.bounds_o = &rb;
                g->bounds_fn(&args);
                ljo::Box b;
                b.lo[0] = rb.lower_x; b.lo[1] = rb.lower_y; b.lo[2] = rb.lower_z;
                b.hi[0] = rb.upper_x; b.hi[1] = rb.upper_y; b.hi[2] = rb.upper_z;
                boxes.push_back(b);
                s->prims.push_back(Prim{gi, p});
                s->tri_pre.push_back(ljo::TriPre{});
                s->bounds.grow(b);
            }
        }
    }
    s->bvh.build(boxes);
}

void rtcGetSceneBounds(RTCScene s, struct RTCBounds *b) {
    b->lower_x = s->bounds.lo[0]; b->lower_y = s->bounds.lo[1]; b->lower_z = s->bounds.lo[2];
    b->upper_x = s->bounds.hi[0]; b->upper_y = s->bounds.hi[1]; b->upper_z = s->bounds.hi[2];
    b->align0 = b->align1 = 0.f;
}

}  // extern "C"

template <bool kAny, typename Fn>
static void traverse(RTCScene s, f3 o, f3 d, float tnear, float *tfar, Fn &&visit_prim) {
    if (s->bvh.nodes.empty()) return;
    f3 inv{1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
    int32_t stack[256];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const ljo::BvhNode &n = s->bvh.nodes[stack[--sp]];
        if (!ljo::box_hit(n.box, o, inv, tnear, *tfar)) continue;
        if (n.left < 0) {
            for (int32_t i = n.first; i < n.first + n.count; i++) {
                if (visit_prim(s->bvh.prim_order[i]) && kAny) return;
            }
        } else {
            stack[sp++] = n.left;
            stack[sp++] = n.right;
        }
    }
}

extern "C" {

void rtcIntersect1(RTCScene s, struct RTCRayHit *rh, struct RTCIntersectArguments *) {
    RTCRay &r = rh->ray;
    f3 o{r.org_x, r.org_y, r.org_z}, d{r.dir_x, r.dir_y, r.dir_z};
    RTCRayQueryContext ctx;
    rtcInitRayQueryContext(&ctx);
    int32_t best = -1;   // global index of the closest primitive so far
    traverse<false>(s, o, d, r.tnear, &r.tfar, [&](int32_t pi) {
        const Prim &p = s->prims[pi];
        RTCGeometryTy *g = s->geoms[p.geom];
        if (g->type == RTC_GEOMETRY_TYPE_TRIANGLE) {
            float t, u, v;
            // equal distances go to the lower primitive index (the GPU's rule)
            if (ljo::tri_intersect(s->tri_pre[pi], o, d, r.tnear, r.tfar, t, u, v) &&
                (t < r.tfar || (best >= 0 && pi < best))) {
                best = pi;
                const ljo::TriPre &tp = s->tri_pre[pi];
                f3 ng = ljo::f3_cross(tp.e1, tp.e2);
                r.tfar = t;
                rh->hit.Ng_x = ng.x; rh->hit.Ng_y = ng.y; rh->hit.Ng_z = ng.z;
                rh->hit.u = u; rh->hit.v = v;
                rh->hit.primID = p.prim;
                rh->hit.geomID = p.geom;
                rh->hit.instID[0] = RTC_INVALID_GEOMETRY_ID;
            }
        } else {
            int valid = -1;
            RTCIntersectFunctionNArguments args;
            args.valid = &valid;
            args.geometryUserPtr = g->user_ptr;
            args.primID = p.prim;
            args.context = &ctx;
            args.rayhit = (RTCRayHitN *)rh;
            args.N = 1;
            args.geomID = p.geom;
            float before = r.tfar;
            g->intersect_fn(&args);
            if (r.tfar != before) best = pi;
        }
        return false;
    });
}

void rtcOccluded1(RTCScene s, struct RTCRay *r, struct RTCOccludedArguments *) {
    f3 o{r->org_x, r->org_y, r->org_z}, d{r->dir_x, r->dir_y, r->dir_z};
    RTCRayQueryContext ctx;
    rtcInitRayQueryContext(&ctx);
    float tfar = r->tfar;
    traverse<true>(s, o, d, r->tnear, &tfar, [&](int32_t pi) {
        const Prim &p = s->prims[pi];
        RTCGeometryTy *g = s->geoms[p.geom];
        if (g->type == RTC_GEOMETRY_TYPE_TRIANGLE) {
            float t, u, v;
            if (ljo::tri_intersect(s->tri_pre[pi], o, d, r->tnear, r->tfar, t, u, v) && t < r->tfar) {
                r->tfar = -INFINITY;
                return true;
            }
        } else {
            int valid = -1;
            RTCOccludedFunctionNArguments args;
            args.valid = &valid;
            args.geometryUserPtr = g->user_ptr;
            args.primID = p.prim;
            args.context = &ctx;
            args.ray = (RTCRayN *)r;
            args.N = 1;
            args.geomID = p.geom;
            g->occluded_fn(&args);
            if (r->tfar < 0) return true;
        }
        return false;
    });
}

}  // extern "C"
