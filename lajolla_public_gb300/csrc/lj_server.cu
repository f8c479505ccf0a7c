// Render server: continuous batching of render jobs over one pool of
// wavefront queues.  No counterpart in the reference (main.cpp renders one
// scene per process); the per-path work is path_tracing
// (src/path_tracing.h:7-325) through shade_segment, or the volumetric path
// tracer's a / b / c steps (lj_volwave.cuh), exactly as in the single-scene
// renderers.  Three path classes share the pool: path jobs whose materials
// are all classic (front of a queue), other path jobs (back of the queue),
// volumetric path jobs (queues of their own).
//
// Device side, one wave (all kernels read their sizes from device memory,
// so a fixed launch sequence can be captured once and replayed):
//   plan     one warp: split the free path slots among the jobs that still
//            have samples to issue, in the host's scheduling order
//            (prefix sums over remaining samples), and advance their
//            issued-sample counters
//   regen    new paths in sample order after the ones that go on: keyed
//            PCG stream, camera ray, state in the current queue of the
//            job's class
//   trace    closest hit of every class's rays; each ray uses the BVH of
//            its job's scene
//   shade    shade_segment with the job's scene and depth options, one
//            instance per path class
//   vol a/b/c  the volumetric steps (b finishes the requests from
//            scattering points; one c instance per material class for the
//            requests from surfaces)
//   shadow   any-hit for the queued NEE rays of the path classes
//   retire   finished paths: 64-bit fixed-point sums into the job's
//            accumulator (one plane per channel: a warp's atomics for one
//            channel land on consecutive words), done counter
// Two waves (ray queues 0 -> 1 -> 0) form one CUDA graph.
//
// Host side, a worker thread admits jobs under the HBM budget, keeps the
// order list current, replays the graph, and every few waves reads the jobs'
// counters back (pinned memory, one event per read) to finish jobs: convert
// the accumulator to the mean image and copy it to pinned host memory.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <thread>
#include <unordered_map>
#include <vector>

#include "lj_host.h"
#include "lj_trace_queue.cuh"
#include "lj_volwave.cuh"
#include "lj_wavefront.cuh"

namespace lj {
namespace {

constexpr int kMaxScenes = 256;
constexpr int kPollsInFlight = 2;
constexpr int kStatWords = 9;   // device counters read back (SrvDev::stats)

struct SrvJob {
    CamRec cam;
    unsigned long long seed;
    long long total;             // npix * spp
    unsigned long long *accum;   // 3 planes of npix sums (R, G, B) in units of 2^-32
    DevBvh bvh;                  // the scene's BVH (a copy: a ray fetched by the
                                 // traversal finds its tree one load sooner)
    int scene, npix, spp, sample_offset;
    int max_depth, rr_depth;
    float spread0;
    float clamp;                 // |sample| bound that keeps the sums inside int64
    int mclass;                  // shade kernel: 0 path, kClassicMats materials; 1 path, any; 2 volpath
    int all_mats;                // volpath: materials outside kClassicMats occur
    int lambert;                 // class 0, every material Lambertian: the class-0 kernel's
                                 // Lambertian-only code shades the job
};

// Material classes of the server's two path shade kernel instances
// (kClassicMats, kAllMats).  A queue holds class-0 paths from its front and
// class-1 paths from its back, so each instance reads a contiguous range.

struct SrvCtr {
    unsigned long long issued, done, dropped, pad;
};

// Path state and ray of every queue entry, in queue order (two buffers:
// the queue a wave reads and the one it fills).  Keeping state in queue
// order makes every state access of regen, shade and retire coalesced; a
// fixed slot per path would scatter them over the whole pool once paths of
// many jobs and depths interleave.
struct StateSoA {
    int *job, *pixel, *nv;
    uint64_t *rng;
    float4 *beta, *L, *prev;
    float4 *ray;             // 2 per entry: org | tnear, dir | tfar
};

// Volumetric paths: their own queue pair (class 2), same idea.
struct VolStateSoA {
    int *job, *pixel;
    uint64_t *rng;
    float4 *beta, *L, *neep, *mdir, *mnee;
    int4 *st;
    float4 *ray;
};

struct SrvDev {
    const DevScene *scenes;
    const SrvJob *jobs;
    SrvCtr *ctr;
    const int *cancel;
    const int *order;            // [0] = entries, [1..] job slots
    int *plan_off;               // per entry: first regen index; [n] = total taken
    int *plan_coff;              // per entry: new paths of the same class in earlier entries
    long long *plan_start;       // per entry: first linear sample index
    StateSoA buf[2];
    float4 *hit;
    VolStateSoA vbuf[2];
    float4 *vhit;
    NeeQueue nee;                // volpath NEE requests of the wave (count: counts + 16)
    float4 *sray;                // shadow rays (2 per entry)
    int *starget;                // entry of the path in the next queue, or retire index | 2^31
    float4 *scontrib;
    int *rjob, *rpixel;          // finished paths
    float4 *rL;
    int *counts;                 // [0],[1] class-0 entries (front) of queue 0 / 1, [2] shadow,
                                 // [3] retire, [5] regen count, [6],[7],[14] class-0 / 1 / 2
                                 // entries that continue into the wave, [8],[9] ray fetch
                                 // counters, [10],[11] class-1 entries (back) of queue 0 / 1,
                                 // [12],[13] entries of volpath queue 0 / 1, [16],[17]
                                 // volpath NEE requests (front, back)
    // queue position of the k-th entry of class 1 (filled from the back)
    LJ_D int back(int k) const { return P - 1 - k; }
    // position of ray r of a queue with n0 class-0 entries
    LJ_D int entry(int r, int n0) const { return r < n0 ? r : back(r - n0); }
    unsigned long long *stats;   // [0] closest rays, [1] shadow rays, [2] shade segments,
                                 // volpath: [3] segments, [4] NEE requests, [5] shadow
                                 // segments, [7] null, [8] real collisions
    int P;                       // queue capacity
    int *status;
};

constexpr int kRetireBit = (int)0x80000000u;

__global__ void k_srv_plan(SrvDev d, int cur) {
    const int lane = threadIdx.x;
    int *counts = d.counts;
    const int n_order = d.order[0];
    // paths that continue into this wave, per class
    const int c0 = counts[cur], c1 = counts[10 + cur], c2 = counts[12 + cur];
    const long long freec = (long long)d.P - c0 - c1 - c2;   // room for new paths
    long long carry = 0, carry0 = 0, carry1 = 0, carry2 = 0;
    for (int base = 0; base < n_order; base += 32) {
        const int k = base + lane;
        long long rem = 0, start = 0;
        int j = -1, cls = 0;
        if (k < n_order) {
            j = d.order[1 + k];
            start = (long long)d.ctr[j].issued;
            cls = d.jobs[j].mclass;
            if (!d.cancel[j]) rem = max(0LL, d.jobs[j].total - start);
        }
        long long incl = rem;
        for (int o = 1; o < 32; o <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const long long off = min(carry + incl - rem, freec);
        const long long n = min(rem, freec - off);
        // prefix of the granted counts within each class
        const long long n0 = cls == 0 ? n : 0, n1 = cls == 1 ? n : 0, n2 = cls == 2 ? n : 0;
        long long i0 = n0, i1 = n1, i2 = n2;
        for (int o = 1; o < 32; o <<= 1) {
            long long y0 = __shfl_up_sync(0xffffffffu, i0, o), y1 = __shfl_up_sync(0xffffffffu, i1, o);
            long long y2 = __shfl_up_sync(0xffffffffu, i2, o);
            if (lane >= o) {
                i0 += y0;
                i1 += y1;
                i2 += y2;
            }
        }
        if (k < n_order) {
            d.plan_off[k] = (int)off;
            d.plan_coff[k] = (int)(cls == 0 ? carry0 + i0 - n0 : (cls == 1 ? carry1 + i1 - n1 : carry2 + i2 - n2));
            d.plan_start[k] = start;
            if (n > 0) d.ctr[j].issued += (unsigned long long)n;
        }
        carry += __shfl_sync(0xffffffffu, incl, 31);
        carry0 += __shfl_sync(0xffffffffu, i0, 31);
        carry1 += __shfl_sync(0xffffffffu, i1, 31);
        carry2 += __shfl_sync(0xffffffffu, i2, 31);
    }
    if (lane == 0) {
        const long long take = min(carry, freec);
        d.plan_off[n_order] = (int)take;
        counts[5] = (int)take;
        counts[6] = c0;
        counts[7] = c1;
        counts[14] = c2;
        counts[cur] = c0 + (int)carry0;   // carry0 + carry1 + carry2 == take
        counts[10 + cur] = c1 + (int)carry1;
        counts[12 + cur] = c2 + (int)carry2;
        counts[cur ^ 1] = 0;
        counts[10 + (cur ^ 1)] = 0;
        counts[12 + (cur ^ 1)] = 0;
        counts[2] = 0;
        counts[3] = 0;
        counts[8] = 0;
        counts[9] = 0;
        counts[16] = 0;
        counts[17] = 0;
    }
}

template <int B>
__global__ void __launch_bounds__(B) k_srv_regen(SrvDev d, int cur) {
    const int n = d.counts[5];
    const int n_order = d.order[0];
    const StateSoA &q = d.buf[cur];
    for (int i = blockIdx.x * B + threadIdx.x; i < n; i += gridDim.x * B) {
        int lo = 0, hi = n_order - 1;   // last entry whose first index is <= i
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (d.plan_off[mid] <= i) lo = mid;
            else hi = mid - 1;
        }
        const int j = d.order[1 + lo];
        const SrvJob &jb = d.jobs[j];
        const long long lin = d.plan_start[lo] + (i - d.plan_off[lo]);
        int pixel, sample;
        if (lin <= 0x7fffffffLL) {   // 32-bit division where it suffices (it is much cheaper)
            const unsigned l = (unsigned)lin, np = (unsigned)jb.npix;
            pixel = (int)(l % np);
            sample = jb.sample_offset + (int)(l / np);
        } else {
            pixel = (int)(lin % jb.npix);
            sample = jb.sample_offset + (int)(lin / jb.npix);
        }
        Pcg rng = pcg_keyed(jb.seed, (uint64_t)pixel, (uint64_t)sample);
        const int x = pixel % jb.cam.w, y = pixel / jb.cam.w;
        float r1 = pcg_uniform(rng), r2 = pcg_uniform(rng);
        V3 o, dir;
        camera_ray(jb.cam, (x + r1) / jb.cam.w, (y + r2) / jb.cam.h, o, dir);
        // after the paths that continue into this wave, in sample order (a
        // fixed, coherent order: neighbouring threads of later kernels get
        // neighbouring pixels)
        const int t = d.plan_coff[lo] + (i - d.plan_off[lo]);
        if (jb.mclass == 2) {   // volumetric path (initial state of k_vol_camera in lj_volpath.cu)
            const VolStateSoA &v = d.vbuf[cur];
            const int s = d.counts[14] + t;
            v.job[s] = j;
            v.pixel[s] = pixel;
            v.rng[s] = rng.state;
            v.beta[s] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
            v.L[s] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            v.neep[s] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            v.mdir[s] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
            v.mnee[s] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
            v.st[s] = make_int4(d.scenes[jb.scene].camera_medium, 0, 1, 1);
            v.ray[2 * s] = make_float4(o.x, o.y, o.z, 0.0f);
            v.ray[2 * s + 1] = make_float4(dir.x, dir.y, dir.z, __int_as_float(0x7f800000));
            continue;
        }
        const int s = jb.mclass == 0 ? d.counts[6] + t : d.back(d.counts[7] + t);
        q.job[s] = j;
        q.pixel[s] = pixel;
        q.rng[s] = rng.state;
        q.beta[s] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
        q.L[s] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        q.prev[s] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        q.nv[s] = 2;
        q.ray[2 * s] = make_float4(o.x, o.y, o.z, 0.0f);
        q.ray[2 * s + 1] = make_float4(dir.x, dir.y, dir.z, __int_as_float(0x7f800000));
    }
}

// Ray queues of the server: each ray uses the BVH of its path's job's scene.
// Rays r < n01 are path-tracer entries (class 0 front, class 1 back), the
// rest volumetric ones.
struct SrvClosestIO {
    const SrvDev &d;
    int cur, n0, n01;   // class-0 entries; class-0 + class-1 entries of queue cur
    LJ_D const DevBvh &bvh(int r) const {
        const int job = r < n01 ? d.buf[cur].job[d.entry(r, n0)] : d.vbuf[cur].job[r - n01];
        return d.jobs[job].bvh;
    }
    LJ_D void load(int r, V3 &o, V3 &dir, float &tn, float &tf) const {
        if (r < n01) load_ray(d.buf[cur].ray, d.entry(r, n0), o, dir, tn, tf);
        else load_ray(d.vbuf[cur].ray, r - n01, o, dir, tn, tf);
    }
    LJ_D void store(int r, const Trav &s) const {
        if (r < n01) d.hit[d.entry(r, n0)] = hit_record(s);
        else d.vhit[r - n01] = hit_record(s);
    }
};
struct SrvShadowIO {
    const SrvDev &d;
    int nxt;
    LJ_D int job_of(int r) const {
        const int t = d.starget[r];
        return t < 0 ? d.rjob[t & 0x7fffffff] : d.buf[nxt].job[t];
    }
    LJ_D const DevBvh &bvh(int r) const { return d.jobs[job_of(r)].bvh; }
    LJ_D void load(int r, V3 &o, V3 &dir, float &tn, float &tf) const { load_ray(d.sray, r, o, dir, tn, tf); }
    LJ_D void store(int r, const Trav &s) const {
        if (s.found()) return;
        const int t = d.starget[r];
        float4 *L = t < 0 ? d.rL + (t & 0x7fffffff) : d.buf[nxt].L + t;
        const float4 c = d.scontrib[r], l = *L;
        *L = make_float4(l.x + c.x, l.y + c.y, l.z + c.z, l.w);
    }
};

// The server's path store for shade_segment: state read from queue cur at
// the entry index, continuing paths appended to queue cur ^ 1 (at the front
// for class 0, the back for class 1), finished ones to the retire list; a
// shadow ray records where its path went.
template <int kClass>
struct QueuePaths {
    const SrvDev &d;
    int cur;
    LJ_D void load(int i, PathState &st, float4 &r0, float4 &r1, float4 &hit) const {
        const StateSoA &q = d.buf[cur];
        st.slot = i;
        st.job = q.job[i];
        st.pixel = q.pixel[i];
        st.rng = q.rng[i];
        st.beta = q.beta[i];
        st.L = q.L[i];
        st.prev = q.prev[i];
        st.nv = q.nv[i];
        r0 = q.ray[2 * i];
        r1 = q.ray[2 * i + 1];
        hit = d.hit[i];
    }
    // the shadow ray's target is filled in by emit, once it is known
    LJ_D int shadow(const PathState &, float4 r0, float4 r1, float4 contrib) const {
        const int k = queue_slot(d.counts + 2);
        d.sray[2 * k] = r0;
        d.sray[2 * k + 1] = r1;
        d.scontrib[k] = contrib;
        return k;
    }
    LJ_D void emit(const PathState &st, const ShadeOut &o) const {
        int target;
        if (o.cont) {
            const int nxt = cur ^ 1;
            const StateSoA &q = d.buf[nxt];
            const int s = kClass == 0 ? queue_slot(d.counts + nxt) : d.back(queue_slot(d.counts + 10 + nxt));
            q.job[s] = st.job;
            q.pixel[s] = st.pixel;
            q.rng[s] = st.rng;
            q.beta[s] = st.beta;
            q.L[s] = st.L;
            q.prev[s] = st.prev;
            q.nv[s] = st.nv;
            q.ray[2 * s] = o.ray0;
            q.ray[2 * s + 1] = o.ray1;
            target = s;
        } else {
            const int r = queue_slot(d.counts + 3);
            d.rjob[r] = st.job;
            d.rpixel[r] = st.pixel;
            d.rL[r] = st.L;
            target = r | kRetireBit;
        }
        if (o.shadow >= 0) d.starget[o.shadow] = target;
    }
};

// traversal: 64 registers (full-SM occupancy of 50%); the per-ray scene
// lookup leaves no room for the packed child test's registers
template <int B>
__global__ void __launch_bounds__(B, 1024 / B) k_srv_trace(SrvDev d, int cur) {
    const int n0 = d.counts[cur], n01 = n0 + d.counts[10 + cur], n = n01 + d.counts[12 + cur];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(d.stats + 0, (unsigned long long)n);
    SrvClosestIO io{d, cur, n0, n01};
    trace_queue<false, B, false>(io, n, d.counts + 8, d.status);
}

// A path store whose entry was loaded before the step runs: the kernel loads
// the entry's state first and looks its job (and so its scene and options)
// up from the loaded job index, so the state loads and the job lookup are in
// flight together instead of one after the other.
template <class Paths>
struct PreloadedPaths {
    const Paths &p;
    const PathState &st;
    float4 r0, r1, hit;
    LJ_D void load(int, PathState &s, float4 &a, float4 &b, float4 &h) const {
        s = st;
        a = r0;
        b = r1;
        h = hit;
    }
    LJ_D int shadow(const PathState &s, float4 a, float4 b, float4 c) const { return p.shadow(s, a, b, c); }
    LJ_D void emit(const PathState &s, const ShadeOut &o) const { p.emit(s, o); }
};

// The scene and job tables are read-only here (restrict: the stores of the
// shade step cannot alias them, so their fields need not be re-read).
// One instance per material class: class 0 (the queue's front) runs the
// smaller kernel compiled for kClassicMats, with a branch of code compiled
// for Lambertian materials alone that the jobs whose materials are all
// Lambertian take (per lane: a job's paths always run the same branch,
// whichever other jobs share their warp).  The shade kernels run at
// kShadeBlock threads whatever the server's block size: class 0 at 5 blocks
// per SM (96 registers; at the 6 blocks of the single-scene classic kernel
// it spilled 3x the bytes with its second branch and ran 3 % slower, at 4
// it lost more warps than the spills cost), class 1 at 8 (64 registers: its
// Disney code waits on memory, and the warps gain more than the spills
// cost -- a terrain job's shading 16 % faster than at 5).  One compiled
// instance per class keeps a job's arithmetic -- and so its image --
// independent of the block size the other kernels use.
constexpr int kShadeBlock = 128;
template <int kClass>
__global__ void __launch_bounds__(kShadeBlock, kClass == 0 ? 5 : 8)
    k_srv_shade(SrvDev d, const DevScene *__restrict__ scenes, const SrvJob *__restrict__ jobs, int cur) {
    const int n = d.counts[kClass == 0 ? cur : 10 + cur];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(d.stats + 2, (unsigned long long)n);
    const QueuePaths<kClass> paths{d, cur};
    for (int i = blockIdx.x * kShadeBlock + threadIdx.x; i < n; i += gridDim.x * kShadeBlock) {
        const int e = kClass == 0 ? i : d.back(i);
        PathState st;
        float4 r0, r1, hit;
        paths.load(e, st, r0, r1, hit);
        const SrvJob &jb = jobs[st.job];
        const ShadeCfg cfg{jb.max_depth, jb.rr_depth, jb.spread0};
        const PreloadedPaths<QueuePaths<kClass>> pre{paths, st, r0, r1, hit};
        // a job always runs the same branch, whatever its warp shares
        if (kClass == 0 && jb.lambert) shade_segment<kLambertMats>(scenes[jb.scene], pre, e, cfg, d.status);
        else shade_segment<kClass == 0 ? kClassicMats : kAllMats>(scenes[jb.scene], pre, e, cfg, d.status);
    }
}

// The volumetric path store: state in queue order in the volpath queues;
// finished paths go to the retire list (radiance in rL.xyz).
struct VolQueueStore {
    const SrvDev &d;
    int cur;
    LJ_D void load(int i, VolState &vs, float4 &r0, float4 &r1, float4 &hit) const {
        const VolStateSoA &v = d.vbuf[cur];
        vs.slot = i;
        vs.job = v.job[i];
        vs.pixel = v.pixel[i];
        vs.rng = v.rng[i];
        vs.beta = v.beta[i];
        vs.L = v.L[i];
        vs.neep = v.neep[i];
        vs.mdir = v.mdir[i];
        vs.mnee = v.mnee[i];
        vs.st = v.st[i];
        r0 = v.ray[2 * i];
        r1 = v.ray[2 * i + 1];
        hit = d.vhit[i];
    }
    // state of a path that waits for its NEE request: kept in place (the c
    // step resets the NEE vertex and the pdf products, and takes the PCG
    // state from the request, so those stay behind)
    LJ_D void save(int i, const VolState &vs) const {
        const VolStateSoA &v = d.vbuf[cur];
        v.beta[i] = vs.beta;
        v.L[i] = vs.L;
        v.st[i] = vs.st;
    }
    LJ_D void load_c(int i, VolState &vs, float4 &r0, float4 &r1, float4 &hit) const {
        const VolStateSoA &v = d.vbuf[cur];
        vs.slot = i;
        vs.job = v.job[i];
        vs.pixel = v.pixel[i];
        vs.beta = v.beta[i];
        vs.L = v.L[i];
        vs.st = v.st[i];
        r0 = v.ray[2 * i];
        r1 = v.ray[2 * i + 1];
        hit = d.vhit[i];
    }
    LJ_D void emit(const VolState &vs, bool alive, float4 ray0, float4 ray1) const {
        if (alive) {
            const int nxt = cur ^ 1;
            const VolStateSoA &v = d.vbuf[nxt];
            const int s = queue_slot(d.counts + 12 + nxt);
            v.job[s] = vs.job;
            v.pixel[s] = vs.pixel;
            v.rng[s] = vs.rng;
            v.beta[s] = vs.beta;
            v.L[s] = vs.L;
            v.neep[s] = vs.neep;
            v.mdir[s] = vs.mdir;
            v.mnee[s] = vs.mnee;
            v.st[s] = vs.st;
            v.ray[2 * s] = ray0;
            v.ray[2 * s + 1] = ray1;
        } else {
            const int r = queue_slot(d.counts + 3);
            d.rjob[r] = vs.job;
            d.rpixel[r] = vs.pixel;
            d.rL[r] = vs.L;
        }
    }
};

// The volumetric store with the entry's state loaded up front (as
// PreloadedPaths): load returns it, the rest is the store's.
struct PreloadedVol {
    const VolQueueStore &p;
    const VolState &vs;
    float4 r0, r1, hit;
    LJ_D void load(int, VolState &s, float4 &a, float4 &b, float4 &h) const {
        s = vs;
        a = r0;
        b = r1;
        h = hit;
    }
    LJ_D void save(int i, const VolState &s) const { p.save(i, s); }
    LJ_D void emit(const VolState &s, bool alive, float4 a, float4 b) const { p.emit(s, alive, a, b); }
};

// Volumetric paths: the a / b / c steps of lj_volwave.cuh over the volpath
// queue and the wave's NEE requests.
template <int B>
__global__ void __launch_bounds__(B, 512 / B)
    k_srv_vol_a(SrvDev d, const DevScene *__restrict__ scenes, const SrvJob *__restrict__ jobs, int cur) {
    const int n = d.counts[12 + cur];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(d.stats + 3, (unsigned long long)n);
    const VolQueueStore store{d, cur};
    for (int i = blockIdx.x * B + threadIdx.x; i < n; i += gridDim.x * B) {
        VolState vs;
        float4 r0, r1, hit;
        store.load(i, vs, r0, r1, hit);
        const SrvJob &jb = jobs[vs.job];
        const ShadeCfg cfg{jb.max_depth, jb.rr_depth, jb.spread0};
        const PreloadedVol pre{store, vs, r0, r1, hit};
        vol_segment_a(scenes[jb.scene], pre, i, cfg, d.nee, d.status, d.stats + 4);
    }
}
template <int B>
__global__ void __launch_bounds__(B, 512 / B)
    k_srv_vol_b(SrvDev d, const DevScene *__restrict__ scenes, const SrvJob *__restrict__ jobs, int cur) {
    const int nf = d.counts[16], n = nf + d.counts[17];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(d.stats + 4, (unsigned long long)n);
    const VolQueueStore store{d, cur};
    for (int r = blockIdx.x * B + threadIdx.x; r < n; r += gridDim.x * B) {
        const int k = d.nee.req(r, nf);
        const SrvJob &jb = jobs[d.vbuf[cur].job[d.nee.entry[k]]];
        if (r < nf) {   // from a scattering point: its c step follows here (NeeToPhase)
            const ShadeCfg cfg{jb.max_depth, jb.rr_depth, jb.spread0};
            vol_nee_b(scenes[jb.scene], d.nee, k, jb.max_depth, d.status, d.stats + 5,
                      NeeToPhase<VolQueueStore>{scenes[jb.scene], store, d.nee, cfg});
        } else {
            vol_nee_b(scenes[jb.scene], d.nee, k, jb.max_depth, d.status, d.stats + 5, NeeToQueue{d.nee});
        }
    }
}
// The c step of the requests from surfaces, in two instances: kKind = 1 / 2
// for jobs whose materials are all in kClassicMats (smaller code) / the
// others.  (Requests from scattering points finish in k_srv_vol_b.)  At 64
// registers and full occupancy: its material code waits on memory, and the
// warps gain more than the spills cost (the serving step's volumetric time
// -9 % against 128 registers).
template <int B, int kKind>
__global__ void __launch_bounds__(B, 1024 / B)
    k_srv_vol_c(SrvDev d, const DevScene *__restrict__ scenes, const SrvJob *__restrict__ jobs, int cur) {
    const int n = d.counts[17];
    const VolQueueStore store{d, cur};
    for (int r = blockIdx.x * B + threadIdx.x; r < n; r += gridDim.x * B) {
        const int k = d.nee.cap - 1 - r;
        // the two instances share the request range: the job's material
        // class decides before any state is read
        const SrvJob &jb = jobs[d.vbuf[cur].job[d.nee.entry[k]]];
        if (jb.all_mats != kKind - 1) continue;
        const ShadeCfg cfg{jb.max_depth, jb.rr_depth, jb.spread0};
        vol_segment_c<kKind == 1 ? kClassicMats : kAllMats, true>(scenes[jb.scene], store, k, cfg, d.nee);
    }
}

template <int B>
__global__ void __launch_bounds__(B, 1024 / B) k_srv_shadow(SrvDev d, int cur) {
    const int n = d.counts[2];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(d.stats + 1, (unsigned long long)n);
    SrvShadowIO io{d, cur ^ 1};
    trace_queue<true, B>(io, n, d.counts + 9, d.status);
}

LJ_D unsigned long long to_fixed(float v, float clamp) {
    v = fminf(fmaxf(v, -clamp), clamp);
    return (unsigned long long)__float2ll_rn(v * 4294967296.0f);   // exact scaling by 2^32
}

template <int B>
__global__ void __launch_bounds__(B) k_srv_retire(SrvDev d) {
    const int n = d.counts[3];
    for (int i = blockIdx.x * B + threadIdx.x; i < n; i += gridDim.x * B) {
        const int j = d.rjob[i];
        const SrvJob &jb = d.jobs[j];
        const float4 L = d.rL[i];
        if (isfinite(L.x) && isfinite(L.y) && isfinite(L.z)) {
            // integer sums: the same totals in any order or layout
            unsigned long long *a = jb.accum + d.rpixel[i];
            const size_t np = (size_t)jb.npix;
            atomicAdd(a, to_fixed(L.x, jb.clamp));
            atomicAdd(a + np, to_fixed(L.y, jb.clamp));
            atomicAdd(a + 2 * np, to_fixed(L.z, jb.clamp));
        } else {
            atomicAdd(&d.ctr[j].dropped, 1ULL);
        }
        // one done-counter atomic per job per warp; most warps hold one job
        const unsigned active = __activemask();
        const int lead = __ffs(active) - 1;
        if (__all_sync(active, j == __shfl_sync(active, j, lead))) {
            if ((int)(threadIdx.x & 31u) == lead) atomicAdd(&d.ctr[j].done, (unsigned long long)__popc(active));
        } else {
            const unsigned same = __match_any_sync(active, j);
            if ((int)(threadIdx.x & 31u) == __ffs(same) - 1)
                atomicAdd(&d.ctr[j].done, (unsigned long long)__popc(same));
        }
    }
}

// n = 3 * npix: HWC image element i from plane i % 3, pixel i / 3
__global__ void k_srv_finalize(const unsigned long long *acc, float *img, long long n, double scale) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) img[i] = (float)((double)(long long)acc[(i % 3) * (n / 3) + i / 3] * scale);
}

struct KernelSet {
    void (*regen)(SrvDev, int);
    void (*trace)(SrvDev, int);
    void (*shade0)(SrvDev, const DevScene *, const SrvJob *, int);
    void (*shade1)(SrvDev, const DevScene *, const SrvJob *, int);
    void (*vol_a)(SrvDev, const DevScene *, const SrvJob *, int);
    void (*vol_b)(SrvDev, const DevScene *, const SrvJob *, int);
    void (*vol_c1)(SrvDev, const DevScene *, const SrvJob *, int);
    void (*vol_c2)(SrvDev, const DevScene *, const SrvJob *, int);
    void (*shadow)(SrvDev, int);
    void (*retire)(SrvDev);
};
template <int B>
KernelSet kernel_set() {
    return KernelSet{k_srv_regen<B>,      k_srv_trace<B>,       k_srv_shade<0>,       k_srv_shade<1>,
                     k_srv_vol_a<B>,      k_srv_vol_b<B>,       k_srv_vol_c<B, 1>,
                     k_srv_vol_c<B, 2>,   k_srv_shadow<B>,      k_srv_retire<B>};
}

int occupancy_grid(const void *fn, int block, int sms) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, 0);
    return std::max(1, sms * std::max(1, per_sm));
}

double now_ms(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

size_t pool_bytes(size_t P) {
    size_t b = 0;
    // two queue buffers: job, pixel, nv, rng, beta, L, prev, ray
    b += 2 * (align256(P * 4) * 3 + align256(P * 8) + align256(P * 16) * 3 + align256(P * 32));
    // hits; shadow rays, targets, contributions; retire job, pixel, radiance
    b += align256(P * 16) + align256(P * 32) + align256(P * 4) + align256(P * 16);
    b += align256(P * 4) * 2 + align256(P * 16);
    // two volpath queue buffers: job, pixel, rng, beta, L, neep, mdir, mnee, st, ray; volpath hits
    b += 2 * (align256(P * 4) * 2 + align256(P * 8) + align256(P * 16) * 6 + align256(P * 32)) + align256(P * 16);
    // NEE requests: entry; org, dir, lp, ln, ss, T, pn, pd, med; rng
    b += align256(P * 4) + 9 * align256(P * 16) + align256(P * 8);
    b += 256 * 2;   // counts, stats
    return b;
}

template <typename T>
T *carve(char *&p, size_t n) {
    T *r = (T *)p;
    p += align256(n * sizeof(T));
    return r;
}

}  // namespace
}  // namespace lj

using namespace lj;

struct HostJob {
    int64_t id = 0;
    lj_scene *scene = nullptr;
    int scene_slot = -1;
    int w = 0, h = 0, spp = 0, sample_offset = 0, max_depth = 0, rr_depth = 0;
    uint64_t seed = 0;
    int64_t total = 0;
    int64_t bytes = 0;
    int slot = -1;
    int state = LJ_JOB_QUEUED;
    int error = 0;
    bool cancel_req = false, cancel_sent = false, finishing = false;
    // counter read-backs enqueued before these sequence numbers predate the
    // job's admission (stale counters of the slot) or its cancel flag
    int64_t admit_seq = 0, cancel_seq = 0;
    unsigned long long *d_accum = nullptr;
    float *d_img = nullptr;
    float *h_img = nullptr;      // pinned, from the server's pool
    size_t h_img_cap = 0;        // its size class in bytes
    cudaEvent_t done_ev = nullptr;
    int64_t samples_done = 0, dropped = 0;
    double t_submit = 0, t_admit = 0, t_finish = 0;
};

struct lj_server {
    lj_ctx *ctx = nullptr;
    int device = 0;
    lj_server_options opt{};
    int block = 128;
    int64_t P = 0;
    cudaStream_t stream = nullptr;
    cudaMemPool_t mempool = nullptr;
    std::chrono::steady_clock::time_point t0;

    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stopping = false;
    std::chrono::steady_clock::time_point stop_time;
    bool dead = false;          // the worker hit a CUDA error
    std::string last_error;

    std::vector<lj_scene *> scenes;            // scene slot -> scene
    std::unordered_map<int64_t, std::unique_ptr<HostJob>> jobs;
    // pinned image buffers by size class, reused: freeing pinned memory
    // synchronizes the device, allocating it is slow
    std::multimap<size_t, float *> pinned_free;
    std::deque<HostJob *> pending;
    std::vector<HostJob *> live;               // job slot -> job
    std::vector<int> free_slots;
    std::vector<int> order;                    // job slots in scheduling order (worker only)
    int64_t next_id = 1;
    int64_t bytes_pool = 0, bytes_scenes = 0, bytes_jobs = 0;

    // device
    void *d_pool = nullptr;
    DevScene *d_scenes = nullptr;
    SrvJob *d_jobs = nullptr;
    SrvCtr *d_ctr = nullptr;
    int *d_cancel = nullptr;
    int *d_order = nullptr;
    int *d_plan_off = nullptr;
    int *d_plan_coff = nullptr;
    long long *d_plan_start = nullptr;
    SrvDev dev{};
    KernelSet ks{};
    int grid[11] = {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1};
    cudaGraphExec_t graph = nullptr;

    // pinned host staging
    SrvJob *h_jobs = nullptr;                  // one staging entry per job slot
    int *h_order[2] = {nullptr, nullptr};
    cudaEvent_t order_ev[2] = {nullptr, nullptr};
    int order_buf = 0;
    int *h_one = nullptr;                      // constant 1 (cancel flag source)
    SrvCtr *h_ctr[kPollsInFlight] = {nullptr, nullptr};
    cudaEvent_t poll_ev[kPollsInFlight] = {nullptr, nullptr};
    bool poll_pending[kPollsInFlight] = {false, false};
    int64_t poll_seq[kPollsInFlight] = {0, 0};
    int64_t next_poll_seq = 1;
    int poll_next = 0;

    unsigned long long *h_qstats[kPollsInFlight] = {nullptr, nullptr};   // device counters (kStatWords)

    // LJ_SERVER_PROFILE: an event pair around every kernel of a batch
    bool profile = false;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
    size_t n_marks = 0;

    // stats
    int64_t n_submitted = 0, n_done = 0, n_failed = 0, n_cancelled = 0;
    int64_t waves = 0, graph_launches = 0, samples_done = 0, kernel_launches = 0;
    unsigned long long counters[kStatWords] = {};   // device counters as of the last read-back
    double class_ms[LJ_KERNEL_CLASSES] = {};
    int64_t class_launches[LJ_KERNEL_CLASSES] = {};
    double busy_ms = 0;
};

namespace {

int srv_error(lj_server *s, int code, const std::string &msg) {
    s->last_error = msg;
    return code;
}

#define SRV_CUDA(expr)                                                                      \
    do {                                                                                    \
        cudaError_t _e = (expr);                                                            \
        if (_e != cudaSuccess) return std::string(#expr) + ": " + cudaGetErrorString(_e);   \
    } while (0)

void mark(lj_server *s, int cls, bool begin) {
    if (!s->profile) return;
    if (begin) {
        if (s->n_marks == s->marks.size()) {
            cudaEvent_t a, b;
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            s->marks.push_back({cls, {a, b}});
        }
        s->marks[s->n_marks].first = cls;
        cudaEventRecord(s->marks[s->n_marks].second.first, s->stream);
    } else {
        cudaEventRecord(s->marks[s->n_marks].second.second, s->stream);
        s->class_launches[cls]++;
        s->n_marks++;
    }
}

// Launch one wave (cur -> cur ^ 1) on the server stream.
void launch_wave(lj_server *s, int cur) {
    const int B = s->block;
    mark(s, LJ_KERNEL_OTHER, true);
    k_srv_plan<<<1, 32, 0, s->stream>>>(s->dev, cur);
    mark(s, LJ_KERNEL_OTHER, false);
    mark(s, LJ_KERNEL_CAMERA, true);
    s->ks.regen<<<s->grid[0], B, 0, s->stream>>>(s->dev, cur);
    mark(s, LJ_KERNEL_CAMERA, false);
    mark(s, LJ_KERNEL_TRACE, true);
    s->ks.trace<<<s->grid[1], B, 0, s->stream>>>(s->dev, cur);
    mark(s, LJ_KERNEL_TRACE, false);
    mark(s, LJ_KERNEL_SHADE, true);
    s->ks.shade0<<<s->grid[2], kShadeBlock, 0, s->stream>>>(s->dev, s->d_scenes, s->d_jobs, cur);
    mark(s, LJ_KERNEL_SHADE, false);
    mark(s, LJ_KERNEL_SHADE, true);
    s->ks.shade1<<<s->grid[5], kShadeBlock, 0, s->stream>>>(s->dev, s->d_scenes, s->d_jobs, cur);
    mark(s, LJ_KERNEL_SHADE, false);
    mark(s, LJ_KERNEL_MEDIUM, true);
    s->ks.vol_a<<<s->grid[6], B, 0, s->stream>>>(s->dev, s->d_scenes, s->d_jobs, cur);
    mark(s, LJ_KERNEL_MEDIUM, false);
    mark(s, LJ_KERNEL_NEE, true);
    s->ks.vol_b<<<s->grid[7], B, 0, s->stream>>>(s->dev, s->d_scenes, s->d_jobs, cur);
    mark(s, LJ_KERNEL_NEE, false);
    mark(s, LJ_KERNEL_MEDIUM, true);
    s->ks.vol_c1<<<s->grid[9], B, 0, s->stream>>>(s->dev, s->d_scenes, s->d_jobs, cur);
    mark(s, LJ_KERNEL_MEDIUM, false);
    mark(s, LJ_KERNEL_MEDIUM, true);
    s->ks.vol_c2<<<s->grid[10], B, 0, s->stream>>>(s->dev, s->d_scenes, s->d_jobs, cur);
    mark(s, LJ_KERNEL_MEDIUM, false);
    mark(s, LJ_KERNEL_SHADOW, true);
    s->ks.shadow<<<s->grid[3], B, 0, s->stream>>>(s->dev, cur);
    mark(s, LJ_KERNEL_SHADOW, false);
    mark(s, LJ_KERNEL_OTHER, true);
    s->ks.retire<<<s->grid[4], B, 0, s->stream>>>(s->dev);
    mark(s, LJ_KERNEL_OTHER, false);
}

// LJ_SERVER_PROFILE: wait for the batch and add up its kernel times.
cudaError_t collect_marks(lj_server *s) {
    if (!s->profile || s->n_marks == 0) return cudaSuccess;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    for (size_t k = 0; k < s->n_marks && e == cudaSuccess; k++) {
        float ms = 0;
        e = cudaEventElapsedTime(&ms, s->marks[k].second.first, s->marks[k].second.second);
        s->class_ms[s->marks[k].first] += ms;
    }
    s->n_marks = 0;
    return e;
}

std::string build_device(lj_server *s) {
    SRV_CUDA(cudaSetDevice(s->device));
    SRV_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = s->device;
    SRV_CUDA(cudaMemPoolCreate(&s->mempool, &props));
    uint64_t keep = UINT64_MAX;
    SRV_CUDA(cudaMemPoolSetAttribute(s->mempool, cudaMemPoolAttrReleaseThreshold, &keep));

    const int64_t P = s->P;
    const int J = s->opt.max_live_jobs;
    size_t pb = pool_bytes((size_t)P);
    SRV_CUDA(cudaMalloc(&s->d_pool, pb));
    s->bytes_pool = (int64_t)pb;
    SRV_CUDA(cudaMalloc(&s->d_scenes, sizeof(DevScene) * kMaxScenes));
    SRV_CUDA(cudaMalloc(&s->d_jobs, sizeof(SrvJob) * J));
    SRV_CUDA(cudaMalloc(&s->d_ctr, sizeof(SrvCtr) * J));
    SRV_CUDA(cudaMalloc(&s->d_cancel, sizeof(int) * J));
    SRV_CUDA(cudaMalloc(&s->d_order, sizeof(int) * (J + 1)));
    SRV_CUDA(cudaMalloc(&s->d_plan_off, sizeof(int) * (J + 1)));
    SRV_CUDA(cudaMalloc(&s->d_plan_coff, sizeof(int) * (J + 1)));
    SRV_CUDA(cudaMalloc(&s->d_plan_start, sizeof(long long) * (J + 1)));
    SRV_CUDA(cudaMemsetAsync(s->d_ctr, 0, sizeof(SrvCtr) * J, s->stream));
    SRV_CUDA(cudaMemsetAsync(s->d_cancel, 0, sizeof(int) * J, s->stream));
    SRV_CUDA(cudaMemsetAsync(s->d_order, 0, sizeof(int) * (J + 1), s->stream));
    s->bytes_pool += (int64_t)(sizeof(DevScene) * kMaxScenes + (sizeof(SrvJob) + sizeof(SrvCtr) + 16) * J);

    SRV_CUDA(cudaMallocHost(&s->h_jobs, sizeof(SrvJob) * J));
    for (int b = 0; b < 2; b++) {
        SRV_CUDA(cudaMallocHost(&s->h_order[b], sizeof(int) * (J + 1)));
        SRV_CUDA(cudaEventCreateWithFlags(&s->order_ev[b], cudaEventDisableTiming));
    }
    SRV_CUDA(cudaMallocHost(&s->h_one, sizeof(int)));
    *s->h_one = 1;
    for (int b = 0; b < kPollsInFlight; b++) {
        SRV_CUDA(cudaMallocHost(&s->h_ctr[b], sizeof(SrvCtr) * J));
        SRV_CUDA(cudaMallocHost(&s->h_qstats[b], sizeof(unsigned long long) * kStatWords));
        memset(s->h_qstats[b], 0, sizeof(unsigned long long) * kStatWords);
        SRV_CUDA(cudaEventCreateWithFlags(&s->poll_ev[b], cudaEventDisableTiming));
    }

    char *cur = (char *)s->d_pool;
    SrvDev &d = s->dev;
    d.scenes = s->d_scenes;
    d.jobs = s->d_jobs;
    d.ctr = s->d_ctr;
    d.cancel = s->d_cancel;
    d.order = s->d_order;
    d.plan_off = s->d_plan_off;
    d.plan_coff = s->d_plan_coff;
    d.plan_start = s->d_plan_start;
    for (int k = 0; k < 2; k++) {
        StateSoA &q = d.buf[k];
        q.job = carve<int>(cur, P);
        q.pixel = carve<int>(cur, P);
        q.nv = carve<int>(cur, P);
        q.rng = carve<uint64_t>(cur, P);
        q.beta = carve<float4>(cur, P);
        q.L = carve<float4>(cur, P);
        q.prev = carve<float4>(cur, P);
        q.ray = carve<float4>(cur, 2 * P);
    }
    d.hit = carve<float4>(cur, P);
    for (int k = 0; k < 2; k++) {
        VolStateSoA &v = d.vbuf[k];
        v.job = carve<int>(cur, P);
        v.pixel = carve<int>(cur, P);
        v.rng = carve<uint64_t>(cur, P);
        v.beta = carve<float4>(cur, P);
        v.L = carve<float4>(cur, P);
        v.neep = carve<float4>(cur, P);
        v.mdir = carve<float4>(cur, P);
        v.mnee = carve<float4>(cur, P);
        v.st = carve<int4>(cur, P);
        v.ray = carve<float4>(cur, 2 * P);
    }
    d.vhit = carve<float4>(cur, P);
    d.nee.cap = (int)P;
    d.nee.entry = carve<int>(cur, P);
    d.nee.org = carve<float4>(cur, P);
    d.nee.dir = carve<float4>(cur, P);
    d.nee.lp = carve<float4>(cur, P);
    d.nee.ln = carve<float4>(cur, P);
    d.nee.ss = carve<float4>(cur, P);
    d.nee.T = carve<float4>(cur, P);
    d.nee.pn = carve<float4>(cur, P);
    d.nee.pd = carve<float4>(cur, P);
    d.nee.med = carve<int4>(cur, P);
    d.nee.rng = carve<uint64_t>(cur, P);
    d.sray = carve<float4>(cur, 2 * P);
    d.starget = carve<int>(cur, P);
    d.scontrib = carve<float4>(cur, P);
    d.rjob = carve<int>(cur, P);
    d.rpixel = carve<int>(cur, P);
    d.rL = carve<float4>(cur, P);
    d.counts = carve<int>(cur, 64);
    d.nee.count = d.counts + 16;
    d.stats = carve<unsigned long long>(cur, 32);
    d.P = (int)P;
    d.status = s->ctx->d_status;
    SRV_CUDA(cudaMemsetAsync(d.stats, 0, 32 * sizeof(unsigned long long), s->stream));
    SRV_CUDA(cudaMemsetAsync(d.counts, 0, 64 * sizeof(int), s->stream));

    switch (s->block) {
    case 64: s->ks = kernel_set<64>(); break;
    case 256: s->ks = kernel_set<256>(); break;
    default: s->ks = kernel_set<128>(); break;
    }
    int sms = 0;
    SRV_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device));
    s->grid[0] = occupancy_grid((const void *)s->ks.regen, s->block, sms);
    s->grid[1] = occupancy_grid((const void *)s->ks.trace, s->block, sms);
    s->grid[2] = occupancy_grid((const void *)s->ks.shade0, kShadeBlock, sms);
    s->grid[5] = occupancy_grid((const void *)s->ks.shade1, kShadeBlock, sms);
    s->grid[6] = occupancy_grid((const void *)s->ks.vol_a, s->block, sms);
    s->grid[7] = occupancy_grid((const void *)s->ks.vol_b, s->block, sms);
    s->grid[9] = occupancy_grid((const void *)s->ks.vol_c1, s->block, sms);
    s->grid[10] = occupancy_grid((const void *)s->ks.vol_c2, s->block, sms);
    s->grid[3] = occupancy_grid((const void *)s->ks.shadow, s->block, sms);
    s->grid[4] = occupancy_grid((const void *)s->ks.retire, s->block, sms);

    s->profile = (s->opt.flags & LJ_SERVER_PROFILE) != 0;
    if (s->opt.use_graphs && !s->profile) {
        cudaGraph_t g = nullptr;
        SRV_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        launch_wave(s, 0);
        launch_wave(s, 1);
        SRV_CUDA(cudaStreamEndCapture(s->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&s->graph, g, 0);
        cudaGraphDestroy(g);
        SRV_CUDA(e);
    }
    SRV_CUDA(cudaStreamSynchronize(s->stream));
    return "";
}

// ---- worker-thread helpers (called with s->mu held unless noted) ----------

std::string push_order(lj_server *s) {
    int b = s->order_buf;
    s->order_buf ^= 1;
    SRV_CUDA(cudaEventSynchronize(s->order_ev[b]));   // the copy from two updates ago
    int *h = s->h_order[b];
    h[0] = (int)s->order.size();
    for (size_t k = 0; k < s->order.size(); k++) h[1 + k] = s->order[k];
    SRV_CUDA(cudaMemcpyAsync(s->d_order, h, sizeof(int) * (s->order.size() + 1), cudaMemcpyHostToDevice,
                             s->stream));
    SRV_CUDA(cudaEventRecord(s->order_ev[b], s->stream));
    return "";
}

void sort_order(lj_server *s) {
    if (s->opt.policy != LJ_SCHED_SRPT) return;   // FIFO: admission order
    std::stable_sort(s->order.begin(), s->order.end(), [&](int a, int b) {
        const HostJob *ja = s->live[a], *jb = s->live[b];
        return ja->total - ja->samples_done < jb->total - jb->samples_done;
    });
}

std::string admit(lj_server *s, HostJob *j) {
    int slot = s->free_slots.back();
    s->free_slots.pop_back();
    j->slot = slot;
    s->live[slot] = j;
    const size_t npix = (size_t)j->w * j->h;
    SRV_CUDA(cudaMallocFromPoolAsync((void **)&j->d_accum, npix * 3 * 8, s->mempool, s->stream));
    SRV_CUDA(cudaMallocFromPoolAsync((void **)&j->d_img, npix * 3 * 4, s->mempool, s->stream));
    SRV_CUDA(cudaMemsetAsync(j->d_accum, 0, npix * 3 * 8, s->stream));
    SrvJob &h = s->h_jobs[slot];
    memset(&h, 0, sizeof(h));
    make_cam_rec(j->scene->camera, j->w, j->h, h.cam);
    h.seed = j->seed;
    h.total = j->total;
    h.accum = j->d_accum;
    h.scene = j->scene_slot;
    h.bvh = j->scene->dev.bvh;   // a served scene's BVH does not change (updates refused)
    h.npix = (int)npix;
    h.spp = j->spp;
    h.sample_offset = j->sample_offset;
    h.max_depth = j->max_depth;
    h.rr_depth = j->rr_depth;
    h.spread0 = 0.25f / (float)std::max(j->w, j->h);
    h.clamp = (float)std::ldexp(1.0, 30) / (float)j->spp;
    const bool classic = (j->scene->mat_mask & ~kClassicMats) == 0 && !(s->opt.flags & LJ_SERVER_ONE_SHADE_KERNEL);
    if (j->scene->options.integrator == LJ_INTEGRATOR_VOLPATH) h.mclass = 2;
    else h.mclass = classic ? 0 : 1;
    h.all_mats = classic ? 0 : 1;
    h.lambert = classic && (j->scene->mat_mask & ~kLambertMats) == 0;
    SRV_CUDA(cudaMemcpyAsync(s->d_jobs + slot, &h, sizeof(SrvJob), cudaMemcpyHostToDevice, s->stream));
    SRV_CUDA(cudaMemsetAsync(s->d_ctr + slot, 0, sizeof(SrvCtr), s->stream));
    SRV_CUDA(cudaMemsetAsync(s->d_cancel + slot, 0, sizeof(int), s->stream));
    j->state = LJ_JOB_RUNNING;
    j->t_admit = now_ms(s->t0);
    j->admit_seq = s->next_poll_seq;
    s->bytes_jobs += j->bytes;
    s->order.push_back(slot);
    return "";
}

// Start finishing a job whose paths have all retired.
std::string finish(lj_server *s, HostJob *j) {
    const long long n = (long long)j->w * j->h * 3;
    const bool cancelled = j->cancel_req;
    if (!cancelled) {
        k_srv_finalize<<<(int)((n + 255) / 256), 256, 0, s->stream>>>(j->d_accum, j->d_img, n,
                                                                       std::ldexp(1.0, -32) / j->spp);
        SRV_CUDA(cudaGetLastError());
        s->kernel_launches++;
        size_t cap = 1 << 16;
        while (cap < sizeof(float) * (size_t)n) cap <<= 1;
        auto it = s->pinned_free.find(cap);
        if (it != s->pinned_free.end()) {
            j->h_img = it->second;
            s->pinned_free.erase(it);
        } else {
            SRV_CUDA(cudaMallocHost(&j->h_img, cap));
        }
        j->h_img_cap = cap;
        SRV_CUDA(cudaMemcpyAsync(j->h_img, j->d_img, sizeof(float) * n, cudaMemcpyDeviceToHost, s->stream));
    }
    SRV_CUDA(cudaFreeAsync(j->d_accum, s->stream));
    SRV_CUDA(cudaFreeAsync(j->d_img, s->stream));
    j->d_accum = nullptr;
    j->d_img = nullptr;
    SRV_CUDA(cudaEventCreateWithFlags(&j->done_ev, cudaEventDisableTiming));
    SRV_CUDA(cudaEventRecord(j->done_ev, s->stream));
    j->finishing = true;
    s->order.erase(std::remove(s->order.begin(), s->order.end(), j->slot), s->order.end());
    return "";
}

bool fits(lj_server *s, const HostJob *j) {
    return s->bytes_pool + s->bytes_scenes + s->bytes_jobs + j->bytes <= s->opt.hbm_budget_bytes;
}

void fail_all(lj_server *s, const std::string &msg) {
    s->dead = true;
    s->last_error = msg;
    for (auto &kv : s->jobs) {
        HostJob *j = kv.second.get();
        if (j->state == LJ_JOB_QUEUED || j->state == LJ_JOB_RUNNING) {
            j->state = LJ_JOB_FAILED;
            j->error = LJ_ERR_CUDA;
            s->n_failed++;
        }
    }
    s->pending.clear();
    s->cv_done.notify_all();
}

// Process one counter read-back (sequence number seq): update progress,
// start finishing jobs whose paths have all retired.
std::string on_snapshot(lj_server *s, const SrvCtr *snap, int64_t seq) {
    bool changed = false;
    for (int slot = 0; slot < (int)s->live.size(); slot++) {
        HostJob *j = s->live[slot];
        if (!j || j->finishing || seq < j->admit_seq) continue;
        const SrvCtr &c = snap[slot];
        j->samples_done = (int64_t)c.done;
        j->dropped = (int64_t)c.dropped;
        const bool complete = j->cancel_sent ? (seq >= j->cancel_seq && c.done == c.issued)
                                             : (int64_t)c.done == j->total;
        if (complete) {
            std::string e = finish(s, j);
            if (!e.empty()) return e;
            changed = true;
        } else if ((int64_t)c.issued >= j->total) {
            // nothing left to issue: keep it out of the plan's order list
            auto it = std::find(s->order.begin(), s->order.end(), slot);
            if (it != s->order.end()) {
                s->order.erase(it);
                changed = true;
            }
        }
    }
    if (s->opt.policy == LJ_SCHED_SRPT && s->order.size() > 1) {
        sort_order(s);
        changed = true;
    }
    if (changed) return push_order(s);
    return "";
}

void reap_finished(lj_server *s) {
    for (int slot = 0; slot < (int)s->live.size(); slot++) {
        HostJob *j = s->live[slot];
        if (!j || !j->finishing) continue;
        if (cudaEventQuery(j->done_ev) != cudaSuccess) continue;
        cudaEventDestroy(j->done_ev);
        j->done_ev = nullptr;
        j->finishing = false;
        j->t_finish = now_ms(s->t0);
        if (j->cancel_req) {
            j->state = LJ_JOB_CANCELLED;
            s->n_cancelled++;
        } else {
            j->state = LJ_JOB_DONE;
            j->samples_done = j->total;
            s->n_done++;
        }
        s->samples_done += j->samples_done;
        s->bytes_jobs -= j->bytes;
        s->live[slot] = nullptr;
        s->free_slots.push_back(slot);
        j->slot = -1;
    }
    s->cv_done.notify_all();
}

bool any_live(lj_server *s) {
    for (HostJob *j : s->live)
        if (j) return true;
    return false;
}

void worker_main(lj_server *s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    auto t_busy = std::chrono::steady_clock::now();
    bool busy = false;
    while (true) {
        std::string err;
        // admissions (FIFO over the pending queue, under the budget)
        bool order_changed = false;
        while (!s->pending.empty() && !s->free_slots.empty()) {
            HostJob *j = s->pending.front();
            if (j->cancel_req) {
                s->pending.pop_front();
                j->state = LJ_JOB_CANCELLED;
                j->t_finish = now_ms(s->t0);
                s->n_cancelled++;
                s->cv_done.notify_all();
                continue;
            }
            if (!fits(s, j)) break;
            s->pending.pop_front();
            err = admit(s, j);
            if (!err.empty()) break;
            order_changed = true;
        }
        // cancellations of running jobs
        for (HostJob *j : s->live) {
            if (!err.empty()) break;
            if (j && j->cancel_req && !j->cancel_sent) {
                cudaError_t e = cudaMemcpyAsync(s->d_cancel + j->slot, s->h_one, sizeof(int),
                                                cudaMemcpyHostToDevice, s->stream);
                if (e != cudaSuccess) err = std::string("cancel: ") + cudaGetErrorString(e);
                j->cancel_sent = true;
                j->cancel_seq = s->next_poll_seq;
            }
        }
        if (err.empty() && order_changed) {
            sort_order(s);
            err = push_order(s);
        }
        if (!err.empty()) {
            fail_all(s, err);
            break;
        }
        const bool live = any_live(s);
        if (live && s->stopping &&
            std::chrono::steady_clock::now() - s->stop_time > std::chrono::seconds(60)) {
            fail_all(s, "stop: cancelled jobs did not drain within 60 s");
            break;
        }
        if (!live) {
            if (busy) {
                s->busy_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_busy).count();
                busy = false;
            }
            if (s->stopping) break;
            s->cv_work.wait_for(lk, std::chrono::milliseconds(50));
            continue;
        }
        if (!busy) {
            busy = true;
            t_busy = std::chrono::steady_clock::now();
        }
        // launch a batch of waves, then a counter read-back
        const int pairs = std::max(1, s->opt.waves_per_poll / 2);
        lk.unlock();
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < pairs && e == cudaSuccess; k++) {
            if (s->graph) {
                e = cudaGraphLaunch(s->graph, s->stream);
            } else {
                launch_wave(s, 0);
                launch_wave(s, 1);
                e = cudaGetLastError();
            }
        }
        if (e == cudaSuccess) e = collect_marks(s);
        lk.lock();
        s->waves += 2 * pairs;
        s->kernel_launches += 22 * pairs;
        if (s->graph) s->graph_launches += pairs;
        const int b = s->poll_next;
        s->poll_next = (b + 1) % kPollsInFlight;
        if (e == cudaSuccess && s->poll_pending[b]) {
            // the read-back issued kPollsInFlight batches ago
            lk.unlock();
            e = cudaEventSynchronize(s->poll_ev[b]);
            lk.lock();
            if (e == cudaSuccess) {
                s->poll_pending[b] = false;
                memcpy(s->counters, s->h_qstats[b], sizeof(s->counters));
                err = on_snapshot(s, s->h_ctr[b], s->poll_seq[b]);
            }
        }
        if (e == cudaSuccess && err.empty()) {
            e = cudaMemcpyAsync(s->h_ctr[b], s->d_ctr, sizeof(SrvCtr) * s->live.size(), cudaMemcpyDeviceToHost,
                                s->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(s->h_qstats[b], s->dev.stats, sizeof(unsigned long long) * kStatWords,
                                    cudaMemcpyDeviceToHost, s->stream);
            if (e == cudaSuccess) e = cudaEventRecord(s->poll_ev[b], s->stream);
            if (e == cudaSuccess) {
                s->poll_pending[b] = true;
                s->poll_seq[b] = s->next_poll_seq++;
            }
        }
        if (e == cudaSuccess && err.empty()) reap_finished(s);
        if (e != cudaSuccess) err = std::string("server: ") + cudaGetErrorString(e);
        if (!err.empty()) {
            fail_all(s, err);
            break;
        }
    }
    // drain: nothing of ours may still run when buffers are freed
    lk.unlock();
    cudaStreamSynchronize(s->stream);
    unsigned long long q[kStatWords] = {};
    bool got = !s->dead && cudaMemcpy(q, s->dev.stats, sizeof(q), cudaMemcpyDeviceToHost) == cudaSuccess;
    lk.lock();
    if (got) memcpy(s->counters, q, sizeof(q));
    reap_finished(s);
    s->cv_done.notify_all();
}

HostJob *find_job(lj_server *s, int64_t id) {
    auto it = s->jobs.find(id);
    return it == s->jobs.end() ? nullptr : it->second.get();
}

void fill_status(const HostJob *j, lj_job_status *st) {
    if (!st) return;
    st->state = j->state;
    st->error = j->error;
    st->width = j->w;
    st->height = j->h;
    st->samples_total = j->total;
    st->samples_done = j->samples_done;
    st->samples_dropped = j->dropped;
    st->submit_ms = j->t_submit;
    st->admit_ms = j->t_admit;
    st->finish_ms = j->t_finish;
}

void release_device(lj_server *s) {
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (auto &kv : s->jobs) {
        HostJob *j = kv.second.get();
        if (j->d_accum) cudaFree(j->d_accum);
        if (j->d_img) cudaFree(j->d_img);
        if (j->h_img) cudaFreeHost(j->h_img);
        if (j->done_ev) cudaEventDestroy(j->done_ev);
        j->d_accum = nullptr;
        j->d_img = nullptr;
        j->h_img = nullptr;
    }
    for (auto &kv : s->pinned_free) cudaFreeHost(kv.second);
    s->pinned_free.clear();
    if (s->graph) cudaGraphExecDestroy(s->graph);
    void *dev_ptrs[] = {s->d_pool, s->d_scenes, s->d_jobs, s->d_ctr, s->d_cancel, s->d_order, s->d_plan_off,
                        s->d_plan_coff, s->d_plan_start};
    for (void *p : dev_ptrs)
        if (p) cudaFree(p);
    if (s->h_jobs) cudaFreeHost(s->h_jobs);
    for (int b = 0; b < 2; b++) {
        if (s->h_order[b]) cudaFreeHost(s->h_order[b]);
        if (s->order_ev[b]) cudaEventDestroy(s->order_ev[b]);
    }
    if (s->h_one) cudaFreeHost(s->h_one);
    for (auto &m : s->marks) {
        cudaEventDestroy(m.second.first);
        cudaEventDestroy(m.second.second);
    }
    s->marks.clear();
    for (int b = 0; b < kPollsInFlight; b++) {
        if (s->h_qstats[b]) cudaFreeHost(s->h_qstats[b]);
        if (s->h_ctr[b]) cudaFreeHost(s->h_ctr[b]);
        if (s->poll_ev[b]) cudaEventDestroy(s->poll_ev[b]);
    }
    if (s->mempool) cudaMemPoolDestroy(s->mempool);
    if (s->stream) cudaStreamDestroy(s->stream);
    for (lj_scene *sc : s->scenes) sc->server_refs--;
    s->scenes.clear();
}

}  // namespace

extern "C" {

int lj_gpu_server_start(lj_ctx *ctx, const lj_server_options *options, lj_server **out) {
    if (!ctx || !out) return LJ_ERR_INVALID_ARG;
    *out = nullptr;
    lj_server_options o{};
    if (options) o = *options;
    if (o.hbm_budget_bytes <= 0) o.hbm_budget_bytes = (int64_t)120 << 30;
    if (o.path_pool <= 0) o.path_pool = (int64_t)1 << 22;
    if (o.block_size == 0) o.block_size = 128;
    if (o.max_live_jobs <= 0) o.max_live_jobs = 256;
    if (o.max_queued_jobs <= 0) o.max_queued_jobs = 65536;
    if (o.waves_per_poll <= 0) o.waves_per_poll = 8;
    if (o.block_size != 64 && o.block_size != 128 && o.block_size != 256)
        return set_error(ctx, LJ_ERR_INVALID_ARG, "server: block_size must be 64, 128 or 256");
    if (o.path_pool > ((int64_t)1 << 28) || o.max_live_jobs > 4096)
        return set_error(ctx, LJ_ERR_INVALID_ARG, "server: path_pool <= 2^28 and max_live_jobs <= 4096");
    if (o.policy != LJ_SCHED_FIFO && o.policy != LJ_SCHED_SRPT)
        return set_error(ctx, LJ_ERR_INVALID_ARG, "server: unknown policy");
    lj_server *s = new (std::nothrow) lj_server();
    if (!s) return set_error(ctx, LJ_ERR_OUT_OF_MEMORY, "server: host allocation failed");
    s->ctx = ctx;
    s->device = ctx->device;
    s->opt = o;
    s->block = o.block_size;
    s->P = o.path_pool;
    s->t0 = std::chrono::steady_clock::now();
    s->live.assign(o.max_live_jobs, nullptr);
    for (int k = o.max_live_jobs - 1; k >= 0; k--) s->free_slots.push_back(k);
    if ((int64_t)pool_bytes((size_t)s->P) > o.hbm_budget_bytes) {
        delete s;
        return set_error(ctx, LJ_ERR_OUT_OF_MEMORY, "server: the path pool alone exceeds the HBM budget");
    }
    std::string e = build_device(s);
    if (!e.empty()) {
        cudaGetLastError();
        release_device(s);
        delete s;
        return set_error(ctx, e.find("memory") != std::string::npos ? LJ_ERR_OUT_OF_MEMORY : LJ_ERR_CUDA,
                         "server: " + e);
    }
    s->worker = std::thread(worker_main, s);
    ctx->servers.push_back(s);
    *out = s;
    return LJ_OK;
}

int lj_gpu_server_submit(lj_server *s, lj_scene *scene, const lj_job_desc *job, int64_t *job_id) {
    if (!s || !scene || !job || !job_id) return LJ_ERR_INVALID_ARG;
    if (scene->ctx != s->ctx) return srv_error(s, LJ_ERR_INVALID_ARG, "submit: scene of another context");
    if (scene->options.integrator != LJ_INTEGRATOR_PATH &&
        !(scene->options.integrator == LJ_INTEGRATOR_VOLPATH &&
          (scene->options.vol_path_version == 0 || scene->options.vol_path_version == 6)))
        return srv_error(s, LJ_ERR_UNSUPPORTED, "submit: the server renders path and volpath (v6) scenes only");
    if (job->spp < 0 || job->width < 0 || job->height < 0 || (job->width > 0) != (job->height > 0))
        return srv_error(s, LJ_ERR_INVALID_ARG, "submit: negative spp / size, or only one of width and height");
    auto j = std::make_unique<HostJob>();
    j->scene = scene;
    j->w = job->width > 0 ? job->width : scene->width;
    j->h = job->height > 0 ? job->height : scene->height;
    j->spp = job->spp > 0 ? job->spp : scene->options.samples_per_pixel;
    j->sample_offset = job->sample_offset;
    j->seed = job->seed;
    j->max_depth = job->override_depth ? job->max_depth : scene->options.max_depth;
    j->rr_depth = job->override_depth ? job->rr_depth : scene->options.rr_depth;
    if (j->spp <= 0 || j->spp > (1 << 20) || j->w <= 0 || j->h <= 0 || (int64_t)j->w * j->h > (1 << 26) ||
        j->max_depth < -1 || job->sample_offset < 0)
        return srv_error(s, LJ_ERR_INVALID_ARG, "submit: bad resolution, spp, sample offset or depth");
    j->total = (int64_t)j->w * j->h * j->spp;
    j->bytes = (int64_t)j->w * j->h * (24 + 12);
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->dead) return srv_error(s, LJ_ERR_CUDA, "submit: server stopped after an error: " + s->last_error);
    if (s->stopping) return srv_error(s, LJ_ERR_INVALID_ARG, "submit: server is stopping");
    if ((int64_t)s->pending.size() >= s->opt.max_queued_jobs)
        return srv_error(s, LJ_ERR_QUEUE_FULL, "submit: admission queue is full");
    // register the scene (kept until the server stops)
    int slot = -1;
    for (size_t k = 0; k < s->scenes.size(); k++)
        if (s->scenes[k] == scene) slot = (int)k;
    int64_t scene_bytes = slot < 0 ? scene->info.device_bytes : 0;
    if (s->bytes_pool + s->bytes_scenes + scene_bytes + j->bytes > s->opt.hbm_budget_bytes)
        return srv_error(s, LJ_ERR_OUT_OF_MEMORY, "submit: the job does not fit the HBM budget");
    if (slot < 0) {
        if ((int)s->scenes.size() >= kMaxScenes)
            return srv_error(s, LJ_ERR_SIZE_LIMIT, "submit: too many distinct scenes for one server");
        slot = (int)s->scenes.size();
        // the table entry is written before any job that uses it is admitted
        cudaSetDevice(s->device);
        cudaError_t e = cudaMemcpy(s->d_scenes + slot, &scene->dev, sizeof(DevScene), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return srv_error(s, LJ_ERR_CUDA, std::string("submit: ") + cudaGetErrorString(e));
        s->scenes.push_back(scene);
        scene->server_refs++;
        s->bytes_scenes += scene_bytes;
    }
    j->scene_slot = slot;
    j->id = s->next_id++;
    j->t_submit = now_ms(s->t0);
    HostJob *raw = j.get();
    s->jobs[raw->id] = std::move(j);
    s->pending.push_back(raw);
    s->n_submitted++;
    *job_id = raw->id;
    s->cv_work.notify_one();
    return LJ_OK;
}

int lj_gpu_server_poll(lj_server *s, int64_t id, lj_job_status *st) {
    if (!s) return LJ_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    HostJob *j = find_job(s, id);
    if (!j) return srv_error(s, LJ_ERR_NOT_FOUND, "poll: unknown job id");
    fill_status(j, st);
    return LJ_OK;
}

int lj_gpu_server_wait(lj_server *s, int64_t id, double timeout_s, float *out_rgb, lj_job_status *st) {
    if (!s) return LJ_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    HostJob *j = find_job(s, id);
    if (!j) return srv_error(s, LJ_ERR_NOT_FOUND, "wait: unknown job id");
    auto pred = [&] { return j->state != LJ_JOB_QUEUED && j->state != LJ_JOB_RUNNING; };
    if (timeout_s < 0) {
        s->cv_done.wait(lk, pred);
    } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) {
        fill_status(j, st);
        return srv_error(s, LJ_ERR_TIMEOUT, "wait: timed out");
    }
    fill_status(j, st);
    if (j->state == LJ_JOB_CANCELLED) return LJ_ERR_CANCELLED;
    if (j->state == LJ_JOB_FAILED) return j->error ? j->error : LJ_ERR_CUDA;
    if (out_rgb) {
        // copy without the lock (the worker keeps launching), then give the
        // pinned buffer back to the pool
        float *buf = j->h_img;
        const size_t cap = j->h_img_cap, bytes = sizeof(float) * 3 * (size_t)j->w * j->h;
        j->h_img = nullptr;
        s->jobs.erase(id);
        lk.unlock();
        memcpy(out_rgb, buf, bytes);
        lk.lock();
        s->pinned_free.emplace(cap, buf);
    }
    return LJ_OK;
}

int lj_gpu_server_cancel(lj_server *s, int64_t id) {
    if (!s) return LJ_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    HostJob *j = find_job(s, id);
    if (!j) return srv_error(s, LJ_ERR_NOT_FOUND, "cancel: unknown job id");
    if (j->state == LJ_JOB_QUEUED || j->state == LJ_JOB_RUNNING) j->cancel_req = true;
    s->cv_work.notify_one();
    return LJ_OK;
}

int lj_gpu_server_stats(lj_server *s, lj_server_stats *st) {
    if (!s || !st) return LJ_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (!any_live(s) && s->pending.empty() && !s->dead) {
        // idle: every path has retired, so the ray counters are final
        unsigned long long q[kStatWords];
        cudaSetDevice(s->device);
        if (cudaMemcpy(q, s->dev.stats, sizeof(q), cudaMemcpyDeviceToHost) == cudaSuccess)
            memcpy(s->counters, q, sizeof(q));
    }
    st->jobs_submitted = s->n_submitted;
    st->jobs_done = s->n_done;
    st->jobs_failed = s->n_failed;
    st->jobs_cancelled = s->n_cancelled;
    st->waves = s->waves;
    st->graph_launches = s->graph_launches;
    st->samples_done = s->samples_done;
    st->bytes_resident = s->bytes_pool + s->bytes_scenes + s->bytes_jobs;
    st->busy_ms = s->busy_ms;
    st->rays_closest = (int64_t)s->counters[0];
    st->rays_shadow = (int64_t)s->counters[1];
    st->path_segments = (int64_t)s->counters[2];
    st->vol_segments = (int64_t)s->counters[3];
    st->nee_requests = (int64_t)s->counters[4];
    st->null_collisions = (int64_t)s->counters[7];
    st->real_collisions = (int64_t)s->counters[8];
    st->kernel_launches = s->kernel_launches;
    for (int c = 0; c < LJ_KERNEL_CLASSES; c++) {
        st->class_ms[c] = s->class_ms[c];
        st->class_launches[c] = s->class_launches[c];
    }
    return LJ_OK;
}

const char *lj_gpu_server_last_error(lj_server *s) { return s ? s->last_error.c_str() : ""; }

int lj_gpu_server_stop(lj_server *s) {
    if (!s) return LJ_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
        s->stop_time = std::chrono::steady_clock::now();
        for (HostJob *j : s->pending) {
            j->state = LJ_JOB_CANCELLED;
            s->n_cancelled++;
        }
        s->pending.clear();
        for (HostJob *j : s->live)
            if (j) j->cancel_req = true;
        s->cv_work.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    int rc = s->dead ? LJ_ERR_CUDA : LJ_OK;
    auto &v = s->ctx->servers;
    v.erase(std::remove(v.begin(), v.end(), s), v.end());
    release_device(s);
    delete s;
    return rc;
}

int lj_gpu_server_autotune(lj_ctx *ctx, lj_scene *const *scenes, const lj_job_desc *jobs,
                           const int32_t *job_scene, int32_t n_jobs, const char *cache_path,
                           lj_server_options *options) {
    if (!ctx || !scenes || !jobs || !job_scene || n_jobs <= 0 || !options) return LJ_ERR_INVALID_ARG;
    const int objective = options->tune_objective;
    if (objective < LJ_TUNE_BALANCED || objective > LJ_TUNE_LATENCY)
        return set_error(ctx, LJ_ERR_INVALID_ARG, "autotune: unknown objective");
    // workload key: device, SM count, objective, total samples and largest
    // scene (log2 buckets), share of volumetric samples (tenths), mean max
    // depth (log2 bucket)
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, ctx->device) != cudaSuccess)
        return set_error(ctx, LJ_ERR_CUDA, "autotune: cannot query the device");
    double total = 0, max_prims = 1, vol = 0, depth = 0;
    for (int i = 0; i < n_jobs; i++) {
        const lj_scene *sc = scenes[job_scene[i]];
        double w = jobs[i].width > 0 ? jobs[i].width : sc->width;
        double h = jobs[i].height > 0 ? jobs[i].height : sc->height;
        double spp = jobs[i].spp > 0 ? jobs[i].spp : sc->options.samples_per_pixel;
        total += w * h * spp;
        if (sc->options.integrator == LJ_INTEGRATOR_VOLPATH) vol += w * h * spp;
        int md = jobs[i].override_depth ? jobs[i].max_depth : sc->options.max_depth;
        depth += md < 0 ? 64 : md;
        max_prims = std::max(max_prims, (double)sc->info.num_prims);
    }
    std::ostringstream key;
    key << prop.name << "|sm" << prop.multiProcessorCount << "|obj" << objective << "|samples2^"
        << (int)std::lround(std::log2(total + 1)) << "|prims2^" << (int)std::lround(std::log2(max_prims))
        << "|vol" << (int)std::lround(10 * vol / std::max(total, 1.0)) << "|depth2^"
        << (int)std::lround(std::log2(depth / n_jobs + 1));
    std::map<std::string, std::string> cache;
    auto field = [](const std::string &v, const char *name, long long *out) {
        size_t p = v.find(std::string("\"") + name + "\":");
        if (p == std::string::npos) return false;
        *out = std::strtoll(v.c_str() + p + std::strlen(name) + 3, nullptr, 10);
        return true;
    };
    if (cache_path) {
        std::ifstream f(cache_path);
        std::string line;
        while (std::getline(f, line)) {
            size_t a = line.find('"'), b = a == std::string::npos ? a : line.find('"', a + 1);
            size_t c = b == std::string::npos ? b : line.find('{', b);
            size_t d = c == std::string::npos ? c : line.find('}', c);
            if (d == std::string::npos) continue;
            cache[line.substr(a + 1, b - a - 1)] = line.substr(c, d - c + 1);
        }
        auto it = cache.find(key.str());
        long long pool = 0, blk = 0, wpp = 0;
        if (it != cache.end() && field(it->second, "path_pool", &pool) && field(it->second, "block_size", &blk) &&
            field(it->second, "waves_per_poll", &wpp)) {
            options->path_pool = pool;
            options->block_size = (int32_t)blk;
            options->waves_per_poll = (int32_t)wpp;
            return LJ_OK;
        }
    }
    struct Cand {
        int64_t pool;
        int32_t block, wpp;
        double rate, latency;   // Msamples/s, median job latency (ms)
    };
    // one run of the job mix, all jobs submitted at once
    auto run = [&](Cand &c, std::string *why) {
        lj_server_options o = *options;
        o.path_pool = c.pool;
        o.block_size = c.block;
        o.waves_per_poll = c.wpp;
        lj_server *srv = nullptr;
        if (lj_gpu_server_start(ctx, &o, &srv) != LJ_OK) return 1;   // e.g. pool above the budget
        auto t0 = std::chrono::steady_clock::now();
        std::vector<int64_t> ids(n_jobs, 0);
        std::vector<double> lat;
        bool ok = true;
        for (int i = 0; i < n_jobs && ok; i++)
            ok = lj_gpu_server_submit(srv, scenes[job_scene[i]], &jobs[i], &ids[i]) == LJ_OK;
        for (int i = 0; i < n_jobs && ok; i++) {
            lj_job_status st{};
            ok = lj_gpu_server_wait(srv, ids[i], 600.0, nullptr, &st) == LJ_OK;
            lat.push_back(st.finish_ms - st.submit_ms);
        }
        double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        *why = lj_gpu_server_last_error(srv);
        if (lj_gpu_server_stop(srv) != LJ_OK) ok = false;
        if (!ok) return -1;
        std::sort(lat.begin(), lat.end());
        c.rate = total / sec * 1e-6;
        c.latency = lat[lat.size() / 2];
        return 0;
    };
    auto better = [&](const Cand &a, const Cand &b, double best_rate) {   // is a preferred to b?
        if (objective == LJ_TUNE_THROUGHPUT) return a.rate > b.rate;
        if (objective == LJ_TUNE_LATENCY) return a.latency < b.latency;
        const bool ia = a.rate >= 0.97 * best_rate, ib = b.rate >= 0.97 * best_rate;
        if (ia != ib) return ia;
        return ia ? a.latency < b.latency : a.rate > b.rate;
    };
    auto pick = [&](std::vector<Cand> &cs) {
        double best_rate = 0;
        for (const Cand &c : cs) best_rate = std::max(best_rate, c.rate);
        size_t k = 0;
        for (size_t i = 1; i < cs.size(); i++)
            if (better(cs[i], cs[k], best_rate)) k = i;
        return cs[k];
    };
    const int64_t pools[] = {(int64_t)1 << 20, (int64_t)1 << 21, (int64_t)1 << 22, (int64_t)1 << 23,
                             (int64_t)1 << 24};
    const int32_t blocks[] = {64, 128, 256};
    const int32_t wpps[] = {4, 8, 16};
    std::vector<Cand> done;
    std::string why;
    // path pool x block size at 8 waves per poll, then waves per poll for the
    // best of those (the poll interval hardly interacts with the other two)
    for (int64_t pool : pools)
        for (int32_t blk : blocks) {
            Cand c{pool, blk, 8, 0, 0};
            int rc = run(c, &why);
            if (rc < 0) return set_error(ctx, LJ_ERR_CUDA, "autotune: candidate run failed: " + why);
            if (rc == 0) done.push_back(c);
        }
    if (done.empty()) return set_error(ctx, LJ_ERR_OUT_OF_MEMORY, "autotune: no candidate fits the HBM budget");
    const Cand first = pick(done);
    for (int32_t w : wpps) {
        if (w == first.wpp) continue;
        Cand c{first.pool, first.block, w, 0, 0};
        int rc = run(c, &why);
        if (rc < 0) return set_error(ctx, LJ_ERR_CUDA, "autotune: candidate run failed: " + why);
        if (rc == 0) done.push_back(c);
    }
    const Cand best = pick(done);
    options->path_pool = best.pool;
    options->block_size = best.block;
    options->waves_per_poll = best.wpp;
    if (cache_path) {
        std::ostringstream v;
        v << "{\"path_pool\": " << best.pool << ", \"block_size\": " << best.block << ", \"waves_per_poll\": "
          << best.wpp << ", \"msamples_s\": " << best.rate << ", \"median_latency_ms\": " << best.latency
          << ", \"candidates\": " << done.size() << "}";
        cache[key.str()] = v.str();
        std::ofstream f(cache_path);
        f << "{\n";
        size_t k = 0;
        for (auto &kv : cache) f << "  \"" << kv.first << "\": " << kv.second << (++k < cache.size() ? "," : "") << "\n";
        f << "}\n";
        if (!f) return set_error(ctx, LJ_ERR_INVALID_ARG, "autotune: cannot write the cache file");
    }
    return LJ_OK;
}

}  // extern "C"
