"""Benchmark: lajolla's rendering hot path on one GB300, served.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (a "step" = serving one batch of render jobs):
  serving  32 jobs with Poisson arrivals (mean 200/s, seeded).  Each job
           renders one of 6 resident scenes -- in turn a seeded Cornell box
           with tessellated walls, a seeded terrain + icosphere + HDR-envmap
           scene (Disney BSDFs) and a seeded heterogeneous volume (256^3
           one-channel FP32 value-noise density, max 20, scaled per
           channel by (1.05, 0.9, 0.8) for a chromatic sigma_t) in a
           dielectric sphere over a tessellated floor (volumetric path
           tracer), 10k-2M triangles,
           log-uniform -- at a square resolution in {128, 256, 512, 1024},
           spp in {4, 16, 64, 256}, max depth uniform in 6..64 (Russian
           roulette from depth 5).  ~0.9e9 camera samples per step, a
           quarter of them volumetric.

Our arm (--impl ours):
  value     Msamples/s of the continuous-batching server (lj_gpu_server_*):
            jobs submitted at their arrival times, the paths of all live jobs
            in one pool of wavefront queues replayed as CUDA graphs, pool and
            block size from the autotuner; each job's image returned to host
            memory.  Step time = host clock from the first arrival to the last
            completion, the device synchronized on both sides.
  plain     the same jobs through the single-scene wavefront renderer, one at
            a time in arrival order (lj_gpu_render_job_device + image to
            host).  Both arms trace the same keyed samples, so their images
            (and errors) match (matched_error).
  latency   p50 / p99 of (completion - arrival) per job, both arms.
  e2e       one step through the C ABI from host memory: the scene pool is
            uploaded (lj_gpu_scene_create_many: descriptors from host, device
            BVH builds, the scenes' uploads overlapped) inside the timed
            region, then the jobs are served.
  roofline  the dominant kernel class of a profiled server step
            (LJ_SERVER_PROFILE: CUDA events around every kernel on the
            server's stream), compulsory algorithmic bytes per launch
            (include/lj_bytes_model.h) / average launch time, against the
            measured HBM copy bandwidth (MEASURED_PEAKS.json); with_bvh adds
            the BVH bytes per ray counted on the same jobs
            (LJ_RENDER_COUNT_BVH), issue_bound the instruction-issue ceiling
            of the kernel's ncu capture.
  quality   per-image relative MSE of one 128^2 job per scene kind at spp 4
            .. 4096, batched and plain, against a 64k-spp render validated
            against the oracle at 3 standard errors; the spp that reaches
            1e-3 is marked.
  single_scene  the Cornell box (256^2, 64 spp), full terrain (5.5M
            triangles, 1080p, 256 spp) and volume (256^3, 512^2, 256 spp)
            configurations, and the intersection + BSDF microbenchmark.
  small_jobs  a burst of 64 small jobs ({64,128,256}^2, 1-16 spp) served
            and rendered plain: batching where no job fills the GPU alone.
  cpu_baseline  the oracle's C++ restatement of the reference path tracer
            (oracle/lj_oracle.cpp, FP64, all host threads) on a bounded
            sample drawn from the GPU arm's own work: (job, pixel, sample)
            keys uniform over a step's W*H*spp, each at its job's resolution
            and depth with the GPU's keyed random numbers; per_sample_parity
            compares a subset of such samples with the GPU's.
The working set (path pool ~1 GB, scenes up to 2M triangles, accumulators)
is larger than L2.

Reference arm (--impl reference): the reference's CPU path tracer on the
host cores -- the reference renderer cannot be built on the benchmark machine
(its sources are not present there), so its C++ restatement in oracle/ runs
instead, pinned sample-for-sample to the reference's own renders
(tests/golden); step i samples the work of the GPU arm's timed step i.

Multi-GPU: replicas only (each rank serves its own copy of the job stream;
no collective on the data path); value sums all ranks' samples over the
slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from lajolla_public_gb300 import abi, scenes  # noqa: E402

WORKLOAD = dict(name="serving", scene_seed=0, n_scenes=6, n_jobs=32, rate=200.0)
METRIC = "Msamples/s (served render jobs, batched; plain GPU and p50/p99 job latency beside it)"
TUNE_CACHE = os.path.join(ROOT, "lajolla_public_gb300", "_lib", "autotune.json")


def make_scenes():
    return scenes.serving_scenes(WORKLOAD["scene_seed"], WORKLOAD["n_scenes"])


def make_jobs(step_seed):
    return scenes.serving_jobs(seed=step_seed, n_jobs=WORKLOAD["n_jobs"], n_scenes=WORKLOAD["n_scenes"],
                               rate=WORKLOAD["rate"])


def job_samples(jobs):
    return sum(j["width"] * j["height"] * j["spp"] for j in jobs)


def config_dict(pool, opts=None):
    w = WORKLOAD
    cfg = {"workload": "serving: %d jobs per step, Poisson arrivals %.0f/s; %d resident scenes "
                       "(tessellated Cornell boxes, terrain+icospheres+envmap, heterogeneous 256^3 volumes in a "
                       "dielectric sphere; %d-%d triangles); "
                       "resolution {128,256,512,1024}^2, spp {4,16,64,256}, max depth 6-64"
                       % (w["n_jobs"], w["rate"], w["n_scenes"], min(s.num_triangles for s in pool),
                          max(s.num_triangles for s in pool)),
           "jobs_per_step": w["n_jobs"], "arrival_rate_per_s": w["rate"],
           "scene_triangles": [s.num_triangles for s in pool],
           "integrator": "path (NEE + MIS, RR from depth 5); volpath v6 for the volume scenes (delta tracking, "
                         "ratio-tracking NEE, spectral MIS)",
           "l2": "working set (path pool ~1 GB, scenes, accumulators) larger than L2",
           "timing": "host clock per step, device synchronized on both sides",
           "parallelism": "replicas"}
    if opts is not None:
        cfg["server"] = {"path_pool": int(opts.path_pool), "block_size": int(opts.block_size),
                         "policy": "SRPT" if opts.policy == abi.LJ_SCHED_SRPT else "FIFO",
                         "cuda_graphs": bool(opts.use_graphs), "waves_per_poll": int(opts.waves_per_poll),
                         "tuned_by": "lj_gpu_server_autotune, objective throughput (cache %s)"
                                     % os.path.relpath(TUNE_CACHE, ROOT)}
    return cfg


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if r[4 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------ byte model
# Algorithmic bytes per unit of work of each wavefront kernel class (the
# same constants as include/lj_bytes_model.h).
BYTES_RAY = 32          # lj_ray: org + tnear + dir + tfar
BYTES_HIT = 16          # t, prim, u, v
BYTES_PATH_STATE = 64   # pixel 4 + rng 8 + beta 16 + L 16 + prev 16 + nv 4
BYTES_SHADE_GEOM = 52   # 3 vertex indices + 3 positions + prim->shape
BYTES_SHADE_MAT = 160   # material record: type, eta, textured flags, 12 x RGB slot values
BYTES_SHADOW_ENTRY = 52  # shadow ray 32 + path 4 + contribution 16
BYTES_VOL_STATE = 112
BYTES_NEE_REQUEST = 108
BYTES_NEE_RESULT = 56
BYTES_VOL_SEGMENT = (2 * (BYTES_RAY + BYTES_HIT + BYTES_VOL_STATE) + 2 * (BYTES_VOL_STATE + BYTES_RAY)
                     + 2 * BYTES_NEE_REQUEST + BYTES_NEE_RESULT)
BYTES_NEE_SHADOW_LOOP = BYTES_NEE_REQUEST + BYTES_NEE_RESULT
BYTES_NODE = 80         # compressed 8-wide BVH node
BYTES_LEAF = 48         # leaf primitive record


def kernel_bytes(cls, samples, rays_closest, rays_shadow, segments, vol_segments=0, nee_requests=0):
    """Compulsory algorithmic bytes moved by all launches of one kernel class
    (queues, hits, path state, shading records; BVH bytes and density-grid
    lookups excluded)."""
    if cls == abi.LJ_KERNEL_MEDIUM:
        return vol_segments * BYTES_VOL_SEGMENT
    if cls == abi.LJ_KERNEL_NEE:
        return nee_requests * BYTES_NEE_SHADOW_LOOP
    if cls == abi.LJ_KERNEL_TRACE:
        return rays_closest * (BYTES_RAY + BYTES_HIT)
    if cls == abi.LJ_KERNEL_SHADOW:
        # shadow entry read + radiance read-modify-write
        return rays_shadow * (BYTES_SHADOW_ENTRY + 32)
    if cls == abi.LJ_KERNEL_SHADE:
        reads = BYTES_RAY + BYTES_HIT + 4 + BYTES_PATH_STATE + BYTES_SHADE_GEOM + BYTES_SHADE_MAT
        writes = BYTES_PATH_STATE + BYTES_RAY + 4
        return segments * (reads + writes) + rays_shadow * BYTES_SHADOW_ENTRY
    if cls == abi.LJ_KERNEL_CAMERA:
        return samples * (BYTES_RAY + 4 + BYTES_PATH_STATE)
    return 0


# ------------------------------------------------------------ arms
def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if n_gpus > 0 else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def pct(xs, q):
    return float(np.percentile(np.asarray(xs, np.float64), q)) if xs else None


def job_desc(j, profile=False, count_bvh=False, sample_offset=0):
    from lajolla_public_gb300 import gpu
    return gpu.job_desc(seed=j["seed"], spp=j["spp"], sample_offset=sample_offset, width=j["width"],
                        height=j["height"], max_depth=j["max_depth"], rr_depth=j["rr_depth"], profile=profile,
                        count_bvh=count_bvh)


def serve_step(srv, gscenes, jobs, keep=()):
    """Submits `jobs` at their arrival times and waits for all of them.
    Returns (seconds, latencies_ms, {index: image} for `keep`)."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ids = []
    for j in jobs:
        dt = j["arrival_s"] - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        ids.append(srv.submit(gscenes[j["scene"]], job_desc(j)))
    lat, imgs, fin = [], {}, []
    for k, jid in enumerate(ids):
        img, st = srv.wait(jid, timeout=600)
        lat.append(st.finish_ms - st.submit_ms)
        fin.append(st.finish_ms)
        if k in keep:
            imgs[k] = img
    torch.cuda.synchronize()
    return time.perf_counter() - t0, lat, imgs


def plain_step(gscenes, jobs, out, stream, keep=()):
    """The same jobs one at a time through the single-scene renderer."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lat, imgs = [], {}
    for k, j in enumerate(jobs):
        dt = j["arrival_s"] - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        n = j["width"] * j["height"] * 3
        gscenes[j["scene"]].render_job_device(out[:n], job_desc(j), stream=stream)
        img = out[:n].cpu()   # synchronizes
        lat.append((time.perf_counter() - t0 - j["arrival_s"]) * 1e3)
        if k in keep:
            imgs[k] = img.numpy().reshape(j["height"], j["width"], 3)
    torch.cuda.synchronize()
    return time.perf_counter() - t0, lat, imgs


def small_jobs(srv, gscenes, out, stream, reps=3):
    """Batching where it matters most: a burst of 64 small jobs (resolution
    {64,128,256}^2, spp {1,4,16}, max depth 6-16, all arriving at once) over
    the same resident scenes, served by the benchmark's server and rendered
    one at a time by the plain renderer; best of `reps` passes each."""
    jobs = scenes.serving_jobs(seed=77, n_jobs=64, n_scenes=WORKLOAD["n_scenes"], rate=1e9,
                               resolutions=(64, 128, 256), spps=(1, 4, 16), depth=(6, 16))
    n = job_samples(jobs)
    b = min(serve_step(srv, gscenes, jobs)[0] for _ in range(reps))
    p = min(plain_step(gscenes, jobs, out, stream)[0] for _ in range(reps))
    _, lat_b, _ = serve_step(srv, gscenes, jobs)
    _, lat_p, _ = plain_step(gscenes, jobs, out, stream)
    return {"what": "burst of 64 jobs: resolution {64,128,256}^2, spp {1,4,16}, max depth 6-16, all arriving "
                    "at once; same scenes and server options as the headline",
            "samples": n, "batched_msamples_s": round(n / b / 1e6, 1), "plain_msamples_s": round(n / p / 1e6, 1),
            "batched_over_plain": round(p / b, 3),
            "latency_ms": {"batched_p50": round(float(np.percentile(lat_b, 50)), 2),
                           "batched_p99": round(float(np.percentile(lat_b, 99)), 2),
                           "plain_p50": round(float(np.percentile(lat_p, 50)), 2),
                           "plain_p99": round(float(np.percentile(lat_p, 99)), 2)}}


def tuned_options(ctx, gscenes):
    """Server options from the autotuner (cached per device and workload)."""
    from lajolla_public_gb300 import gpu
    tune = scenes.serving_jobs(seed=999, n_jobs=8, n_scenes=WORKLOAD["n_scenes"], resolutions=(128, 256, 512, 1024),
                               spps=(4, 16, 64))
    jd = [job_desc(j) for j in tune]
    os.makedirs(os.path.dirname(TUNE_CACHE), exist_ok=True)
    # the headline is throughput (latency is reported beside it), so the
    # tuning ranks by throughput; the library's default objective trades a
    # little of it for latency
    opt = gpu.server_options(policy=abi.LJ_SCHED_SRPT, tune_objective=abi.LJ_TUNE_THROUGHPUT)
    return gpu.autotune(ctx, gscenes, jd, [j["scene"] for j in tune], cache_path=TUNE_CACHE, options=opt)


SCENE_KINDS = ("cornell box", "terrain + envmap", "volume")   # serving_scenes cycles through them


def quality(srv, gscenes, pool, cs, out, stream, res=128, depth=16, ref_spp=65536,
            spps=(4, 16, 64, 256, 1024, 4096), check_px=128, check_spp=4096, key_px=512, key_samples=2):
    """Per-image relative MSE (sum of squared errors / sum of squares of the
    reference) of one 128 x 128 job per scene kind against a 64k-spp render
    of the same job by the plain GPU renderer with an independent seed.
    Each reference is first checked against the oracle twice: per pixel, on
    `check_px` random pixels its value lies within 3 standard errors of the
    oracle's mean of `check_spp` keyed samples (enough samples that
    heavy-tailed pixels show their tails); and per sample, the GPU's samples
    of the reference's own keys (whole images at `key_samples` sample
    indices) equal the oracle's on `key_px` pixels each.  The job is then
    rendered at each spp by the server (batched) and by the plain renderer;
    both trace the same keyed samples, so their errors match.  rel_mse x spp
    stays flat when the error is the estimator's variance (no bias)."""
    from lajolla_public_gb300 import gpu
    rows = []
    n = res * res * 3
    for kind_i, kind in enumerate(SCENE_KINDS):
        si = kind_i   # first scene of each kind
        sc = pool[si]
        seed = 4242 + si
        job = dict(scene=si, seed=seed, width=res, height=res, max_depth=depth, rr_depth=5)
        t0 = time.perf_counter()
        gscenes[si].render_job_device(out[:n], job_desc(dict(job, spp=ref_spp, seed=seed ^ 0x5bd1e995)),
                                      stream=stream)
        ref = out[:n].cpu().numpy().reshape(res, res, 3).astype(np.float64)
        ref_s = time.perf_counter() - t0
        # the reference against the oracle: per pixel (independent keys) ...
        px = cs.rng.integers(0, res * res, check_px).astype(np.int32)
        osm = cs.oss[si].render_job_samples(seed ^ 0x1234567, res, res, depth, 5, np.repeat(px, check_spp),
                                            np.tile(np.arange(check_spp, dtype=np.int32), check_px),
                                            nthreads=cs.cores).reshape(check_px, check_spp, 3)
        osm = np.where(np.isfinite(osm), osm, 0.0)
        m_o, sd_o = osm.mean(axis=1), osm.std(axis=1)
        se = np.sqrt(sd_o ** 2 / check_spp + sd_o ** 2 / ref_spp) + 1e-9
        within = float((np.abs(ref.reshape(-1, 3)[px] - m_o) <= 3 * se).all(axis=1).mean())
        # ... and per sample (the reference's own keys)
        agree = []
        for _ in range(key_samples):
            k = int(cs.rng.integers(0, ref_spp))
            gscenes[si].render_job_device(out[:n], job_desc(dict(job, spp=1, seed=seed ^ 0x5bd1e995),
                                                            sample_offset=k), stream=stream)
            g1 = out[:n].cpu().numpy().reshape(-1, 3).astype(np.float64)
            kp = cs.rng.integers(0, res * res, key_px).astype(np.int32)
            o1 = cs.oss[si].render_job_samples(seed ^ 0x5bd1e995, res, res, depth, 5, kp,
                                               np.full(key_px, k, np.int32), nthreads=cs.cores)
            o1 = np.where(np.isfinite(o1).all(axis=1, keepdims=True), o1, 0.0)
            agree.append((np.abs(g1[kp] - o1) <= 1e-2 * np.maximum(np.abs(o1), 1e-1)).all(axis=1).mean())
        den = float(np.mean(ref ** 2)) + 1e-30
        per_spp, first_ok = [], None
        for spp in spps:
            jb = dict(job, spp=spp)
            jid = srv.submit(gscenes[si], job_desc(jb))
            img_b, _ = srv.wait(jid, timeout=600)
            gscenes[si].render_job_device(out[:n], job_desc(jb), stream=stream)
            img_p = out[:n].cpu().numpy().reshape(res, res, 3)
            rb = float(np.mean((img_b - ref) ** 2) / den)
            rp = float(np.mean((img_p - ref) ** 2) / den)
            ok = max(rb, rp) <= 1e-3
            if ok and first_ok is None:
                first_ok = spp
            per_spp.append({"spp": spp, "batched": rb, "plain": rp, "rel_mse_x_spp": round(rb * spp, 4),
                            "meets_1e-3": ok,
                            "batched_vs_plain_max_abs": float(np.abs(img_b - img_p).max())})
        rows.append({"scene": kind, "scene_triangles": sc.num_triangles,
                     "job": "%dx%d, max depth %d, RR from 5" % (res, res, depth), "ref_spp": ref_spp,
                     "ref_render_s": round(ref_s, 3),
                     "ref_vs_oracle_within_3se": round(within, 4),
                     "ref_vs_oracle": "%d pixels x %d oracle samples" % (check_px, check_spp),
                     "ref_keys_vs_oracle_agree": round(float(np.mean(agree)), 4),
                     "ref_keys_vs_oracle": "%d sample indices x %d pixels of the reference's keys, 1e-2 relative"
                                           % (key_samples, key_px),
                     "rel_mse": per_spp, "min_spp_meeting_1e-3": first_ok})
    return rows


def bvh_bytes(gscenes, jobs, out, stream):
    """BVH bytes per ray of the plain renderer over `jobs` (the same keyed
    paths the server traces): an instrumented traversal of every 16th entry
    of every closest-hit and shadow-ray queue (LJ_RENDER_COUNT_BVH) counts
    the 80-byte wide nodes fetched and the 48-byte leaf records tested."""
    tot = np.zeros((3, 2), np.int64)
    for j in jobs:
        n = j["width"] * j["height"] * 3
        st = gscenes[j["scene"]].render_job_device(out[:n], job_desc(j, count_bvh=True), stream=stream, stats=True)
        tot += np.array([list(st.bvh_rays), list(st.bvh_nodes), list(st.bvh_prims)], np.int64)
    res = {}
    for k, name in ((0, "closest"), (1, "shadow")):
        r = max(1, int(tot[0, k]))
        res[name] = {"rays_counted": int(tot[0, k]), "nodes_per_ray": round(tot[1, k] / r, 3),
                     "leaf_records_per_ray": round(tot[2, k] / r, 3),
                     "bvh_bytes_per_ray": round((BYTES_NODE * tot[1, k] + BYTES_LEAF * tot[2, k]) / r, 1)}
    return res


def single_scene_configs(ctx, stream):
    """The single-scene configurations through lj_gpu_render_device: a
    timed render (CUDA events around the call's kernels, after a warm-up
    render) and a profiled one (events around every kernel) for the class
    split."""
    import torch
    from lajolla_public_gb300 import gpu
    cases = (("cornell_box", "seeded Cornell box (36 triangles, fits in L2), 256x256, 64 spp, max depth 6",
              lambda: scenes.cornell_box(seed=0)),
             ("terrain", "2048x1024-grid fractal terrain + 64 subdivision-5 icospheres (5.5M triangles), Disney "
                         "BSDFs, 1024x512 HDR envmap, 1920x1080, 256 spp, max depth 8",
              lambda: scenes.terrain_scene(seed=0)),
             ("volume", "256^3 heterogeneous chromatic medium (max density 20, HG g 0.7) in a dielectric sphere "
                        "(eta 1.33) over a plane, sphere light, 512x512, 256 spp, max depth 64 (volpath v6)",
              lambda: scenes.volume_scene(seed=0)))
    rows = {}
    for name, what, mk in cases:
        sc = mk()
        g = gpu.GpuScene(ctx, sc)
        out = torch.empty(sc.width * sc.height * 3, dtype=torch.float32, device="cuda")
        g.render_device(out, seed=1, spp=4, stream=stream)
        st = g.render_device(out, seed=2, stream=stream)
        sp = g.render_device(out, seed=3, stream=stream, profile=True)
        rays = st.rays_closest + st.rays_shadow
        rows[name] = {"what": what, "msamples_per_s": round(st.samples / st.device_ms / 1e3, 2),
                      "mrays_per_s": round(rays / st.device_ms / 1e3, 1), "device_ms": round(st.device_ms, 2),
                      "samples": int(st.samples), "rays_closest": int(st.rays_closest),
                      "rays_shadow": int(st.rays_shadow), "bvh_build_ms": round(g.info().build_ms, 2),
                      "kernel_ms_profiled": {abi.KERNEL_CLASS_NAMES[c]: round(sp.class_ms[c], 2)
                                             for c in range(abi.LJ_KERNEL_CLASSES) if sp.class_launches[c]}}
        g.close()
        del out
    return rows


def run_ours(args):
    import torch
    from lajolla_public_gb300 import gpu

    rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    ctx = gpu.Context(local)
    pool = make_scenes()
    gscenes = [gpu.GpuScene(ctx, s) for s in pool]
    stream = torch.cuda.current_stream().cuda_stream
    max_px = 1024 * 1024
    out = torch.empty(max_px * 3, dtype=torch.float32, device="cuda")

    opts = tuned_options(ctx, gscenes)
    srv = gpu.Server(ctx, opts)

    # warm-up steps (both arms)
    for i in range(args.warmup):
        jobs = make_jobs(100 + i)
        serve_step(srv, gscenes, jobs)
        if i == 0:
            plain_step(gscenes, jobs, out, stream)

    # timed steps
    clocks = ClockSampler(local)
    clocks.start()
    st0 = srv.stats()
    barrier(world)
    b_secs, b_lat, p_secs, p_lat = [], [], [], []
    samples = 0
    match = 0.0
    for i in range(args.steps):
        jobs = make_jobs(1000 + i)
        samples += job_samples(jobs)
        keep = tuple(range(len(jobs))) if i == 0 else ()
        sec, lat, bimgs = serve_step(srv, gscenes, jobs, keep)
        b_secs.append(sec)
        b_lat += lat
        sec, lat, pimgs = plain_step(gscenes, jobs, out, stream, keep)
        p_secs.append(sec)
        p_lat += lat
        for k in keep:   # batched and plain images of the same jobs (same keyed samples)
            match = max(match, float(np.abs(bimgs[k] - pimgs[k]).max() / (np.abs(pimgs[k]).max() + 1e-30)))
        del bimgs, pimgs
    barrier(world)
    ck = clocks.stop()
    st1 = srv.stats()
    b_total = max_over_ranks(sum(b_secs), world)
    p_total = max_over_ranks(sum(p_secs), world)
    value = samples * world / b_total / 1e6
    plain_value = samples * world / p_total / 1e6
    launches = st1.kernel_launches - st0.kernel_launches

    # e2e: upload the scene pool from host memory inside the timed region,
    # then serve the first timed step's jobs
    srv_e2e = gpu.Server(ctx, opts)
    jobs = make_jobs(1000)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g2 = gpu.create_scenes(ctx, pool)
    torch.cuda.synchronize()
    upload_s = time.perf_counter() - t0
    sec, _, _ = serve_step(srv_e2e, g2, jobs)
    e2e_s = time.perf_counter() - t0
    srv_e2e.stop()
    e2e_build_ms = [round(g.info().build_ms, 2) for g in g2]
    for g in g2:
        g.close()
    e2e_value = job_samples(jobs) * world / max_over_ranks(e2e_s, world) / 1e6
    update = scene_update_times(ctx, pool)
    h2d = sum(scene_host_bytes(s) for s in pool) + len(jobs) * 40
    d2h = sum(j["width"] * j["height"] * 12 for j in jobs)

    # roofline: a profiled server step (events around every kernel)
    prof = gpu.Server(ctx, gpu.server_options(path_pool=opts.path_pool, block_size=opts.block_size,
                                              policy=opts.policy, use_graphs=False, profile=True))
    jobs = make_jobs(1000)
    serve_step(prof, gscenes, jobs)
    ps = prof.stats()
    prof.stop()
    # the plain renderer's kernel classes on the same jobs
    plain_ms = [0.0] * abi.LJ_KERNEL_CLASSES
    plain_rays = [0, 0, 0]
    for j in jobs:
        n = j["width"] * j["height"] * 3
        st = gscenes[j["scene"]].render_job_device(out[:n], job_desc(j, profile=True), stream=stream, stats=True)
        for c in range(abi.LJ_KERNEL_CLASSES):
            plain_ms[c] += st.class_ms[c]
        plain_rays[0] += st.rays_closest
        plain_rays[1] += st.rays_shadow
        plain_rays[2] += st.path_segments
    bvh = bvh_bytes(gscenes, jobs, out, stream)
    peak, peak_kind = measured_peaks()
    cls_ms = list(ps.class_ms)
    dom = max((c for c in range(abi.LJ_KERNEL_CLASSES) if c != abi.LJ_KERNEL_OTHER), key=lambda c: cls_ms[c])
    nb = kernel_bytes(dom, job_samples(jobs), ps.rays_closest, ps.rays_shadow, ps.path_segments,
                      ps.vol_segments, ps.nee_requests)
    launches_dom = max(1, ps.class_launches[dom])
    avg_launch_s = cls_ms[dom] / 1e3 / launches_dom
    achieved = nb / launches_dom / avg_launch_s / 1e9
    units = {abi.LJ_KERNEL_TRACE: ps.rays_closest, abi.LJ_KERNEL_SHADOW: ps.rays_shadow,
             abi.LJ_KERNEL_SHADE: ps.path_segments, abi.LJ_KERNEL_MEDIUM: ps.vol_segments,
             abi.LJ_KERNEL_NEE: ps.nee_requests}.get(dom, job_samples(jobs))
    kname = {abi.LJ_KERNEL_CAMERA: "k_srv_regen", abi.LJ_KERNEL_MEDIUM: "k_srv_vol_a + k_srv_vol_c",
             abi.LJ_KERNEL_NEE: "k_srv_vol_b"}.get(dom, "k_srv_" + abi.KERNEL_CLASS_NAMES[dom])
    traffic, traffic_src = load_traffic(kname, units / launches_dom)
    with_bvh = None
    if dom in (abi.LJ_KERNEL_TRACE, abi.LJ_KERNEL_SHADOW):
        key = "closest" if dom == abi.LJ_KERNEL_TRACE else "shadow"
        nb_bvh = nb + units * bvh[key]["bvh_bytes_per_ray"]
        ach_bvh = nb_bvh / launches_dom / avg_launch_s / 1e9
        with_bvh = {"achieved": round(ach_bvh, 1), "frac": round(ach_bvh / peak, 4),
                    "bytes_per_launch": round(nb_bvh / launches_dom),
                    "bvh_bytes_per_ray": bvh[key]["bvh_bytes_per_ray"],
                    "how": "compulsory bytes + 80 B per wide node fetched + 48 B per leaf record tested, per ray "
                           "counted by an instrumented traversal of every 16th queue entry of the plain renderer "
                           "on the same jobs"}
    issue = load_issue(kname)
    if dom in (abi.LJ_KERNEL_MEDIUM, abi.LJ_KERNEL_NEE):
        note = ("volumetric steps are latency bound, not HBM bound: their dependent density-grid lookups "
                "(8 x 16 B per tracking step) mostly hit L1/L2 (ncu of the volume scene's a / b / c steps)")
    elif issue:
        note = ("traversal is instruction-issue bound, not HBM bound: ncu of a full secondary-ray wave shows "
                "%d%% issue active with %.1f of 32 lanes busy, DRAM a few %% of peak, L2 serving most BVH reads"
                % (round(100 * issue["issue_active"]), issue["threads_per_inst"]))
    else:
        note = "traversal is instruction-issue bound, not HBM bound (DRAM a few % of peak)"

    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Msamples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(b_total * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene and job generators)", "config": config_dict(pool, opts),
        "latency_ms": {"p50": round(pct(b_lat, 50), 2), "p99": round(pct(b_lat, 99), 2), "jobs": len(b_lat)},
        "plain": {"value": round(plain_value, 3), "unit": "Msamples/s",
                  "ms_per_step": round(p_total * 1e3 / args.steps, 3),
                  "latency_ms": {"p50": round(pct(p_lat, 50), 2), "p99": round(pct(p_lat, 99), 2)},
                  "what": "same jobs, one at a time, lj_gpu_render_job_device + image to host"},
        "batched_over_plain": round(value / plain_value, 3),
        "clocks": ck,
        "e2e": {"value": round(e2e_value, 3), "unit": "Msamples/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "scene_upload_s": round(upload_s, 4),
                "scene_build_ms": e2e_build_ms,
                "what": "scene pool uploaded from host (lj_gpu_scene_create_many, BVH builds) + one step served, "
                        "images to host"},
        "scene_update": update,
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                     else "fallback 6800 GB/s", "traffic": traffic, "traffic_source": traffic_src,
                     "bytes_per_launch": round(nb / launches_dom), "avg_launch_us": round(avg_launch_s * 1e6, 2),
                     "bytes": "compulsory (queues, hits, path state, shading records); BVH and density-grid "
                              "bytes excluded (with_bvh adds the BVH bytes)",
                     "with_bvh": with_bvh, "issue_bound": issue,
                     "note": note},
        "bvh_bytes_per_ray": bvh,
        "matched_error": {"batched_vs_plain_max_rel_diff": match,
                          "what": "largest |batched - plain| / max |plain| over the first timed step's job images: "
                                  "both forms trace the same keyed samples, so their errors match"},
        "kernel_ms_per_step": {abi.KERNEL_CLASS_NAMES[c]: round(cls_ms[c], 3) for c in range(abi.LJ_KERNEL_CLASSES)},
        "plain_kernel_ms_per_step": {abi.KERNEL_CLASS_NAMES[c]: round(plain_ms[c], 3)
                                     for c in range(abi.LJ_KERNEL_CLASSES)},
        "plain_rays_per_step": {"closest": plain_rays[0], "shadow": plain_rays[1], "segments": plain_rays[2]},
        "rays_per_step": {"closest": ps.rays_closest, "shadow": ps.rays_shadow, "segments": ps.path_segments,
                          "vol_segments": ps.vol_segments, "nee_requests": ps.nee_requests,
                          "null_collisions": ps.null_collisions, "real_collisions": ps.real_collisions},
        "mrays_per_s": round((st1.rays_closest - st0.rays_closest + st1.rays_shadow - st0.rays_shadow)
                             / b_total / 1e6, 1),
    }
    line["small_jobs"] = small_jobs(srv, gscenes, out, stream)
    if args.microbench:
        line["microbench"] = microbench(ctx)
    if args.configs:
        line["single_scene"] = single_scene_configs(ctx, stream)
    if rank == 0:
        line["cpu_baseline"], cs = cpu_baseline(pool, make_jobs(1000), target_s=args.cpu_seconds)
        line["per_sample_parity"] = per_sample_parity(cs, gscenes, make_jobs(1000), out, stream)
        if args.quality:
            line["quality"] = quality(srv, gscenes, pool, cs, out, stream)
        print(json.dumps(line), flush=True)
    srv.stop()
    for g in gscenes:
        g.close()
    ctx.close()


def microbench(ctx, n_tris=1 << 20, n_rays=1 << 24, n_bsdf=1 << 24, reps=3):
    """Intersection + BSDF microbenchmark: a 1M-triangle soup (centroids
    U[0,1]^3, vertex offsets N(0, 0.01)) against 16M rays (origins
    U[-0.5,1.5]^3, directions uniform on the sphere), closest and any hit;
    16M RoughPlastic and Disney BSDF eval / pdf / sample calls (wi, wo on the
    upper hemisphere, roughness U[0.01,1], metallic / specular U[0,1], fixed
    uniform random numbers).  Inputs generated on the device, seeded; best of
    `reps` launches, CUDA events on torch's stream."""
    import ctypes as C
    import torch
    from lajolla_public_gb300 import gpu
    g = gpu.GpuScene(ctx, scenes.soup_scene(1, n_tris))
    build_ms = g.info().build_ms
    gen = torch.Generator(device="cuda").manual_seed(7)
    rays = torch.empty((n_rays, 8), dtype=torch.float32, device="cuda")
    rays[:, 0:3] = torch.rand((n_rays, 3), generator=gen, device="cuda") * 2.0 - 0.5
    rays[:, 3] = 0.0
    d = torch.randn((n_rays, 3), generator=gen, device="cuda")
    rays[:, 4:7] = d / d.norm(dim=1, keepdim=True)
    rays[:, 7] = float("inf")
    hits = torch.empty((n_rays, 4), dtype=torch.float32, device="cuda")
    occ = torch.empty(n_rays, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    L = gpu.lib()

    def timed(fn):
        best = None
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ms = a.elapsed_time(b)
            best = ms if best is None else min(best, ms)
        return best

    ms_c = timed(lambda: ctx.check(L.lj_gpu_trace_closest(g.h, C.c_void_p(rays.data_ptr()),
                                                          C.c_void_p(hits.data_ptr()), n_rays, C.c_void_p(stream))))
    ms_a = timed(lambda: ctx.check(L.lj_gpu_trace_any(g.h, C.c_void_p(rays.data_ptr()),
                                                      C.c_void_p(occ.data_ptr()), n_rays, C.c_void_p(stream))))
    hit_frac = float((hits[:, 1].view(torch.int32) >= 0).float().mean())
    out = {"workload": "1M-triangle soup, 16M rays; 16M BSDF calls per material and op",
           "bvh_build_ms": round(build_ms, 2), "closest_mrays_s": round(n_rays / ms_c / 1e3, 1),
           "any_mrays_s": round(n_rays / ms_a / 1e3, 1), "hit_fraction": round(hit_frac, 3)}
    del rays, hits, occ

    def hemi(n):
        v = torch.randn((n, 3), generator=gen, device="cuda")
        v = v / v.norm(dim=1, keepdim=True)
        v[:, 2] = v[:, 2].abs()
        return v.contiguous()

    wi, wo = hemi(n_bsdf), hemi(n_bsdf)
    rnd = torch.rand((n_bsdf, 3), generator=gen, device="cuda")
    u = lambda lo, hi: torch.rand(n_bsdf, generator=gen, device="cuda") * (hi - lo) + lo
    plastic = torch.stack([u(0, 1), u(0, 1), u(0, 1), u(0, 1), u(0, 1), u(0, 1), u(0.01, 1),
                           torch.full((n_bsdf,), 1.5, device="cuda")], dim=1).contiguous()
    one, zero = torch.ones(n_bsdf, device="cuda"), torch.zeros(n_bsdf, device="cuda")
    disney = torch.stack([u(0, 1), u(0, 1), u(0, 1), zero, u(0, 1), zero, u(0, 1), u(0.01, 1), zero, zero, zero,
                          zero, zero, one, torch.full((n_bsdf,), 1.5, device="cuda")], dim=1).contiguous()
    for name, mtype, params in (("roughplastic", abi.LJ_MAT_ROUGHPLASTIC, plastic),
                                ("disney", abi.LJ_MAT_DISNEY_BSDF, disney)):
        for opname, op in (("eval", abi.LJ_BSDF_OP_EVAL), ("pdf", abi.LJ_BSDF_OP_PDF),
                           ("sample", abi.LJ_BSDF_OP_SAMPLE)):
            ms = timed(lambda: ctx.bsdf(mtype, op, params, wi, dir_out=wo, rnd=rnd, stream=stream))
            out["%s_%s_mcalls_s" % (name, opname)] = round(n_bsdf / ms / 1e3, 1)
    g.close()
    return out


def scene_update_times(ctx, pool):
    """A resident scene whose geometry moved, brought up to date in place
    (lj_gpu_scene_update_mesh: the largest mesh of the pool's largest scene
    displaced, BVH refitted or rebuilt) against creating it again from host
    memory (lj_gpu_scene_create); host clock, device synchronized."""
    import torch
    from lajolla_public_gb300 import gpu
    sc = max(pool, key=lambda x: x.num_triangles)
    mesh = max((i for i, s in enumerate(sc.shapes) if s["kind"] == abi.LJ_SHAPE_MESH),
               key=lambda i: len(sc.shapes[i]["indices"]))
    p = sc.shapes[mesh]["positions"]
    moved = (p + np.random.default_rng(5).normal(0, 1e-3, p.shape)).astype(np.float32)
    out = {"scene_triangles": sc.num_triangles, "mesh_triangles": int(len(sc.shapes[mesh]["indices"]))}
    for name in ("create", "refit", "rebuild"):
        best = None
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if name == "create":
                g = gpu.GpuScene(ctx, sc)
                torch.cuda.synchronize()
                dt = time.perf_counter() - t0
            else:
                g = gpu.GpuScene(ctx, sc)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                g.update_mesh(mesh, moved, rebuild=(name == "rebuild"))
                dt = time.perf_counter() - t0
            g.close()
            best = dt if best is None else min(best, dt)
        out[name + "_ms"] = round(best * 1e3, 2)
    return out


def scene_host_bytes(sc):
    import ctypes as C
    b = 0
    for s in sc.shapes:
        if s["kind"] == abi.LJ_SHAPE_MESH:
            b += s["positions"].nbytes + s["indices"].nbytes
            b += 0 if s["normals"] is None else s["normals"].nbytes
            b += 0 if s["uvs"] is None else s["uvs"].nbytes
    b += C.sizeof(abi.lj_shape_desc) * len(sc.shapes) + C.sizeof(abi.lj_material_desc) * len(sc.materials)
    b += C.sizeof(abi.lj_light_desc) * len(sc.lights) + C.sizeof(abi.lj_scene_desc)
    for im in sc.images:
        b += np.asarray(im, np.float32).nbytes
    for m in sc.media:
        b += C.sizeof(abi.lj_medium_desc)
        for key in ("albedo", "density"):
            v = m.get(key)
            if v is not None and v.get("data") is not None:
                b += np.asarray(v["data"], np.float32).nbytes
    return int(b)


def load_issue(kernel_name):
    """Instruction-issue ceiling of the dominant kernel from its committed
    ncu capture (profiles/traffic.json): issue-active fraction x active
    threads per warp instruction / 32 is the fraction of the SMs' lane
    slots doing work; None if not captured."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        v = json.load(open(p)).get(kernel_name)
        if isinstance(v, dict) and v.get("issue_active") and v.get("threads_per_inst"):
            return {"issue_active": v["issue_active"], "threads_per_inst": v["threads_per_inst"],
                    "lane_utilisation": round(v["issue_active"] * v["threads_per_inst"] / 32, 3),
                    "source": v.get("issue_source", "ncu")}
    return None


def load_traffic(kernel_name, units_per_launch):
    """DRAM bytes per launch of the dominant kernel from its committed ncu
    capture (profiles/traffic.json): the mean over every launch of the
    kernel in one step of this workload where that was captured, else the
    per-unit figure of a smaller case times the units of an average launch
    here; with the figure's source, or (None, None)."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        v = json.load(open(p)).get(kernel_name)
        if isinstance(v, dict) and v.get("dram_bytes_per_launch"):
            return round(float(v["dram_bytes_per_launch"])), v.get("source")
        if isinstance(v, dict) and v.get("dram_bytes_per_unit"):
            return round(float(v["dram_bytes_per_unit"]) * units_per_launch), v.get("source")
    return None, None


# ------------------------------------------------------------ CPU side
class CpuSampler:
    """The oracle's restatement of the reference path tracer (and of the
    volpath v6 algorithm for the volume scenes) on all host cores, over
    exactly the GPU arm's work: a run draws n keys (job, pixel, sample index)
    uniformly over the camera samples of a step's jobs (so jobs are weighted
    by W * H * spp), and renders each at its job's resolution, max depth and
    Russian-roulette depth with the GPU's keyed random numbers
    (job seed, pixel, sample).  calibrate() grows n until one run takes at
    least 60 % of the target time (at most 32 Mi keys)."""

    CAP = 1 << 25

    def __init__(self, pool):
        from oracle import ljo
        ljo.build()
        self.pool = pool
        self.cores = os.cpu_count() or 1
        self.rng = np.random.default_rng(7)
        self.oss = [ljo.OracleScene(s) for s in pool]   # BVH builds on the CPU, once
        self.n = 256
        self.split = {}

    def draw(self, jobs, n):
        """n keys uniform over the jobs' camera samples, grouped by job:
        [(job index, pixels, sample indices)]."""
        w = np.array([j["width"] * j["height"] * j["spp"] for j in jobs], np.float64)
        ji = self.rng.choice(len(jobs), size=n, p=w / w.sum())
        out = []
        for k in np.unique(ji):
            cnt = int((ji == k).sum())
            j = jobs[k]
            out.append((int(k), self.rng.integers(0, j["width"] * j["height"], cnt).astype(np.int32),
                        self.rng.integers(0, j["spp"], cnt).astype(np.int32)))
        return out

    def render(self, jobs, keys):
        """Renders the keys; returns ({job index: (n, 3) radiance}, seconds,
        {class: [samples, seconds]})."""
        vals, split = {}, {"path": [0, 0.0], "volpath": [0, 0.0]}
        t_all = time.perf_counter()
        for k, px, sm in keys:
            j = jobs[k]
            cls = "volpath" if self.pool[j["scene"]].integrator == abi.LJ_INTEGRATOR_VOLPATH else "path"
            t0 = time.perf_counter()
            vals[k] = self.oss[j["scene"]].render_job_samples(j["seed"], j["width"], j["height"], j["max_depth"],
                                                             j["rr_depth"], px, sm, nthreads=self.cores)
            split[cls][0] += len(px)
            split[cls][1] += time.perf_counter() - t0
        return vals, time.perf_counter() - t_all, split

    def run(self, jobs, n=None):
        keys = self.draw(jobs, self.n if n is None else n)
        _, dt, split = self.render(jobs, keys)
        self.split = split
        return dt

    def calibrate(self, jobs, target_s):
        n = 256
        dt = self.run(jobs, n)
        while dt < 0.6 * target_s and n < self.CAP:
            n = int(min(self.CAP, max(2 * n, n * 0.8 * target_s / max(dt, 1e-3))))
            dt = self.run(jobs, n)
        self.n = n
        return dt

    def describe(self, dt):
        sp = ", ".join("%s %d samples in %.2f s" % (c, v[0], v[1]) for c, v in self.split.items() if v[0])
        return ("%d (job, pixel, sample) keys drawn uniformly over the step's %d jobs' W*H*spp camera samples "
                "(the GPU arm's sample distribution), each at its job's resolution, max depth and RR depth with "
                "the GPU's keyed random numbers (%.1f s: %s); C++ restatement of src/path_tracing.h pinned to "
                "the reference's renders (and of the volpath v6 handout algorithm for the volume scenes), "
                "%d threads" % (self.n, WORKLOAD["n_jobs"], dt, sp, self.cores))

    def rate(self, dt):
        return self.n / dt / 1e6


def cpu_baseline(pool, jobs, target_s=10.0):
    cs = CpuSampler(pool)
    cs.calibrate(jobs, target_s)
    dt = cs.run(jobs)
    split = {c: {"samples": v[0], "seconds": round(v[1], 3),
                 "msamples_per_s": round(v[0] / v[1] / 1e6, 4) if v[1] > 0 else None} for c, v in cs.split.items()}
    return {"value": round(cs.rate(dt), 4), "unit": "Msamples/s", "cores": cs.cores, "kind": "port",
            "sample": cs.describe(dt), "split": split}, cs


def per_sample_parity(cs, gscenes, jobs, out, stream, per_job=256, rtol=1e-2, floor=1e-1):
    """The CPU sampler's values against the GPU's for the same keys, on one
    job of each scene: the GPU renders the job's whole image at one sample
    index (spp 1), the oracle the same sample of `per_job` random pixels.
    A sample agrees when it is within rtol relative (floor absolute); FP32
    against FP64 may flip a path's branch (roulette, a CDF boundary, a
    null collision), so a few do not."""
    from lajolla_public_gb300 import gpu
    seen, n_all, n_ok, rows = set(), 0, 0, []
    for k, j in enumerate(jobs):
        if j["scene"] in seen:
            continue
        seen.add(j["scene"])
        smp = int(cs.rng.integers(0, j["spp"]))
        n = j["width"] * j["height"] * 3
        gscenes[j["scene"]].render_job_device(out[:n], gpu.job_desc(seed=j["seed"], spp=1, sample_offset=smp,
                                                                      width=j["width"], height=j["height"],
                                                                      max_depth=j["max_depth"],
                                                                      rr_depth=j["rr_depth"]), stream=stream)
        img = out[:n].cpu().numpy().reshape(-1, 3).astype(np.float64)
        px = cs.rng.integers(0, j["width"] * j["height"], per_job).astype(np.int32)
        vals, _, _ = cs.render(jobs, [(k, px, np.full(per_job, smp, np.int32))])
        ref = vals[k]
        fin = np.isfinite(ref).all(axis=1)
        ref = np.where(fin[:, None], ref, 0.0)    # the GPU drops non-finite samples
        ok = (np.abs(img[px] - ref) <= rtol * np.maximum(np.abs(ref), floor)).all(axis=1)
        n_all += per_job
        n_ok += int(ok.sum())
        rows.append({"scene": int(j["scene"]), "job": "%dx%d depth %d sample %d" % (j["width"], j["height"],
                                                                                  j["max_depth"], smp),
                     "agree": round(float(ok.mean()), 4)})
    return {"samples": n_all, "agree_fraction": round(n_ok / max(1, n_all), 4),
            "tolerance": "%g relative, %g absolute floor" % (rtol, floor), "jobs": rows}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    pool = make_scenes()
    cs = CpuSampler(pool)
    cs.calibrate(make_jobs(1000), args.cpu_seconds / 2)   # each step a bounded sample of about half --cpu-seconds
    for i in range(args.warmup):
        cs.run(make_jobs(100 + i), max(256, cs.n // 16))
    vals, texts, secs = [], [], []
    split = {"path": [0, 0.0], "volpath": [0, 0.0]}
    for i in range(args.steps):
        dt = cs.run(make_jobs(1000 + i))   # the jobs of our arm's timed step i
        secs.append(dt)
        vals.append(cs.rate(dt))
        texts.append(cs.describe(dt))
        for c in split:
            split[c][0] += cs.split[c][0]
            split[c][1] += cs.split[c][1]
    value = statistics.mean(vals)
    cores = cs.cores
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Msamples/s",
            "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * sum(secs) / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded scene generator)",
            "config": config_dict(pool),
            "cpu_baseline": {"value": round(value, 4), "unit": "Msamples/s", "cores": cores, "kind": "port",
                             "sample": "per step: " + texts[-1],
                             "split": {c: {"samples": v[0], "seconds": round(v[1], 3)} for c, v in split.items()}},
            "e2e": {"value": round(value, 4), "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "same sample distribution as the GPU arm (step i draws from the jobs of the GPU arm's timed "
                    "step i); the reference renderer cannot be built on the benchmark machine (its sources are "
                    "not there), so its C++ restatement in oracle/ runs instead (the reference has no server: "
                    "it renders one scene per process)"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-microbench", dest="microbench", action="store_false",
                    help="skip the intersection + BSDF microbenchmark")
    ap.add_argument("--no-configs", dest="configs", action="store_false",
                    help="skip the single-scene configurations (Cornell box, full terrain, volume)")
    ap.add_argument("--no-quality", dest="quality", action="store_false",
                    help="skip the relative-MSE measurement against 64k-spp references")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
