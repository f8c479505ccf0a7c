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
            (and errors) match: rel_mse reports both against a 4096-spp
            render for a few jobs.
  latency   p50 / p99 of (completion - arrival) per job, both arms.
  e2e       one step through the C ABI from host memory: the scene pool is
            uploaded (lj_gpu_scene_create: descriptors from host, device BVH
            build) inside the timed region, then the jobs are served.
  roofline  the dominant kernel class of a profiled server step
            (LJ_SERVER_PROFILE: CUDA events around every kernel on the
            server's stream), compulsory algorithmic bytes per launch
            (include/lj_bytes_model.h) / average launch time, against the
            measured HBM copy bandwidth (MEASURED_PEAKS.json).
  cpu_baseline  the oracle's C++ restatement of the reference path tracer
            (oracle/lj_oracle.cpp, FP64, all host threads) on a bounded
            sample of the same scenes.
The working set (path pool ~1 GB, scenes up to 2M triangles, accumulators)
is larger than L2.

Reference arm (--impl reference): the reference's CPU path tracer on the
host cores -- the reference renderer cannot be built on the benchmark machine
(its sources are not present there), so its C++ restatement in oracle/ runs
instead, pinned sample-for-sample to the reference's own renders
(tests/golden), on a bounded sample of the serving scenes per step.

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
                         "tuned_by": "lj_gpu_server_autotune (cache %s)" % os.path.relpath(TUNE_CACHE, ROOT)}
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


def job_desc(j, profile=False):
    from lajolla_public_gb300 import gpu
    return gpu.job_desc(seed=j["seed"], spp=j["spp"], width=j["width"], height=j["height"],
                        max_depth=j["max_depth"], rr_depth=j["rr_depth"], profile=profile)


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


def tuned_options(ctx, gscenes):
    """Server options from the autotuner (cached per device and workload)."""
    from lajolla_public_gb300 import gpu
    tune = scenes.serving_jobs(seed=999, n_jobs=8, n_scenes=WORKLOAD["n_scenes"], resolutions=(128, 256, 512, 1024),
                               spps=(4, 16, 64))
    jd = [job_desc(j) for j in tune]
    os.makedirs(os.path.dirname(TUNE_CACHE), exist_ok=True)
    opt = gpu.server_options(policy=abi.LJ_SCHED_SRPT)
    return gpu.autotune(ctx, gscenes, jd, [j["scene"] for j in tune], cache_path=TUNE_CACHE, options=opt)


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
    keep_imgs = None
    for i in range(args.steps):
        jobs = make_jobs(1000 + i)
        samples += job_samples(jobs)
        keep = tuple(sorted(range(len(jobs)), key=lambda k: jobs[k]["width"] * jobs[k]["spp"])[:3]) if i == 0 else ()
        sec, lat, bimgs = serve_step(srv, gscenes, jobs, keep)
        b_secs.append(sec)
        b_lat += lat
        sec, lat, pimgs = plain_step(gscenes, jobs, out, stream, keep)
        p_secs.append(sec)
        p_lat += lat
        if i == 0:
            keep_imgs = (jobs, keep, bimgs, pimgs)
    barrier(world)
    ck = clocks.stop()
    st1 = srv.stats()
    b_total = max_over_ranks(sum(b_secs), world)
    p_total = max_over_ranks(sum(p_secs), world)
    value = samples * world / b_total / 1e6
    plain_value = samples * world / p_total / 1e6
    launches = st1.kernel_launches - st0.kernel_launches

    # matched error: a few jobs of the first step against 4096-spp renders
    jobs0, keep, bimgs, pimgs = keep_imgs
    rel_mse = []
    for k in keep:
        j = dict(jobs0[k])
        ref_job = dict(j, spp=4096, seed=j["seed"] ^ 0x5bd1e995)
        n = j["width"] * j["height"] * 3
        gscenes[j["scene"]].render_job_device(out[:n], job_desc(ref_job), stream=stream)
        ref = out[:n].cpu().numpy().reshape(j["height"], j["width"], 3).astype(np.float64)
        den = float(np.mean(ref ** 2)) + 1e-30
        rel_mse.append({"job": "%dx%d %d spp depth %d" % (j["width"], j["height"], j["spp"], j["max_depth"]),
                        "batched": float(np.mean((bimgs[k] - ref) ** 2) / den),
                        "plain": float(np.mean((pimgs[k] - ref) ** 2) / den),
                        "batched_vs_plain_max_abs": float(np.abs(bimgs[k] - pimgs[k]).max())})

    # e2e: upload the scene pool from host memory inside the timed region,
    # then serve the first timed step's jobs
    srv_e2e = gpu.Server(ctx, opts)
    jobs = make_jobs(1000)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g2 = [gpu.GpuScene(ctx, s) for s in pool]
    torch.cuda.synchronize()
    upload_s = time.perf_counter() - t0
    sec, _, _ = serve_step(srv_e2e, g2, jobs)
    e2e_s = time.perf_counter() - t0
    srv_e2e.stop()
    for g in g2:
        g.close()
    e2e_value = job_samples(jobs) * world / max_over_ranks(e2e_s, world) / 1e6
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
    traffic = load_traffic(kname, units / launches_dom)
    if dom in (abi.LJ_KERNEL_MEDIUM, abi.LJ_KERNEL_NEE):
        note = ("volumetric steps are latency bound, not HBM bound: their dependent density-grid lookups "
                "(8 x 16 B per tracking step) mostly hit L1/L2 (ncu of the volume scene's a / b / c steps)")
    else:
        note = ("traversal is instruction-issue bound, not HBM bound: ncu on a terrain job shows "
                "79% issue active, 3.1 IPC, 2% of DRAM peak")

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
        "rel_mse_vs_4096spp": rel_mse,
        "clocks": ck,
        "e2e": {"value": round(e2e_value, 3), "unit": "Msamples/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "scene_upload_s": round(upload_s, 4),
                "what": "scene pool uploaded from host (lj_gpu_scene_create, BVH build) + one step served, "
                        "images to host"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                     else "fallback 6800 GB/s", "traffic": traffic,
                     "bytes_per_launch": round(nb / launches_dom), "avg_launch_us": round(avg_launch_s * 1e6, 2),
                     "bytes": "compulsory (queues, hits, path state, shading records); BVH and density-grid "
                              "bytes excluded",
                     "note": note},
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
    srv.stop()
    if args.microbench:
        line["microbench"] = microbench(ctx)
    if rank == 0:
        line["cpu_baseline"] = cpu_baseline(pool, target_s=args.cpu_seconds)
        print(json.dumps(line), flush=True)
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


def load_traffic(kernel_name, units_per_launch):
    """DRAM bytes per launch of the dominant kernel: the per-unit figure of
    the committed ncu capture (profiles/traffic.json, measured on a smaller
    case of the same kernel) times the units of an average launch here, or
    None."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        d = json.load(open(p))
        v = d.get(kernel_name)
        if isinstance(v, dict) and v.get("dram_bytes_per_unit"):
            return round(float(v["dram_bytes_per_unit"]) * units_per_launch)
    return None


# ------------------------------------------------------------ CPU side
class CpuSampler:
    """The oracle restatement on all host cores over random pixels of every
    scene of the pool (1 spp each, the scenes' own resolution and depth).
    calibrate() grows the pixel count until one run takes at least 60 % of
    target_s (at most 4 Mi pixels per scene); run() renders that many."""

    CAP = 1 << 22

    def __init__(self, pool):
        from oracle import ljo
        ljo.build()
        self.pool = pool
        self.cores = os.cpu_count() or 1
        self.rng = np.random.default_rng(7)
        self.oss = [ljo.OracleScene(s) for s in pool]   # BVH builds on the CPU, once
        self.n_px = 256
        self.seed = 0

    def run(self, n_px=None):
        n_px = self.n_px if n_px is None else n_px
        self.seed += 1
        t0 = time.perf_counter()
        for s, o in zip(self.pool, self.oss):
            px = self.rng.integers(0, s.width * s.height, n_px).astype(np.int32)
            o.render_samples(px, 1, seed=self.seed, nthreads=self.cores)
        return time.perf_counter() - t0

    def calibrate(self, target_s):
        n_px = 256
        dt = self.run(n_px)
        while dt < 0.6 * target_s and n_px < self.CAP:
            n_px = int(min(self.CAP, max(2 * n_px, n_px * 0.8 * target_s / max(dt, 1e-3))))
            dt = self.run(n_px)
        self.n_px = n_px
        return dt

    def describe(self, dt):
        n = self.n_px * len(self.pool)
        return ("%d random pixels x 1 spp of each of the %d serving scenes (%d samples, %.1f s); C++ "
                "restatement of src/path_tracing.h pinned to the reference's renders (and of the volpath v6 "
                "handout algorithm for the volume scenes), %d threads"
                % (self.n_px, len(self.pool), n, dt, self.cores))

    def rate(self, dt):
        return self.n_px * len(self.pool) / dt / 1e6


def cpu_baseline(pool, target_s=10.0):
    cs = CpuSampler(pool)
    cs.calibrate(target_s)
    dt = cs.run()
    return {"value": round(cs.rate(dt), 4), "unit": "Msamples/s", "cores": cs.cores, "kind": "port",
            "sample": cs.describe(dt)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    pool = make_scenes()
    cs = CpuSampler(pool)
    cs.calibrate(args.cpu_seconds / 2)   # each step a bounded sample of about half --cpu-seconds
    for i in range(args.warmup):
        cs.run(max(256, cs.n_px // 16))
    vals, texts, secs = [], [], []
    for i in range(args.steps):
        dt = cs.run()
        secs.append(dt)
        vals.append(cs.rate(dt))
        texts.append(cs.describe(dt))
    value = statistics.mean(vals)
    cores = cs.cores
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Msamples/s",
            "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * sum(secs) / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded scene generator)",
            "config": config_dict(pool),
            "cpu_baseline": {"value": round(value, 4), "unit": "Msamples/s", "cores": cores, "kind": "port",
                             "sample": "per step: " + texts[-1]},
            "e2e": {"value": round(value, 4), "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "the reference renderer cannot be built on the benchmark machine (its sources are not "
                    "there); its C++ restatement in oracle/ runs instead, on a bounded sample of the "
                    "serving scenes (the reference has no server: it renders one scene per process)"}
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
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
