"""Benchmark: lajolla's path-tracing hot path on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (a "step" = one full render of the scene):
  cbox     seeded Cornell box, 36 FP32 triangles, quad light (17,12,4),
           Lambertian U[0.1,0.8]^3, 256x256, 64 spp, max depth 6, box filter
           -- the reference's CPU-runnable path-tracing configuration.

Our arm (--impl ours): scene resident on the GPU; K timed renders through
lj_gpu_render_device on torch's current stream, each bracketed by CUDA
events, with a 512 MiB write between steps to flush L2 (the wavefront state,
~0.8 GB, is larger than L2 as well).  value = Msamples/s (all ranks).
e2e: the same metric through the C ABI with host buffers -- each step uploads
the scene description from host memory (lj_gpu_scene_create, BVH build
included) and renders into a host buffer (lj_gpu_render, device->host copy
of the image included).
roofline: the dominant kernel class of a profiled render (LJ_RENDER_PROFILE),
algorithmic bytes per launch (include/lj_bytes_model.h) / its average launch
time, against the measured HBM copy bandwidth (MEASURED_PEAKS.json).
cpu_baseline: the oracle's C++ restatement of the reference path
(oracle/lj_oracle.cpp, same algorithm, FP64, all host threads) on a bounded
sample of the same scene.

Reference arm (--impl reference): the reference's CPU path on the host
cores -- the reference renderer cannot be built on this machine (its sources
are not present here), so its C++ restatement in oracle/ runs instead,
pinned sample-for-sample to the reference's own renders (tests/golden).

Multi-GPU: replicas only (each rank renders its own copy of the job; no
collective on the data path); value sums all ranks' samples over the slowest
rank's time.
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

WORKLOAD = dict(name="cbox", seed=0, width=256, height=256, spp=64, max_depth=6)
METRIC = "Msamples/s (path-traced camera samples per second)"


def make_scene():
    w = WORKLOAD
    return scenes.cornell_box(seed=w["seed"], width=w["width"], height=w["height"], spp=w["spp"],
                              max_depth=w["max_depth"])


def config_dict(sc):
    w = WORKLOAD
    return {"workload": "cbox: seeded Cornell box %dx%d, %d spp, max depth %d, %d triangles, 1 quad light"
                        % (w["width"], w["height"], w["spp"], w["max_depth"], sc.num_triangles),
            "width": w["width"], "height": w["height"], "spp": w["spp"], "max_depth": w["max_depth"],
            "triangles": sc.num_triangles, "integrator": "path (NEE + MIS, RR from depth 5)",
            "l2": "wavefront state (~0.8 GB) larger than L2; 512 MiB L2 flush between timed steps",
            "parallelism": "replicas"}


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
BYTES_NODE = 80         # compressed 8-wide node
BYTES_PRIM = 48         # leaf triangle record (v0, e1, e2)
BYTES_PATH_STATE = 64   # pixel 4 + rng 8 + beta 16 + L 16 + prev 16 + nv 4
BYTES_SHADE_GEOM = 52   # 3 vertex indices + 3 positions + prim->shape
BYTES_SHADE_MAT = 160   # material record: type, eta, textured flags, 12 x RGB slot values
BYTES_SHADOW_ENTRY = 52  # shadow ray 32 + path 4 + contribution 16


def kernel_bytes(cls, st, bvh_per_closest, bvh_per_shadow):
    """Algorithmic bytes moved by all launches of one kernel class."""
    if cls == abi.LJ_KERNEL_TRACE:
        return st.rays_closest * (BYTES_RAY + BYTES_HIT + bvh_per_closest)
    if cls == abi.LJ_KERNEL_SHADOW:
        # shadow entry read + radiance read-modify-write + traversal
        return st.rays_shadow * (BYTES_SHADOW_ENTRY + 32 + bvh_per_shadow)
    if cls == abi.LJ_KERNEL_SHADE:
        seg = st.path_segments
        reads = BYTES_RAY + BYTES_HIT + 4 + BYTES_PATH_STATE + BYTES_SHADE_GEOM + BYTES_SHADE_MAT
        writes = BYTES_PATH_STATE + BYTES_RAY + 4
        return seg * (reads + writes) + st.rays_shadow * BYTES_SHADOW_ENTRY
    if cls == abi.LJ_KERNEL_CAMERA:
        return st.samples * (BYTES_RAY + 4 + BYTES_PATH_STATE)
    return 0


# ------------------------------------------------------------ CPU baseline
def cpu_baseline(sc, target_s=10.0):
    """The oracle restatement on all host cores, bounded to ~target_s seconds."""
    from oracle import ljo
    ljo.build()
    o = ljo.OracleScene(sc)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    o.render(mode="keyed", seed=1, spp=1, nthreads=cores)
    t1 = time.perf_counter() - t0
    spp = int(max(1, min(sc.spp, target_s / max(t1, 1e-3))))
    t0 = time.perf_counter()
    o.render(mode="keyed", seed=2, spp=spp, nthreads=cores)
    dt = time.perf_counter() - t0
    samples = sc.width * sc.height * spp
    return {"value": samples / dt / 1e6, "unit": "Msamples/s", "cores": cores, "kind": "port",
            "sample": "%dx%d at %d spp (%d samples, %.1f s) of the same scene; C++ restatement of "
                      "src/path_tracing.h pinned to the reference's renders" % (sc.width, sc.height, spp,
                                                                               samples, dt)}


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
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args):
    import torch
    from lajolla_public_gb300 import gpu

    rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    ctx = gpu.Context(local)
    sc = make_scene()
    g = gpu.GpuScene(ctx, sc)
    n_px = sc.width * sc.height
    out = torch.empty(n_px * 3, dtype=torch.float32, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream

    for i in range(args.warmup):
        g.render_device(out, seed=100 + i, stream=stream, stats=False)
    torch.cuda.synchronize()

    # profiled render (not timed): per-kernel-class times + counts
    st_prof = g.render_device(out, seed=7, stream=stream, stats=True, profile=True)
    rays = scenes.random_rays(9, 65536)
    # BVH bytes per ray from the instrumented traversal on camera-like rays
    cam_rays = torch.from_numpy(_camera_rays(sc, 65536)).cuda()
    nn_c, np_c = g.trace_counters(cam_rays, any_hit=False)
    nn_s, np_s = g.trace_counters(cam_rays, any_hit=True)
    bvh_closest = (nn_c * BYTES_NODE + np_c * BYTES_PRIM) / len(cam_rays)
    bvh_shadow = (nn_s * BYTES_NODE + np_s * BYTES_PRIM) / len(cam_rays)
    del rays

    # timed region
    clocks = ClockSampler(local)
    clocks.start()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    launches = 0
    st = None
    for i in range(args.steps):
        flush.fill_(i & 0xff)
        starts[i].record()
        st = g.render_device(out, seed=1000 + i, stream=stream, stats=False)
        ends[i].record()
    torch.cuda.synchronize()
    barrier(world)
    ck = clocks.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = max_over_ranks(sum(step_ms), world)
    launches = st_prof.kernel_launches * args.steps
    samples_per_step = n_px * sc.spp
    value = samples_per_step * args.steps * world / (total_ms / 1e3) / 1e6

    # e2e through the C ABI with host buffers
    e2e_ms = []
    desc_bytes = scene_host_bytes(sc)
    img_bytes = n_px * 3 * 4
    for i in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g2 = gpu.GpuScene(ctx, sc)
        g2.render(seed=2000 + i)
        g2.close()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_value = samples_per_step * world / (max_over_ranks(statistics.mean(e2e_ms), world) / 1e3) / 1e6

    # roofline of the dominant kernel class
    peak, peak_kind = measured_peaks()
    cls_ms = list(st_prof.class_ms)
    dom = int(np.argmax(cls_ms[:abi.LJ_KERNEL_OTHER]))
    # compulsory bytes (queues, hits, path state): what must cross HBM; the
    # BVH bytes of a small scene are served by L1/L2 and reported separately
    nb = kernel_bytes(dom, st_prof, 0.0, 0.0)
    nb_bvh = kernel_bytes(dom, st_prof, bvh_closest, bvh_shadow)
    launches_dom = max(1, st_prof.class_launches[dom])
    avg_launch_s = cls_ms[dom] / 1e3 / launches_dom
    achieved = nb / launches_dom / avg_launch_s / 1e9
    achieved_bvh = nb_bvh / launches_dom / avg_launch_s / 1e9
    traffic = load_traffic(abi.KERNEL_CLASS_NAMES[dom])

    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Msamples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene generator)", "config": config_dict(sc),
        "clocks": ck,
        "e2e": {"value": round(e2e_value, 3), "unit": "Msamples/s", "h2d_bytes_per_step": desc_bytes,
                "d2h_bytes_per_step": img_bytes,
                "what": "lj_gpu_scene_create (upload + device BVH build) + lj_gpu_render (image to host)"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": abi.KERNEL_CLASS_NAMES[dom], "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                     else "fallback 6800 GB/s", "traffic": traffic,
                     "bytes_per_launch": round(nb / launches_dom), "avg_launch_us": round(avg_launch_s * 1e6, 2),
                     "with_bvh": {"achieved": round(achieved_bvh, 1), "bytes_per_launch": round(nb_bvh / launches_dom),
                                  "note": "incl. BVH node/leaf bytes (lj_gpu_trace_counters); for a small scene "
                                          "they are L1/L2 hits, not HBM traffic"}},
        "kernel_ms_per_step": {abi.KERNEL_CLASS_NAMES[c]: round(cls_ms[c], 3) for c in range(abi.LJ_KERNEL_CLASSES)},
        "rays_per_step": {"closest": st_prof.rays_closest, "shadow": st_prof.rays_shadow,
                          "segments": st_prof.path_segments},
        "mrays_per_s": round((st_prof.rays_closest + st_prof.rays_shadow) / (st_prof.device_ms / 1e3) / 1e6, 1),
        "bvh_bytes_per_ray": {"closest": round(bvh_closest, 1), "shadow": round(bvh_shadow, 1)},
    }
    if rank == 0:
        line["cpu_baseline"] = cpu_baseline(sc, target_s=args.cpu_seconds)
        print(json.dumps(line), flush=True)
    g.close()
    ctx.close()


def _camera_rays(sc, n):
    """Primary-like rays from the camera toward random screen points (host)."""
    rng = np.random.default_rng(3)
    m = sc.cam_to_world
    aspect = sc.width / sc.height
    t = np.tan(np.radians(sc.fov / 2))
    sx, sy = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    d_cam = np.stack([-sx * t, -sy * t / aspect, np.ones(n)], axis=1)
    d = d_cam @ m[:3, :3].T
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = m[:3, 3]
    r[:, 4:7] = d
    r[:, 7] = np.inf
    return r


def scene_host_bytes(sc):
    b = 0
    for s in sc.shapes:
        if s["kind"] == abi.LJ_SHAPE_MESH:
            b += s["positions"].nbytes + s["indices"].nbytes
            b += 0 if s["normals"] is None else s["normals"].nbytes
            b += 0 if s["uvs"] is None else s["uvs"].nbytes
    import ctypes as C
    b += C.sizeof(abi.lj_shape_desc) * len(sc.shapes) + C.sizeof(abi.lj_material_desc) * len(sc.materials)
    b += C.sizeof(abi.lj_light_desc) * len(sc.lights) + C.sizeof(abi.lj_scene_desc)
    for im in sc.images:
        b += np.asarray(im, np.float32).nbytes
    return int(b)


def load_traffic(kernel_name):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/*.json), or None."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        d = json.load(open(p))
        v = d.get(kernel_name)
        if isinstance(v, dict):
            return v.get("dram_bytes_per_launch")
    return None


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import ljo
    ljo.build()
    sc = make_scene()
    o = ljo.OracleScene(sc)
    cores = os.cpu_count() or 1
    # bounded sample per step: the full image at `spp_step` samples per pixel
    t0 = time.perf_counter()
    o.render(mode="keyed", seed=1, spp=1, nthreads=cores)
    t1 = time.perf_counter() - t0
    spp_step = int(max(1, min(sc.spp, 8.0 / max(t1, 1e-3))))
    for i in range(args.warmup):
        o.render(mode="keyed", seed=10 + i, spp=1, nthreads=cores)
    times = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        o.render(mode="keyed", seed=100 + i, spp=spp_step, nthreads=cores)
        times.append(time.perf_counter() - t0)
    samples = sc.width * sc.height * spp_step
    value = samples * args.steps / sum(times) / 1e6
    sample = ("%dx%d at %d spp per step (%d samples) of the %d-spp job; lajolla's path tracer "
              "(C++ restatement, FP64, %d threads)" % (sc.width, sc.height, spp_step, samples, sc.spp, cores))
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Msamples/s",
            "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * sum(times) / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded scene generator)",
            "config": config_dict(sc),
            "cpu_baseline": {"value": round(value, 4), "unit": "Msamples/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 4), "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "the reference renderer itself cannot be compiled on this machine (its sources are not "
                    "shipped here); its C++ restatement in oracle/ runs instead"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
