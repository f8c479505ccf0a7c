"""Small, repeatable GPU cases for profiling, and a summary of ncu launch lists.

    python -m lajolla_public_gb300.profile_case run CASE [--warmup W] [--repeat R]
    python -m lajolla_public_gb300.profile_case summarize LAUNCHES.csv

`run` renders one named case W + R times (plain single-scene renderer unless
the case says otherwise) and prints the device time of the last render with
its per-kernel-class split; it is meant to run under `ncu -k ... -s ... -c ...`
with a capture of a few launches.

Cases:
  cbox          seeded Cornell box, 256x256, 64 spp, max depth 6
  terrain       seeded terrain + 16 icospheres + envmap, 1.26M triangles,
                512x512, 16 spp, max depth 8
  terrain_full  the full terrain configuration: 2048x1024 grid + 64
                subdivision-5 icospheres (5.5M triangles), 1024x512 HDR
                envmap, 1920x1080, 256 spp, max depth 8
  volume        seeded heterogeneous medium (256^3 grid, max density 20) in a
                dielectric sphere, 512x512, 256 spp, max depth 64 (volpath v6)
  volume_mid    the volume case at 256x256, 16 spp (one wavefront batch)
  volume_small  the volume case at 128x128, 64 spp, 64^3 grid
  terrain_srv, cbox_srv, volume_srv, volume_small_srv
                the case as one server job (server kernels)
  serving       one step of the serving benchmark on the server: its 6
                resident scenes and the 32 jobs of its first timed step
                (job seed 1000), submitted at once

`summarize` reads the CSV that `ncu --metrics gpu__time_duration.sum --csv
--log-file F` writes and prints launches, total time and share per kernel.
"""
import argparse
import csv
import sys
import time
from collections import OrderedDict

import numpy as np

from . import abi, scenes


def make_case(name):
    if name == "cbox":
        return scenes.cornell_box(seed=0, width=256, height=256, spp=64, max_depth=6)
    if name == "cbox_srv":
        return scenes.cornell_box(seed=0, width=256, height=256, spp=64, max_depth=6)
    if name in ("terrain_full", "terrain_full_srv"):
        return scenes.terrain_scene(seed=0)
    if name in ("terrain", "terrain_srv"):
        return scenes.resized_terrain_scene(seed=5, n_tris=1261476, width=512, height=512, spp=16, max_depth=8)
    if name in ("volume", "volume_srv"):
        return scenes.volume_scene(seed=0, width=512, height=512, spp=256, max_depth=64, grid=256)
    if name in ("volume_mid", "volume_mid_srv"):
        return scenes.volume_scene(seed=0, width=256, height=256, spp=16, max_depth=64, grid=256)
    if name in ("volume_small", "volume_small_srv"):
        return scenes.volume_scene(seed=0, width=128, height=128, spp=64, max_depth=64, grid=64)
    raise SystemExit("unknown case %r" % name)


def run_serving(args):
    from . import gpu
    pool = scenes.serving_scenes(0, 6)
    jobs = scenes.serving_jobs(seed=1000, n_jobs=32, n_scenes=6, rate=200.0)
    ctx = gpu.Context(0)
    gs = [gpu.GpuScene(ctx, s) for s in pool]
    opts = gpu.server_options(path_pool=args.pool, block_size=args.block, use_graphs=not args.profile,
                              profile=args.profile, policy=abi.LJ_SCHED_SRPT)
    with gpu.Server(ctx, opts) as srv:
        for rep in range(args.warmup + args.repeat):
            t0 = time.perf_counter()
            ids = [srv.submit(gs[j["scene"]], seed=j["seed"], spp=j["spp"], width=j["width"], height=j["height"],
                              max_depth=j["max_depth"], rr_depth=j["rr_depth"]) for j in jobs]
            for i in ids:
                srv.wait(i, timeout=600)
            dt = time.perf_counter() - t0
        st = srv.stats()
    n = sum(j["width"] * j["height"] * j["spp"] for j in jobs)
    cls = {abi.KERNEL_CLASS_NAMES[c]: round(st.class_ms[c] / (args.warmup + args.repeat), 3)
           for c in range(abi.LJ_KERNEL_CLASSES)}
    print("serving: %d samples, last step %.1f ms (host clock), %.1f Msamples/s, pool %d block %d, per-step "
          "classes %s, waves %d, launches %d, vol segments %d, NEE requests %d"
          % (n, dt * 1e3, n / dt / 1e6, args.pool, args.block, cls, st.waves, st.kernel_launches,
             st.vol_segments, st.nee_requests))
    for g in gs:
        g.close()
    ctx.close()


def run(args):
    import torch
    from . import gpu
    if args.case == "serving":
        return run_serving(args)
    sc = make_case(args.case)
    ctx = gpu.Context(0)
    g = gpu.GpuScene(ctx, sc)
    n = sc.width * sc.height * 3
    if args.case.endswith("_srv"):
        opts = gpu.server_options(path_pool=args.pool, block_size=args.block, use_graphs=not args.profile,
                                  profile=args.profile, one_shade_kernel=args.one_shade_kernel)
        with gpu.Server(ctx, opts) as srv:
            for i in range(args.warmup + args.repeat):
                t0 = time.perf_counter()
                srv.wait(srv.submit(g, seed=i), timeout=600)
                dt = time.perf_counter() - t0
            st = srv.stats()
        cls = {abi.KERNEL_CLASS_NAMES[c]: round(st.class_ms[c] / (args.warmup + args.repeat), 3)
               for c in range(abi.LJ_KERNEL_CLASSES)}
        print("%s: %d samples, last job %.2f ms (host clock), pool %d block %d, per-job classes %s, "
              "rays over all jobs: closest %d shadow %d, waves %d, vol segments %d, NEE requests %d"
              % (args.case, sc.width * sc.height * sc.spp, dt * 1e3, args.pool, args.block, cls, st.rays_closest,
                 st.rays_shadow, st.waves, st.vol_segments, st.nee_requests))
    else:
        out = torch.empty(n, dtype=torch.float32, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        st = None
        for i in range(args.warmup + args.repeat):
            st = g.render_device(out, seed=i, stream=stream, stats=True, profile=True)
        cls = {abi.KERNEL_CLASS_NAMES[c]: round(st.class_ms[c], 3) for c in range(abi.LJ_KERNEL_CLASSES)}
        print("%s: %d samples, %.2f ms, %.1f Msamples/s, closest %d shadow %d, null %d real %d, classes %s"
              % (args.case, st.samples, st.device_ms, st.samples / st.device_ms / 1e3, st.rays_closest,
                 st.rays_shadow, st.null_collisions, st.real_collisions, cls))
    g.close()
    ctx.close()


def summarize(args):
    tot = OrderedDict()
    with open(args.csv, newline="") as f:
        lines = [l for l in f if l.startswith('"')]
    for row in csv.DictReader(lines):
        if row.get("Metric Name") != "gpu__time_duration.sum":
            continue
        name = row["Kernel Name"].split("(")[0].replace("lj::<unnamed>::", "").replace("lj::", "")
        v = float(row["Metric Value"].replace(",", ""))
        unit = row.get("Metric Unit", "ns")
        us = v / 1e3 if unit == "ns" else (v * 1e3 if unit == "msecond" else v)
        n, t = tot.get(name, (0, 0.0))
        tot[name] = (n + 1, t + us)
    total = sum(t for _, t in tot.values()) or 1.0
    print("%-44s %9s %13s %7s" % ("kernel", "launches", "total_us", "share"))
    for name, (n, t) in sorted(tot.items(), key=lambda kv: -kv[1][1]):
        short = name if len(name) <= 44 else name[:41] + "..."
        print("%-44s %9d %13.1f %6.1f%%" % (short, n, t, 100.0 * t / total))
    print("%-44s %9d %13.1f" % ("TOTAL", sum(n for n, _ in tot.values()), total))


def main(argv=None):
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    r = sub.add_parser("run")
    r.add_argument("case")
    r.add_argument("--warmup", type=int, default=1)
    r.add_argument("--repeat", type=int, default=1)
    r.add_argument("--pool", type=int, default=1 << 22, help="server path pool")
    r.add_argument("--block", type=int, default=128, help="server block size")
    r.add_argument("--profile", action="store_true", help="server: time each kernel class")
    r.add_argument("--one-shade-kernel", action="store_true", help="server: all-materials shade kernel only")
    s = sub.add_parser("summarize")
    s.add_argument("csv")
    args = ap.parse_args(argv)
    if args.cmd == "run":
        run(args)
    else:
        summarize(args)


if __name__ == "__main__":
    main()
